// 2D Jacobi time loop for sm_103a: persistent cooperative kernel in which
// every warp streams its own column strip.
//
// Work decomposition:
//   The internal field is row-major with pitch = ns * SW columns, SW = 32*V
//   (V elements = 16 bytes per lane). Warp w of the grid owns strip s and row
//   band b: columns [s*SW, s*SW+SW), rows [r0, r1). Adjacent strips of one
//   band sit in the same CTA.
//   Each step the warp sweeps its band row by row. Rows are fetched with
//   cp.async.cg (16 bytes per lane, plus one 16-byte chunk per edge lane for
//   the H columns left and right of the strip) into a private ring of DR
//   shared-memory slots, D rows ahead of use. The TMA variant (Cf::TMA)
//   fetches the same rows with tensor copies instead: one lane of the warp
//   issues two cp.async.bulk.tensor.2d boxes per row (each half of the strip
//   with EL margin columns) that complete on the slot's mbarrier, and every
//   lane waits on that barrier before reading the slot. The vertical window of 2H+1 rows
//   lives in registers and horizontal neighbours move between lanes by warp
//   shuffles. Nothing synchronises the block inside a step: warps exchange
//   halos only through the field in global memory, and steps are separated by
//   one bounded grid barrier.
//   PERKS caching: rows [r0+H, r0+H+C) of every band stay in shared memory for
//   the whole launch. Each lane owns its V columns of those rows, reads them
//   into its register window before overwriting them, and so updates them in
//   place; the strip's first and last H columns of those rows are also stored
//   to the field, where the neighbouring strips read them as halo.
//   With `alternate`, odd steps sweep bottom-up so that the rows written last
//   are read first (from L2); interior lines of interior rows are loaded with
//   an evict-first policy and dropped from L2 without write-back once read
//   (they are dead until the next step overwrites them).
//
// Boundary: clamp-to-edge as the reference (row and edge-column indices are
// clamped; elements of the last strip beyond width_x take the value of column
// width_x-1), or Dirichlet (outer H cells keep their input value).
#pragma once
#include <cuda.h>
#include <cstdint>
#include <type_traits>
#include "ptx.cuh"
#include "shapes.cuh"
#include "tune2d.cuh"

namespace perks {

struct Stencil2DParams {
  CUtensorMap map[2];   // TMA variant: box {HALF, 1} over field 0 / 1 (a half row with its margin)
  CUtensorMap emap[2];  // TMA variant: box {EL, 1}: the margin columns alone (resident rows)
  void* f[2];        // internal fields, pitch elements per row
  int wy, wx, pitch; // domain and padded row pitch (elements)
  int ns, nb;        // strips and bands
  int steps, t0;     // steps in this launch, global index of its first step
  int C;             // resident rows per warp (0 = none)
  int dirichlet, alternate, persistent;
  unsigned* bar;     // grid barrier words [2]
  unsigned* status;  // error word
  WaitCtl ctl;       // wait budget (and the test hook of the grid barrier)
  float one = 1.0f;  // 1.0 the compiler cannot see (packed FP32 sums, see f32x2.cuh)
};

// Shape geometry and the built-in choice of warps per CTA. NVO overrides the
// 16-byte vectors per lane (0 = built-in).
template <class T, int SHAPE, int NVO = 0>
struct Geom2D {
  static constexpr int H = ShapeInfo<SHAPE>::H;
  static constexpr bool BOX = ShapeInfo<SHAPE>::box;
  static constexpr int V16 = 16 / sizeof(T);             // elements per 16-byte vector
  // vectors per lane per row (built-in: one for the widest FP64 windows, to
  // fit registers; the measured table may choose one for wide FP32 windows)
  static constexpr int NV = NVO ? NVO : (sizeof(T) == 8 && H >= 5) ? 1 : 2;
  static constexpr int V = NV * V16;                     // elements per lane (8 FP32 / 4 FP64)
  static constexpr int SW = 32 * V;                      // strip width
  static constexpr int WN = 2 * H + 1;                   // window rows
  // registers the window needs (32-bit words), to pick the warps per CTA
  // (box shapes also hold the double-precision partial sums of the reference order)
  static constexpr int REG_EST =
      int(sizeof(T) / 4) * (BOX ? WN * (V + 2 * H) + V : WN * (V + 1) + (V + 2 * H) + V) + (BOX ? 72 : 40);
  static constexpr int NW_REG = (REG_EST <= 64 && !BOX) ? 32 : REG_EST <= 80 ? 24 : REG_EST <= 110 ? 16 : 8;
  // FP32 star shapes of radius 2 and 3: 12 warps (168 registers per thread)
  // measured faster than 16 (128 registers) and 8 on GB300 (2ds9pt 686 vs 662
  // GCells/s, 2d13pt 487 vs 416, reference order, 8192^2)
  static constexpr int NW_DEF = (sizeof(T) == 4 && !BOX && (H == 2 || H == 3)) ? 12 : NW_REG;
  static constexpr int d_def(int nw) { return nw >= 24 ? 3 : nw == 16 ? 4 : 6; }
  // FP32 star shapes in the reference order run their arithmetic on packed pairs
  static constexpr bool PAIR = sizeof(T) == 4 && !BOX && SHAPE <= PERKS_2DS25PT;
};

// Warps per CTA, rows in flight, division form, rows per copy wait and
// vectors per lane for one kernel: the measured table (tune2d.cuh), else the
// built-in choice. The tuning tool overrides them for a whole translation
// unit with PERKS_TUNE_*; an override of 0 (for the division form: below 0)
// keeps the table's value, so that one knob can be swept alone.
#ifndef PERKS_TUNE_NV
#define PERKS_TUNE_NV 0
#endif
#ifndef PERKS_TUNE_NW
#define PERKS_TUNE_NW 0
#endif
#ifndef PERKS_TUNE_D
#define PERKS_TUNE_D 0
#endif
#ifndef PERKS_TUNE_FIN
#define PERKS_TUNE_FIN (-1)
#endif
#ifndef PERKS_TUNE_RP
#define PERKS_TUNE_RP 0
#endif
template <class T, int SHAPE, bool FAST>
struct Pick2D {
  static constexpr Tune2D t = kTune2D[sizeof(T) == 8][FAST][SHAPE];
  static constexpr int NVC = PERKS_TUNE_NV ? PERKS_TUNE_NV : t.nv;  // 0 = built-in
  static constexpr int NW = PERKS_TUNE_NW ? PERKS_TUNE_NW : t.nw ? t.nw : Geom2D<T, SHAPE, NVC>::NW_DEF;
  static constexpr int D = PERKS_TUNE_D ? PERKS_TUNE_D : t.d ? t.d : Geom2D<T, SHAPE, NVC>::d_def(NW);
  static constexpr int FIN = FAST ? 0 : PERKS_TUNE_FIN >= 0 ? PERKS_TUNE_FIN : t.fin;
  static constexpr int RP = PERKS_TUNE_RP ? PERKS_TUNE_RP : t.rp ? t.rp : 1;
};

// Full configuration. The chosen values are template arguments, so kernels
// built with different choices never share a name.
template <class T, int SHAPE, int NW_, int D_, int FIN_, int RP_, int NV_ = 0, bool TMA_ = false>
struct Cfg2DT : Geom2D<T, SHAPE, NV_> {
  using G = Geom2D<T, SHAPE, NV_>;
  static constexpr int NW = NW_;
  static constexpr int NT = NW * 32;
  static constexpr int D = D_;                           // rows in flight per warp
  static constexpr int RP = RP_;                         // rows per copy wait (1 or 2)
  static constexpr int DR = D + RP;                      // ring slots per warp
  static constexpr int FIN = FIN_;                       // division form (divconst.cuh)
  static constexpr bool TMA = TMA_;                      // rows fetched by tensor copies
  // TMA slot: two half rows [x0-EL, x0+SW/2) and [x0+SW/2, x0+SW+EL), each
  // padded to a multiple of 128 bytes so that every copy destination is
  // 128-byte aligned; EL = H rounded up to whole 16-byte vectors, so that
  // every copy starts on a 16-byte boundary of the row.
  static constexpr int EL = ((G::H + G::V16 - 1) / G::V16) * G::V16;
  static constexpr int HALF = G::SW / 2 + EL;
  static constexpr int HALF_P = ((HALF * int(sizeof(T)) + 127) / 128) * 128 / int(sizeof(T));
  static constexpr int SLOT = TMA ? 2 * HALF_P : G::SW + 2 * G::H * G::V16;  // cp.async: strip row + one chunk per edge lane
  static constexpr size_t slots_bytes = size_t(NW) * DR * SLOT * sizeof(T);
  static constexpr size_t mbar_bytes = TMA ? (size_t(NW) * DR * 8 + 127) / 128 * 128 : 0;  // one mbarrier per slot
  static constexpr size_t ring_bytes = slots_bytes + mbar_bytes;
  static constexpr size_t res_row_bytes = size_t(NW) * G::SW * sizeof(T);  // one resident row for every warp
  static_assert(2 * G::H <= 32, "edge lanes");
  static_assert(NW >= 1 && NW <= 32 && D >= 1 && D <= 8, "launch shape");
  static_assert(RP == 1 || (RP == 2 && D >= 2), "rows per copy wait");
  static_assert(!TMA || HALF <= 256, "a tensor-copy box is at most 256 elements wide");
  static_assert(!TMA || DR <= 32, "slot phase bits");
};
template <class T, int SHAPE, bool FAST = false, bool TMA = false>
using Cfg2D = Cfg2DT<T, SHAPE, Pick2D<T, SHAPE, FAST>::NW, Pick2D<T, SHAPE, FAST>::D, Pick2D<T, SHAPE, FAST>::FIN,
                    Pick2D<T, SHAPE, FAST>::RP, Pick2D<T, SHAPE, FAST>::NVC, TMA>;

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, uint64_t pol) {
  asm volatile("cp.async.cg.shared.global.L2::cache_hint [%0], [%1], 16, %2;" ::"r"(smem_u32(smem)), "l"(gmem),
               "l"(pol)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
// One 2D tensor box global -> shared, completing on `bar` (tx-count).
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar,
                                            uint64_t policy) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cta.global.tile.mbarrier::complete_tx::bytes.L2::cache_hint"
      " [%0], [%1, {%2, %3}], [%4], %5;" ::"r"(smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar)), "l"(policy)
      : "memory");
}

// Vector loads/stores of a lane's V elements (NV 16-byte vectors), vector k
// at src + k * S elements: S = 16 bytes for a lane's contiguous columns in
// the field; S = 32 x 16 bytes for the vector-major shared-memory rows, where
// vector k of lane l sits at (32 k + l) x 16 bytes, so that each warp-wide
// vector access is one contiguous 512-byte run (no bank conflicts).
template <int NV, int S = 4>
__device__ __forceinline__ void load_lane(const float* src, float (&o)[4 * NV]) {
#pragma unroll
  for (int k = 0; k < NV; k++) {
    const float4 v = *reinterpret_cast<const float4*>(src + k * S);
    o[4 * k] = v.x; o[4 * k + 1] = v.y; o[4 * k + 2] = v.z; o[4 * k + 3] = v.w;
  }
}
template <int NV, int S = 2>
__device__ __forceinline__ void load_lane(const double* src, double (&o)[2 * NV]) {
#pragma unroll
  for (int k = 0; k < NV; k++) {
    const double2 v = *reinterpret_cast<const double2*>(src + k * S);
    o[2 * k] = v.x; o[2 * k + 1] = v.y;
  }
}
template <int NV, int S = 4>
__device__ __forceinline__ void store_lane(float* dst, const float (&o)[4 * NV]) {
#pragma unroll
  for (int k = 0; k < NV; k++)
    *reinterpret_cast<float4*>(dst + k * S) = make_float4(o[4 * k], o[4 * k + 1], o[4 * k + 2], o[4 * k + 3]);
}
template <int NV, int S = 2>
__device__ __forceinline__ void store_lane(double* dst, const double (&o)[2 * NV]) {
#pragma unroll
  for (int k = 0; k < NV; k++) *reinterpret_cast<double2*>(dst + k * S) = make_double2(o[2 * k], o[2 * k + 1]);
}

// A window row in registers: V values of this lane and one edge value.
template <class T, int V>
struct Row2D {
  T v[V];
  T e;
};
template <class T, int N>
struct Win2D {
  T h[N];
};

// Compile-time loop: f(std::integral_constant<int, i>) for i = 0..N-1, so that
// register-array indices derived from i are constants.
template <int N, class F>
__device__ __forceinline__ void static_for(F&& f) {
  if constexpr (N > 0) {
    static_for<N - 1>(f);
    f(std::integral_constant<int, N - 1>{});
  }
}

template <class T, int SHAPE, bool FAST, class Cf>
__global__ void __launch_bounds__(Cf::NT, 1) stencil2d_kernel(const __grid_constant__ Stencil2DParams p) {
  constexpr int H = Cf::H, V = Cf::V, V16 = Cf::V16, NV = Cf::NV, SW = Cf::SW, NW = Cf::NW, D = Cf::D,
                DR = Cf::DR, SLOT = Cf::SLOT;
  constexpr int WN = Cf::WN;
  constexpr bool BOX = Cf::BOX;
  constexpr int WW = V + 2 * H;  // horizontal window of one row
  using RowT = Row2D<T, V>;
  using WinT = Win2D<T, WW>;

  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  T* const ring = reinterpret_cast<T*>(smem_raw) + size_t(wid) * DR * SLOT;
  T* const res = reinterpret_cast<T*>(smem_raw + Cf::ring_bytes);  // [C][NW][SW]

  const int wy = p.wy, wx = p.wx, pitch = p.pitch;
  const int item = blockIdx.x * NW + wid;
  const bool active = item < p.ns * p.nb;
  const int strip = active ? item % p.ns : 0;
  const int band = active ? item / p.ns : 0;
  const int x0 = strip * SW;
  const int r0 = int((long long)band * wy / p.nb), r1 = int((long long)(band + 1) * wy / p.nb);
  const int TY = r1 - r0;
  const int C = active ? max(0, min(p.C, TY - 2 * H)) : 0;
  const int rres0 = r0 + H;
  const int xl = x0 + lane * V;            // this lane's first column
  const bool dir = p.dirichlet != 0;
  const bool alt = p.alternate != 0;
  const bool ghost_strip = (x0 + SW > wx) && !dir;  // strip reaches past the last column
  const int lw = wx - 1 - x0;              // strip-local last column
  // Edge lanes: lane k < H needs column x0-1-k, lane H+k needs x0+SW+k, both
  // clamped to the domain (this is the reference's clamp boundary). Each edge
  // lane fetches the aligned 16-byte chunk holding its column.
  const bool edge_lane = lane < 2 * H;
  const int edge_col = lane < H ? max(x0 - 1 - lane, 0) : min(x0 + SW + (lane - H), wx - 1);
  const int edge_chunk = (edge_col / V16) * V16;
  const int edge_sub = edge_col - edge_chunk;
  // TMA slot: margin EL, then the strip; lanes 16..31 start in the second half
  constexpr int PADE = Cf::HALF_P - Cf::HALF;
  T* const my_ring_v = Cf::TMA ? ring + Cf::EL + lane * V + (lane >= 16 ? PADE : 0)
                               : ring + lane * V;                // this lane's columns in a slot
  T* const my_ring_e = ring + SW + min(lane, 2 * H - 1) * V16;  // cp.async: this edge lane's chunk in a slot
  // TMA: slot position of this edge lane's column. A column clamped into the
  // strip (the domain's first or last column) is taken from the registers
  // instead, because resident rows copy only the margins.
  int epos = 0;
  if (Cf::TMA && edge_lane) {
    const int l = edge_col - x0 + Cf::EL;
    epos = l + (l >= Cf::HALF ? PADE : 0);
  }
  uint64_t* const mb = reinterpret_cast<uint64_t*>(smem_raw + Cf::slots_bytes) + size_t(wid) * DR;  // TMA
  // Shuffle sources and selectors of the horizontal window (row independent).
  int src_l[H], src_r[H];
  bool use_in_l[H], use_in_r[H];
#pragma unroll
  for (int d = 1; d <= H; d++) {
    src_l[d - 1] = max(d - 1 - lane * V, 0);
    src_r[d - 1] = H + max(d - 1 - (31 - lane) * V, 0);
    use_in_l[d - 1] = lane * V >= d;
    use_in_r[d - 1] = (31 - lane) * V >= d;
  }

  GridBarrier gbar{p.bar, p.status, gridDim.x, p.ctl};
  const uint64_t pol = policy_evict_normal();
  const uint64_t pol_first = policy_evict_first();
  const F2 one2(p.one);
  bool ok = true;
  // TMA: one mbarrier per slot of this warp's ring (one arrival: the issuing
  // lane's expect_tx); per slot the parity of its next phase and whether a
  // copy into it is in flight
  unsigned ph = 0, pend = 0;
  bool copy_ok = true;
  if constexpr (Cf::TMA) {
    if (lane == 0)
      for (int i = 0; i < DR; i++) mbar_init(&mb[i], 1);
    fence_mbar_init();
    __syncwarp();
  }

  auto res_ptr = [&](int r) -> T* { return res + (size_t(r - rres0) * NW + wid) * SW + lane * V; };
  auto is_res = [&](int r) { return r >= rres0 && r < rres0 + C; };

  if (C > 0) {
    const T* fin = static_cast<const T*>(p.f[p.t0 & 1]);
    for (int k = 0; k < C; k++) {
      T v[V];
      load_lane<NV>(fin + size_t(rres0 + k) * pitch + xl, v);
      store_lane<NV>(res_ptr(rres0 + k), v);
    }
  }

  for (int it = 0; it < p.steps && ok; it++) {
    const int t = p.t0 + it;
    const T* fin = static_cast<const T*>(p.f[t & 1]);
    T* fout = static_cast<T*>(p.f[(t + 1) & 1]);
    const bool fwd = !alt || ((t & 1) == 0);

    if (active) {
      const int rbase = fwd ? r0 : r1 - 1, rstep = fwd ? 1 : -1;
      auto row_of = [&](int q) { return min(max(rbase + rstep * q, 0), wy - 1); };
      auto interior = [&](int r) { return r >= r0 + H && r < r1 - H; };
      int sf = 0;  // ring slot of the next position to fetch (positions advance by one)
      int sl = 0;  // ring slot of the next position to load into registers
      // Issue the copies for sweep position q (one commit group per position).
      auto fetch = [&](int q) {
        if constexpr (Cf::TMA) {
          // two half rows with their margins; for a resident row only the
          // margins (the neighbouring strips' edge columns)
          if (q < TY + H && copy_ok) {
            const int r = row_of(q);
            T* slot = ring + size_t(sf) * SLOT;
            if (lane == 0) {
              if (!is_res(r)) {
                const uint64_t pl = (alt && interior(r)) ? pol_first : pol;
                mbar_arrive_expect_tx(&mb[sf], unsigned(2 * Cf::HALF * sizeof(T)));
                tma_load_2d(slot, &p.map[t & 1], x0 - Cf::EL, r, &mb[sf], pl);
                tma_load_2d(slot + Cf::HALF_P, &p.map[t & 1], x0 + SW / 2, r, &mb[sf], pl);
              } else {
                mbar_arrive_expect_tx(&mb[sf], unsigned(2 * Cf::EL * sizeof(T)));
                tma_load_2d(slot, &p.emap[t & 1], x0 - Cf::EL, r, &mb[sf], pol);
                tma_load_2d(slot + Cf::HALF_P + SW / 2, &p.emap[t & 1], x0 + SW, r, &mb[sf], pol);
              }
            }
            pend |= 1u << sf;
          }
        } else {
          if (q < TY + H) {
            const int r = row_of(q);
            const T* src = fin + size_t(r) * pitch;
            T* slot = ring + size_t(sf) * SLOT;
            if (!is_res(r)) {
              const uint64_t pl = (alt && interior(r)) ? pol_first : pol;
#pragma unroll
              for (int k = 0; k < NV; k++)
                cp_async16(my_ring_v + size_t(sf) * SLOT + k * V16, src + xl + k * V16, pl);
            }
            if (edge_lane) cp_async16(slot + SW + lane * V16, src + edge_chunk, pol);
          }
          cp_async_commit();
        }
        sf = (sf + 1 == DR) ? 0 : sf + 1;
      };
      // Move position q from the ring (or resident storage) into registers.
      auto load_row = [&](int q) -> RowT {
        RowT out;
        const int r = row_of(q);
        const bool rr = is_res(r);
        if constexpr (Cf::TMA) {
          if (copy_ok) {
            const bool w = __all_sync(0xffffffffu, mbar_wait(&mb[sl], (ph >> sl) & 1u, p.ctl.budget));
            if (w) {
              ph ^= 1u << sl;
              pend &= ~(1u << sl);
            } else {
              if (lane == 0) atomicOr(p.status, kErrCopyTimeout);
              copy_ok = false;
            }
          }
        }
        load_lane<NV>(rr ? res_ptr(r) : my_ring_v + size_t(sl) * SLOT, out.v);
        if constexpr (Cf::TMA) {
          out.e = edge_lane ? ring[size_t(sl) * SLOT + epos] : T(0);
          if (x0 == 0) {  // columns left of the domain clamp to column 0
            const T c0 = __shfl_sync(0xffffffffu, out.v[0], 0);
            if (lane < H) out.e = c0;
          }
          if (lw < SW) {  // columns right of the domain clamp to its last column, in this strip
            const int le = lw % V;
            T cl = out.v[0];
#pragma unroll
            for (int i = 1; i < V; i++) cl = (le == i) ? out.v[i] : cl;
            cl = __shfl_sync(0xffffffffu, cl, lw / V);
            if (edge_lane && lane >= H && x0 + SW + (lane - H) > wx - 1) out.e = cl;
          }
        } else {
          out.e = edge_lane ? my_ring_e[size_t(sl) * SLOT + edge_sub] : T(0);
        }
        if (ghost_strip) {
          // elements beyond the last column take that column's value
          const int le = lw % V;
          T edge = out.v[0];
#pragma unroll
          for (int i = 1; i < V; i++) edge = (le == i) ? out.v[i] : edge;
          edge = __shfl_sync(0xffffffffu, edge, min(lw / V, 31));
          const int lim = lw - lane * V;  // elements i > lim are beyond the domain
#pragma unroll
          for (int i = 0; i < V; i++) out.v[i] = (i > lim) ? edge : out.v[i];
        }
        if (alt && !rr && interior(r)) {
          // the middle lines of this strip row are dead once read: drop them
          // from L2 without write-back (edge lines stay: neighbours read them)
          __syncwarp();
          constexpr int LE = 128 / int(sizeof(T));  // elements per 128-byte line
          constexpr int LPL = LE / V;               // lanes per line
          const int c = lane * V;
          if ((lane % LPL) == 0 && c >= LE && c + LE <= SW - LE) l2_discard_line(fin + size_t(r) * pitch + x0 + c);
        }
        sl = (sl + 1 == DR) ? 0 : sl + 1;
        return out;
      };

      // Star shapes keep V values (+ one edge value) per window row and build
      // the horizontal window of the centre row when it is needed; box shapes
      // build each row's horizontal window once, when the row arrives.
      RowT w[BOX ? 1 : WN];       // star: window rows, slot (position + H) mod WN
      WinT wf[BOX ? WN : 1];      // box: full horizontal window of each row
      // Horizontal window of one row: own V values and H neighbours on each
      // side, from the neighbouring lanes or, at the strip edge, the edge lanes.
      auto hwin = [&](const RowT r) -> WinT {
        WinT out;
#pragma unroll
        for (int i = 0; i < V; i++) out.h[H + i] = r.v[i];
#pragma unroll
        for (int d = 1; d <= H; d++) {
          const int dl = (d + V - 1) / V;  // lanes away
          const T vin = __shfl_up_sync(0xffffffffu, r.v[dl * V - d], dl);
          const T ved = __shfl_sync(0xffffffffu, r.e, src_l[d - 1]);
          out.h[H - d] = use_in_l[d - 1] ? vin : ved;
          const T vin2 = __shfl_down_sync(0xffffffffu, r.v[(d - 1) % V], dl);
          const T ved2 = __shfl_sync(0xffffffffu, r.e, src_r[d - 1]);
          out.h[H + V - 1 + d] = use_in_r[d - 1] ? vin2 : ved2;
        }
        return out;
      };
      auto bring = [&](int q, auto kc) {
        constexpr int k = decltype(kc)::value;  // window slot
        if constexpr (BOX) wf[k] = hwin(load_row(q));
        else w[k] = load_row(q);
      };
      for (int q = -H; q < -H + D; q++) fetch(q);
      int qn = -H;  // next position to bring into the window
      static_for<2 * H>([&](auto kc) {
        if constexpr (!Cf::TMA) cp_async_wait<D - 1>();
        __syncwarp();
        bring(qn, kc);
        fetch(qn + D);
        qn++;
      });

      // Compute and store output row q; j = q mod WN picks the window slots.
      auto do_row = [&](int q, auto jc, auto fwd_c) {
        constexpr int j = decltype(jc)::value;
        constexpr bool F = decltype(fwd_c)::value;
        const int y = F ? r0 + q : r1 - 1 - q;
        // window slot of row y+dy
        auto ws = [](int dy) constexpr { return (j + H + (F ? dy : -dy) + 2 * WN) % WN; };
        WinT hc;  // star: horizontal window of the centre row
        if constexpr (!BOX) hc = hwin(w[ws(0)]);
        T o[V];
        if constexpr (Cf::PAIR && !FAST && Cf::FIN == 2) {
          // two adjacent cells per packed FP32 instruction; the division's
          // finish only for a warp row with a subnormal midpoint or a
          // non-finite value (divconst.cuh, FIN = 2)
          F2 xs[V / 2], q[V / 2];
          float e[V];
#pragma unroll
          for (int i = 0; i < V; i += 2) {
            auto u2 = [&](int, int dy, int dx) -> F2 {
              if (dy == 0) return F2::pack(hc.h[H + i + dx], hc.h[H + i + 1 + dx]);
              return F2::pack(w[ws(dy)].v[i], w[ws(dy)].v[i + 1]);
            };
            xs[i / 2] = star2d_sum<F2, SHAPE>(u2, [one2](F2 a, F2 b) { return RN<F2>::fma(b, one2, a); });
            F2 ep;
            q[i / 2] = div_const_q1<118>(xs[i / 2], ep);
            ep.unpack(e[i], e[i + 1]);
          }
          if (__any_sync(0xffffffffu, div_needs_finish<118>(e))) {
#pragma unroll
            for (int i = 0; i < V / 2; i++) q[i] = div_const<118, 1>(xs[i]);
          }
#pragma unroll
          for (int i = 0; i < V; i += 2) q[i / 2].unpack(o[i], o[i + 1]);
        } else if constexpr (Cf::PAIR && !FAST) {
          // two adjacent cells per packed FP32 instruction
#pragma unroll
          for (int i = 0; i < V; i += 2) {
            auto u2 = [&](int, int dy, int dx) -> F2 {
              if (dy == 0) return F2::pack(hc.h[H + i + dx], hc.h[H + i + 1 + dx]);
              return F2::pack(w[ws(dy)].v[i], w[ws(dy)].v[i + 1]);
            };
            star2d_ref<F2, SHAPE, Cf::FIN>(u2, [one2](F2 a, F2 b) { return RN<F2>::fma(b, one2, a); })
                .unpack(o[i], o[i + 1]);
          }
        } else {
#pragma unroll
          for (int i = 0; i < V; i++) {
            auto u = [&](int, int dy, int dx) -> T {
              if constexpr (BOX) return wf[ws(dy)].h[H + i + dx];
              else return dy == 0 ? hc.h[H + i + dx] : w[ws(dy)].v[i];
            };
            o[i] = stencil_point<T, SHAPE, FAST, Cf::FIN>(u);
          }
        }
        if (dir) {
          const bool row_fixed = y < H || y >= wy - H;
#pragma unroll
          for (int i = 0; i < V; i++) {
            const int x = xl + i;
            T old;
            if constexpr (BOX) old = wf[ws(0)].h[H + i];
            else old = w[ws(0)].v[i];
            if (row_fixed || x < H || x >= wx - H) o[i] = old;
          }
        }
        T* dst = fout + size_t(y) * pitch + xl;
        if (is_res(y)) {
          store_lane<NV>(res_ptr(y), o);
          if (lane * V < H || (lane + 1) * V > SW - H) store_lane<NV>(dst, o);
        } else {
          store_lane<NV>(dst, o);
        }
      };
      auto step_rows = [&](auto fwd_c) {
        if constexpr (Cf::RP == 1) {
          for (int q0 = 0; q0 < TY; q0 += WN) {
            static_for<WN>([&](auto jc) {
              constexpr int j = decltype(jc)::value;
              const int q = q0 + j;
              if (q < TY) {
                if constexpr (!Cf::TMA) cp_async_wait<D - 1>();
                __syncwarp();
                bring(qn, std::integral_constant<int, (j + 2 * H) % WN>{});
                fetch(qn + D);
                qn++;
                do_row(q, jc, fwd_c);
              }
            });
          }
        } else {
          // Two rows per copy wait: one wait and one warp barrier cover both,
          // and the two rows' arithmetic can overlap. The ring has D + 2
          // slots, so the two slots fetched here were freed by the previous
          // pair, before this pair's barrier.
          for (int q0 = 0; q0 < TY; q0 += 2 * WN) {
            static_for<WN>([&](auto pc) {
              constexpr int j0 = 2 * decltype(pc)::value, j1 = j0 + 1;
              const int q = q0 + j0;
              if (q < TY) {
                if constexpr (!Cf::TMA) cp_async_wait<D - 2>();
                __syncwarp();
                bring(qn, std::integral_constant<int, (j0 + 2 * H) % WN>{});
                fetch(qn + D);
                fetch(qn + D + 1);
                qn++;
                do_row(q, std::integral_constant<int, j0 % WN>{}, fwd_c);
                if (q + 1 < TY) {
                  bring(qn, std::integral_constant<int, (j1 + 2 * H) % WN>{});
                  qn++;
                  do_row(q + 1, std::integral_constant<int, j1 % WN>{}, fwd_c);
                }
              }
            });
          }
        }
      };
      if (fwd) step_rows(std::true_type{});
      else step_rows(std::false_type{});
      if constexpr (!Cf::TMA) cp_async_wait<0>();
      __syncwarp();
    }
    if constexpr (Cf::TMA) {
      // this step's stores before the next step's tensor copies read them
      fence_proxy_async_global();
      if (!__syncthreads_and(copy_ok)) ok = false;
    }
    if (ok && it + 1 < p.steps && p.persistent) {
      if (!gbar.sync()) ok = false;
    }
  }
  if constexpr (Cf::TMA) {
    // after a failed wait: leave no tensor copy in flight into this CTA's
    // shared memory (a budget of its own; copies end by themselves)
    if (pend != 0 && lane == 0) {
      for (int i = 0; i < DR; i++) {
        if (!((pend >> i) & 1u)) continue;
        const long long c0 = clock64();
        while (!mbar_try_wait(&mb[i], (ph >> i) & 1u)) {
          if (clock64() - c0 > (1ll << 30)) break;
        }
      }
    }
  }
  if (ok && C > 0) {
    T* fnew = static_cast<T*>(p.f[(p.t0 + p.steps) & 1]);
    for (int k = 0; k < C; k++) {
      T v[V];
      load_lane<NV>(res_ptr(rres0 + k), v);
      store_lane<NV>(fnew + size_t(rres0 + k) * pitch + xl, v);
    }
  }
}

// Naive comparator (the reference's kernel2d_restrict,
// stencil/2dstencil/jacobi-naive.cu:7-106): one thread per cell, every
// neighbour read from global memory at its clamped index, one launch per
// time step, nothing staged on chip. Same arithmetic as the other kernels.
template <class T, int SHAPE, bool FAST, int FIN>
__global__ void __launch_bounds__(256) stencil2d_naive(const T* __restrict__ fin, T* __restrict__ fout, int wy,
                                                       int wx, int pitch, int dirichlet) {
  constexpr int H = ShapeInfo<SHAPE>::H;
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int y = blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= wx || y >= wy) return;
  auto u = [&](int, int dy, int dx) -> T {
    const int yy = min(max(y + dy, 0), wy - 1), xx = min(max(x + dx, 0), wx - 1);
    return fin[size_t(yy) * pitch + xx];
  };
  T o = stencil_point<T, SHAPE, FAST, FIN>(u);
  if (dirichlet && (y < H || y >= wy - H || x < H || x >= wx - H)) o = fin[size_t(y) * pitch + x];
  fout[size_t(y) * pitch + x] = o;
}

}  // namespace perks
