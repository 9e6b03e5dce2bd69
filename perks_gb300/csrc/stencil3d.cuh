// 3D Jacobi time loop for sm_103a: persistent cooperative kernel with a
// warp-specialised plane pipeline.
//
// Work decomposition:
//   The internal field is [height][width_y][px] (px = width_x rounded up to
//   16 bytes). An x-y tile is SW columns (32 lanes x V elements) by TY rows.
//   The (tile, plane) pairs of the whole domain, tile-major, are split into
//   gridDim.x equal ranges; CTA b sweeps its range every step as one or two
//   z-runs ("segments") of one tile each, so every SM gets the same number of
//   cells whatever the domain's shape.
//   A CTA has NWC compute warps and one producer warp. For each input plane
//   of a segment the producer issues three tiled TMA copies into one of NR
//   shared-memory ring slots: the tile's TY + 2H rows of SW columns, and the
//   HP columns left and right of it as two separate strips (a box is at most
//   256 elements wide; the strips keep every destination 128-byte aligned).
//   Coordinates outside the field read as zero and are never used: the
//   consumers clamp every index. The copies complete the slot's "full"
//   mbarrier. (One cp.async.bulk per row costs about 100 SM cycles of copy
//   issue each, which capped the kernel at ~2.9G rows/s.)
//   Compute warp w owns RY rows of the tile: for output plane z it reads
//   planes z-H..z+H from the ring, keeps a rolling window of rows in
//   registers, moves horizontal neighbours between lanes by shuffles, writes
//   its rows of the output plane to the field, and arrives on the "empty"
//   mbarrier (count NWC) of plane z-H, after which the producer may refill that
//   slot. Nothing synchronises the whole CTA inside a step; steps are
//   separated by one bounded grid barrier.
//   With `alternate`, odd steps sweep the segments and their planes in reverse,
//   so that the planes written last are read first while still in L2.
//   PERKS caching (persistent launches): up to `kr` planes of one of the
//   CTA's segments stay in shared memory for the whole launch, each as a
//   [TY][SW] tile. Only planes no other CTA reads are chosen: at least H
//   planes away from both ends of the segment's z-run (as the 2D kernel's
//   bands keep no row within H of their ends). For such a plane the producer warp
//   copies the resident tile into the slot's TY interior rows itself (16-byte
//   shared loads and stores) before it arrives on the slot's full barrier, and
//   the tensor copies bring only the H halo rows above and below and the pad
//   strips from the field. Its output goes back into the resident tile, and to the field
//   only where neighbouring tiles read it: the first and last H rows, and the
//   HP columns at each side (vector 0 of lane 0, vector NV-1 of lane 31). The
//   full planes are written to the field once, at the end of the launch.
//
// Boundary: clamp-to-edge as the reference (plane, row and column indices
// clamped), or Dirichlet (outer H cells keep their input value). Rows and
// planes outside the domain are never copied.
#pragma once
#include <cuda.h>
#include <cstdint>
#include <type_traits>
#include "ptx.cuh"
#include "shapes.cuh"
#include "stencil2d.cuh"  // static_for
#include "tune3d.cuh"

namespace perks {

template <class T>
__device__ __forceinline__ void vec16_load(const T* src, T* dst) {
  if constexpr (sizeof(T) == 4) {
    const float4 v = *reinterpret_cast<const float4*>(src);
    dst[0] = v.x; dst[1] = v.y; dst[2] = v.z; dst[3] = v.w;
  } else {
    const double2 v = *reinterpret_cast<const double2*>(src);
    dst[0] = v.x; dst[1] = v.y;
  }
}
// 16-byte shared-memory store that the compiler does not order against other
// memory accesses (no memory clobber): for the resident plane tiles, which
// the compute loop writes but never reads, so that the ring loads of later
// rows may still be scheduled ahead of it. Readers of the tiles sit behind a
// barrier.
__device__ __forceinline__ void sts16_unordered(float* dst, const float* v) {
  asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(smem_u32(dst)), "f"(v[0]), "f"(v[1]), "f"(v[2]),
               "f"(v[3]));
}
__device__ __forceinline__ void sts16_unordered(double* dst, const double* v) {
  asm volatile("st.shared.v2.f64 [%0], {%1, %2};" ::"r"(smem_u32(dst)), "d"(v[0]), "d"(v[1]));
}

template <class T>
__device__ __forceinline__ void vec16_store(T* dst, const T* src) {
  if constexpr (sizeof(T) == 4)
    *reinterpret_cast<float4*>(dst) = make_float4(src[0], src[1], src[2], src[3]);
  else
    *reinterpret_cast<double2*>(dst) = make_double2(src[0], src[1]);
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar,
                                            uint64_t policy) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cta.global.tile.mbarrier::complete_tx::bytes.L2::cache_hint"
      " [%0], [%1, {%2, %3, %4}], [%5], %6;" ::"r"(smem_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar)), "l"(policy)
      : "memory");
}

struct Stencil3DParams {
  CUtensorMap map[2];   // box {SW, TY+2H, 1} over field 0 / 1
  CUtensorMap pmap[2];  // box {HP, TY+2H, 1}: the pad strips
  CUtensorMap hmap[2];  // box {SW, H, 1}: the halo rows of a resident plane
  void* f[2];
  int kr;             // resident planes per CTA (0: none)
  int h, wy, wx, px;  // domain and x pitch (elements)
  int gx, gy;         // x-y tile grid
  int steps, t0;
  int dirichlet, alternate, persistent;
  unsigned* bar;
  unsigned* status;
  WaitCtl ctl;  // wait budget (and the test hook of the grid barrier)
  float one = 1.0f;  // 1.0 the compiler cannot see (packed FP32 sums, see f32x2.cuh)
};

// Compute warps, rows per compute warp and the ring depth (KB of planes in
// flight) of one kernel: the measured table (tune3d.cuh), else the built-in
// choice. The tuning tool overrides them for a whole translation unit with
// PERKS_TUNE3_*.
//
// Built-in choice, from timing FP32 variants at 512^3: the 7-point star does
// best with 8 warps of 4 rows, the radius-2 and box shapes with 11 warps of 3
// rows (12 warps: 168 registers per thread). FP64 is bound by the FP64 pipe:
// 8 warps of 4 rows keep its larger windows out of local memory.
template <class T, int SHAPE, bool FAST>
struct Pick3D {
  static constexpr bool WIDE = sizeof(T) == 4 && (ShapeInfo<SHAPE>::box || ShapeInfo<SHAPE>::H >= 2);
  static constexpr Tune3D t = kTune3D[sizeof(T) == 8][FAST][SHAPE - PERKS_3D7PT];
#ifdef PERKS_TUNE3_NWC
  static constexpr int NWC = PERKS_TUNE3_NWC;
#else
  static constexpr int NWC = t.nwc ? t.nwc : WIDE ? 11 : 8;
#endif
#ifdef PERKS_TUNE3_RY
  static constexpr int RY = PERKS_TUNE3_RY;
#else
  static constexpr int RY = t.ry ? t.ry : WIDE ? 3 : 4;
#endif
#ifdef PERKS_TUNE3_DKB
  static constexpr int DKB = PERKS_TUNE3_DKB;
#else
  static constexpr int DKB = t.dkb ? t.dkb : 72;
#endif
};

// Full configuration; the chosen values are template arguments, so kernels
// built with different choices never share a name.
template <class T, int SHAPE, int NWC_, int RY_, int DKB_, bool RES_ = false>
struct Cfg3DT {
  static constexpr bool RES = RES_;  // built with resident planes (the launcher picks it when a plane fits)
  static constexpr int H = ShapeInfo<SHAPE>::H;
  static constexpr bool BOX = ShapeInfo<SHAPE>::box;
  static constexpr int V16 = 16 / sizeof(T);
  static constexpr int NV = (BOX || H >= 2) ? 1 : 2;      // 16-byte vectors per lane
  static constexpr int V = NV * V16;                      // columns per lane
  static constexpr int SW = 32 * V;                       // tile width
  static constexpr int HP = ((H + V16 - 1) / V16) * V16;  // pad columns each side (16-byte multiple)
  static constexpr int NWC = NWC_;                        // compute warps (one more is the producer)
  static constexpr int RY = RY_;                          // rows per compute warp
  static constexpr int TY = NWC * RY;                     // tile height
  static constexpr int NT = (NWC + 1) * 32;
  static constexpr int SR = TY + 2 * H;                   // slot rows
  static constexpr int AL = 128 / sizeof(T);
  // slot: [SR][SW] tile rows, then [SR][HP] left pad, then [SR][HP] right pad
  static constexpr int MAIN = ((SR * SW + AL - 1) / AL) * AL;
  static constexpr int PADSZ = ((SR * HP + AL - 1) / AL) * AL;
  static constexpr int PLANE = MAIN + 2 * PADSZ;           // slot stride (elements)
  static constexpr unsigned tx_bytes = unsigned((SR * SW + 2 * SR * HP) * sizeof(T));
  static constexpr size_t slot_bytes = size_t(PLANE) * sizeof(T);
  // planes in flight beyond the 2H+1 being read: about DKB KB (every slot
  // size of the tables' 72 KB gives at least 2), within a 200 KB ring, and at
  // least 1 (a ring larger than shared memory is refused by the launcher)
  static constexpr int DMAX = int((200u * 1024u) / slot_bytes) - (2 * H + 1);
  static constexpr int DWANT = int((unsigned(DKB_) * 1024u + slot_bytes - 1) / slot_bytes) > 1
                                   ? int((unsigned(DKB_) * 1024u + slot_bytes - 1) / slot_bytes)
                                   : 1;
  static constexpr int D = (DMAX < DWANT ? DMAX : DWANT) < 1 ? 1 : (DMAX < DWANT ? DMAX : DWANT);
  static constexpr int NR = 2 * H + 1 + D;                // ring slots
  static constexpr size_t ring_bytes = size_t(NR) * slot_bytes;
  static constexpr size_t smem_bytes = ring_bytes + 2 * NR * sizeof(uint64_t);
  static constexpr size_t res_offset = (smem_bytes + 127) / 128 * 128;  // resident plane tiles
  static constexpr size_t res_plane_bytes = size_t(TY) * SW * sizeof(T);
  // bytes the tensor copies of a resident plane complete: halo rows and pads
  static constexpr unsigned tx_res_bytes = unsigned((2 * H * SW + 2 * SR * HP) * sizeof(T));
  static_assert(NWC >= 1 && NWC <= 31 && RY >= 1, "launch shape");
  static_assert(H <= V16, "horizontal neighbours are at most one lane away");
  static_assert(SW <= 256 && SR <= 256, "TMA box extent");
};
template <class T, int SHAPE, bool FAST = false, bool RES = false>
using Cfg3D = Cfg3DT<T, SHAPE, Pick3D<T, SHAPE, FAST>::NWC, Pick3D<T, SHAPE, FAST>::RY, Pick3D<T, SHAPE, FAST>::DKB, RES>;

template <class T, int SHAPE, bool FAST, class Cf>
__global__ void __launch_bounds__(Cf::NT, 1) stencil3d_kernel(const __grid_constant__ Stencil3DParams p) {
  constexpr int H = Cf::H, V = Cf::V, V16 = Cf::V16, NV = Cf::NV, SW = Cf::SW, HP = Cf::HP, RY = Cf::RY,
                NWC = Cf::NWC, TY = Cf::TY, PLANE = Cf::PLANE, NR = Cf::NR, MAIN = Cf::MAIN, PADSZ = Cf::PADSZ;
  constexpr bool BOX = Cf::BOX;
  constexpr int WV = V16 + 2 * H;  // horizontal window of one vector
  constexpr int NP = 2 * H + 1;    // planes one output reads

  extern __shared__ __align__(128) unsigned char smem_raw[];
  T* const ring = reinterpret_cast<T*>(smem_raw);
  uint64_t* const full = reinterpret_cast<uint64_t*>(smem_raw + Cf::ring_bytes);
  uint64_t* const empty = full + NR;

  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const bool producer = wid == NWC;
  const int h = p.h, wy = p.wy, wx = p.wx, px = p.px;
  const bool dir = p.dirichlet != 0;
  const long long total = (long long)p.gx * p.gy * h;
  const long long c_lo = total * blockIdx.x / gridDim.x, c_hi = total * (blockIdx.x + 1) / gridDim.x;
  const int nseg = c_hi > c_lo ? int((c_hi - 1) / h - c_lo / h + 1) : 0;
  // resident planes: [rz0, rz0 + rn) of tile rtile, the segment with the most
  // planes that no other CTA reads
  int rtile = -1, rz0 = 0, rn = 0;
  if (Cf::RES && p.kr > 0) {
    for (int k = 0; k < nseg; k++) {
      const long long tb = c_lo / h + k;
      const int zl = int(max(c_lo, tb * h) - tb * h), zh = int(min(c_hi, (tb + 1) * h) - tb * h);
      const int a = zl + H, b = zh - H;
      const int n = min(p.kr, b - a);
      if (n > rn) {
        rn = n;
        rtile = int(tb);
        rz0 = a;
      }
    }
  }
  T* const resb = reinterpret_cast<T*>(smem_raw + Cf::res_offset);  // [rn][TY][SW]
  auto res_index = [&](int tile, int z) {
    if constexpr (!Cf::RES) return -1;
    return (tile == rtile && z >= rz0 && z < rz0 + rn) ? z - rz0 : -1;
  };

  if (threadIdx.x == 0) {
    for (int i = 0; i < NR; i++) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], NWC);
    }
    fence_mbar_init();
  }
  // the resident planes' tiles from the input field (each compute warp its
  // own rows)
  if (Cf::RES && rn > 0 && !producer) {
    const T* f0 = static_cast<const T*>(p.f[p.t0 & 1]);
    const int x0 = (rtile % p.gx) * SW, y0 = (rtile / p.gx) * TY;
    for (int j = 0; j < rn; j++) {
      for (int r = wid * RY; r < wid * RY + RY; r++) {
        if (y0 + r >= wy) break;
        const T* src = f0 + (size_t(rz0 + j) * wy + y0 + r) * px + x0 + lane * V16;
        T* dst = resb + (size_t(j) * TY + r) * SW + lane * V16;
#pragma unroll
        for (int k2 = 0; k2 < NV; k2++) {
          if (x0 + k2 * 32 * V16 + lane * V16 < px) {
            T v[V16];
            vec16_load(src + k2 * 32 * V16, v);
            vec16_store(dst + k2 * 32 * V16, v);
          }
        }
      }
    }
  }
  __syncthreads();

  GridBarrier gbar{p.bar, p.status, gridDim.x, p.ctl};
  const uint64_t pol = policy_evict_normal();
  bool ok = true;
  // Positions: every plane a CTA loads gets the next global position P; its
  // slot is P % NR, and the k-th use of a slot (k = P / NR) completes phase k
  // of the slot's full barrier and, once all compute warps are done with it,
  // phase k of its empty barrier.
  long long pc = 0;      // positions of all finished segments
  long long issued = 0;  // producer: positions issued so far

  for (int it = 0; it < p.steps && ok; it++) {
    const int t = p.t0 + it;
    const T* fin = static_cast<const T*>(p.f[t & 1]);
    T* fout = static_cast<T*>(p.f[(t + 1) & 1]);
    const bool fwd = !p.alternate || (t & 1) == 0;
    if (producer && it > 0) fence_proxy_async_global();
    for (int k = 0; k < nseg && ok; k++) {
      const long long tb = c_lo / h + (fwd ? k : nseg - 1 - k);  // tile of this segment
      const int z_lo = int(max(c_lo, tb * h) - tb * h), z_hi = int(min(c_hi, (tb + 1) * h) - tb * h);
      const int ZN = z_hi - z_lo;
      const int tile = int(tb);
      const int x0 = (tile % p.gx) * SW, y0 = (tile / p.gx) * TY;
      // segment position q in [-H, ZN+H) is global position pc + H + q
      const int sb = int((pc + H) % NR);
      const unsigned par0 = unsigned(((pc + H) / NR + 1) & 1);
      auto slot_index = [&](int q) { return (sb + q + NR) % NR; };
      auto slot_parity = [&](int q) { return (par0 + unsigned((sb + q + NR) / NR)) & 1u; };

      if (producer) {
        for (int q = -H; q < ZN + H; q++) {
          const int s = slot_index(q);
          if (pc + H + q >= NR) {  // wait until every compute warp released the slot's previous plane
            bool w = mbar_wait(&empty[s], slot_parity(q) ^ 1u, p.ctl.budget);
            w = __all_sync(0xffffffffu, w);
            if (!w) {
              if (lane == 0) atomicOr(p.status, kErrCopyTimeout);
              ok = false;
              break;
            }
          }
          const int z = fwd ? z_lo + q : z_hi - 1 - q;
          const int rj = (Cf::RES && z >= 0 && z < h) ? res_index(tile, z) : -1;
          if (Cf::RES && rj >= 0) {
            // the resident tile into the slot's interior rows, by the whole
            // warp, before the arrival that lets the compute warps read it
            T* dst = ring + size_t(s) * PLANE + H * SW;
            const T* src = resb + size_t(rj) * TY * SW;
            for (int e = lane * V16; e < TY * SW; e += 32 * V16) {
              T v[V16];
              vec16_load(src + e, v);
              vec16_store(dst + e, v);
            }
            __syncwarp();
          }
          if (lane == 0) {
            if (z >= 0 && z < h) {
              T* slot = ring + size_t(s) * PLANE;
              if (!Cf::RES || rj < 0) {
                mbar_arrive_expect_tx(&full[s], Cf::tx_bytes);
                tma_load_3d(slot, &p.map[t & 1], x0, y0 - H, z, &full[s], pol);
              } else {  // interior rows from the resident tile, halo rows from the field
                mbar_arrive_expect_tx(&full[s], Cf::tx_res_bytes);
                tma_load_3d(slot, &p.hmap[t & 1], x0, y0 - H, z, &full[s], pol);
                tma_load_3d(slot + (H + TY) * SW, &p.hmap[t & 1], x0, y0 + TY, z, &full[s], pol);
              }
              tma_load_3d(slot + MAIN, &p.pmap[t & 1], x0 - HP, y0 - H, z, &full[s], pol);
              tma_load_3d(slot + MAIN + PADSZ, &p.pmap[t & 1], x0 + SW, y0 - H, z, &full[s], pol);
            } else {
              mbar_arrive_expect_tx(&full[s], 0u);  // a plane outside the domain: never read
            }
          }
          __syncwarp();
          issued = pc + H + q + 1;
        }
      } else {
        // Lane layout: vector k (V16 elements, 16 bytes) of a lane holds tile
        // columns k*32*V16 + lane*V16 + [0, V16), so every warp-wide 16-byte
        // access is one contiguous 512-byte run (no bank conflicts).
        const bool ghost = !dir && x0 + SW > wx;  // columns past the domain inside the tile
        const int lw = wx - 1 - x0;               // tile-local last column
        const int lw_i = min(lw / (32 * V16), NV - 1) * V16 + lw % V16;  // its element index
        const int lw_lane = (lw / V16) & 31;                              // and lane
        auto col = [&](int i) { return (i / V16) * (32 * V16) + lane * V16 + i % V16; };
        auto plane_ptr = [&](int z) -> const T* {
          const int zc = min(max(z, 0), h - 1);
          const int q = fwd ? zc - z_lo : z_hi - 1 - zc;
          return ring + size_t(slot_index(q)) * PLANE;
        };
        // a row of a slot: its index there (clamped to the domain)
        struct RowRef {
          const T* plane;
          int ri;
        };
        auto row_ref = [&](const T* plane, int y) -> RowRef {
          return RowRef{plane, min(max(y, 0), wy - 1) - (y0 - H)};
        };
        // this lane's V values of a row; in a ghost tile columns past the
        // domain take the value of column wx-1
        auto load_vals = [&](RowRef rw, T(&v)[V]) {
          const T* row = rw.plane + rw.ri * SW;
#pragma unroll
          for (int k = 0; k < NV; k++) vec16_load(row + k * 32 * V16 + lane * V16, v + k * V16);
          if (ghost) {
            T edge = v[0];
#pragma unroll
            for (int i = 1; i < V; i++) edge = (lw_i == i) ? v[i] : edge;
            edge = __shfl_sync(0xffffffffu, edge, lw_lane);
#pragma unroll
            for (int i = 0; i < V; i++) v[i] = (col(i) > lw) ? edge : v[i];
          }
        };
        // per vector: its V16 values with H neighbours on each side. A lane
        // sends the value its right (left) neighbour lane needs; lane 31 (0)
        // sends from the previous (next) vector, which is what lane 0 (31)
        // needs across the vector boundary. The tile's outer neighbours are
        // read at the clamped column from the tile row or a pad strip (every
        // lane reads the same word: a broadcast).
        auto hwin = [&](RowRef rw, const T(&v)[V], T(&w)[NV][WV]) {
          const T* row = rw.plane + rw.ri * SW;
          const T* padl = rw.plane + MAIN + rw.ri * HP;
          const T* padr = rw.plane + MAIN + PADSZ + rw.ri * HP;
#pragma unroll
          for (int k = 0; k < NV; k++) {
#pragma unroll
            for (int e = 0; e < V16; e++) w[k][H + e] = v[k * V16 + e];
#pragma unroll
            for (int d = 1; d <= H; d++) {
              const T give_l = (k > 0 && lane == 31) ? v[(k - 1) * V16 + V16 - d] : v[k * V16 + V16 - d];
              const T give_r = (k + 1 < NV && lane == 0) ? v[(k + 1) * V16 + d - 1] : v[k * V16 + d - 1];
              const T from_l = __shfl_sync(0xffffffffu, give_l, (lane + 31) & 31);
              const T from_r = __shfl_sync(0xffffffffu, give_r, (lane + 1) & 31);
              if (k == 0) {
                const T pad = *(x0 == 0 ? row : padl + HP - d);  // column max(x0-d, 0)
                w[k][H - d] = lane > 0 ? from_l : pad;
              } else {
                w[k][H - d] = from_l;
              }
              if (k == NV - 1) {
                const int c = min(SW + d - 1, lw);  // tile-local column min(x0+SW+d-1, wx-1)
                const T pad = *(c < SW ? row + c : padr + (c - SW));
                w[k][H + V16 - 1 + d] = lane < 31 ? from_r : pad;
              } else {
                w[k][H + V16 - 1 + d] = from_r;
              }
            }
          }
        };

        int wq = -H;  // next segment position to wait for
        for (int q = 0; q < ZN && ok; q++) {
          for (; wq <= q + H; wq++) {
            bool w = mbar_wait(&full[slot_index(wq)], slot_parity(wq), p.ctl.budget);
            w = __all_sync(0xffffffffu, w);
            if (!w) {
              if (lane == 0) atomicOr(p.status, kErrCopyTimeout);
              ok = false;
              break;
            }
          }
          if (!ok) break;
          const int z = fwd ? z_lo + q : z_hi - 1 - q;
          const T* pl[NP];
#pragma unroll
          for (int j = 0; j < NP; j++) pl[j] = plane_ptr(z - H + j);
          const bool zfix = z < H || z >= h - H;
          const int yw = y0 + wid * RY;  // this warp's first row
          const int rj = res_index(tile, z);
          // one output plane; RP: the plane is resident (its output goes into
          // its tile, and to the field only what the neighbouring tiles
          // read). Instantiated twice, so that the loop of the planes that
          // stream is the plain one.
          auto do_plane = [&](auto rpc) {
            constexpr bool RP = decltype(rpc)::value;
            // finish one output row: Dirichlet cells keep the old value, store
            auto finish = [&](int y, T(&o)[V], const T(&c)[V]) {
              if (dir) {
                const bool fixed = zfix || y < H || y >= wy - H;
#pragma unroll
                for (int i = 0; i < V; i++) {
                  const int x = x0 + col(i);
                  o[i] = (fixed || x < H || x >= wx - H) ? c[i] : o[i];
                }
              }
              if (y < wy) {
                T* dst = fout + (size_t(z) * wy + y) * px + x0 + lane * V16;
                if constexpr (RP) {
                  T* rrow = resb + (size_t(rj) * TY + (y - y0)) * SW + lane * V16;
#pragma unroll
                  for (int k2 = 0; k2 < NV; k2++) sts16_unordered(rrow + k2 * 32 * V16, o + k2 * V16);
                  if (y - y0 < H || y - y0 >= TY - H) {
#pragma unroll
                    for (int k2 = 0; k2 < NV; k2++)
                      if (x0 + k2 * 32 * V16 + lane * V16 < px) vec16_store(dst + k2 * 32 * V16, o + k2 * V16);
                  } else {
                    if (lane == 0) vec16_store(dst, o);
                    if (lane == 31 && x0 + (NV - 1) * 32 * V16 + 31 * V16 < px)
                      vec16_store(dst + (NV - 1) * 32 * V16, o + (NV - 1) * V16);
                  }
                } else {
#pragma unroll
                  for (int k2 = 0; k2 < NV; k2++)
                    if (x0 + k2 * 32 * V16 + lane * V16 < px) vec16_store(dst + k2 * 32 * V16, o + k2 * V16);
                }
              }
            };
            if constexpr (BOX) {
              // rows yw-1 .. yw+RY of the three planes, three at a time
              T bw[3][3][NV][WV];  // [plane][row % 3][vector][window]
              auto bring = [&](int j) {  // row yw-1+j of every plane into bw[.][j % 3]
#pragma unroll
                for (int dz = 0; dz < 3; dz++) {
                  const RowRef rw = row_ref(pl[dz], yw - 1 + j);
                  T v[V];
                  load_vals(rw, v);
                  hwin(rw, v, bw[dz][j % 3]);
                }
              };
              bring(0);
              bring(1);
              static_for<RY>([&](auto ryc) {
                constexpr int ry = decltype(ryc)::value;
                bring(ry + 2);
                T o[V], c[V];
#pragma unroll
                for (int i = 0; i < V; i++) {
                  const int kk = i / V16, e = i % V16;
                  auto u = [&](int dz, int dy, int dx) -> T { return bw[dz + 1][(ry + 1 + dy) % 3][kk][H + e + dx]; };
                  o[i] = stencil_point<T, SHAPE, FAST>(u);
                  c[i] = bw[1][(ry + 1) % 3][kk][H + e];
                }
                finish(yw + ry, o, c);
              });
            } else {
              constexpr int NC = 2 * H + 1;
              T cr[NC][V];  // rolling rows of the centre plane: row yw-H+j in cr[j % NC]
              static_for<2 * H>([&](auto jc) {
                constexpr int j = decltype(jc)::value;
                load_vals(row_ref(pl[H], yw - H + j), cr[j]);
              });
              static_for<RY>([&](auto ryc) {
                constexpr int ry = decltype(ryc)::value;
                const int y = yw + ry;
                load_vals(row_ref(pl[H], y + H), cr[(ry + 2 * H) % NC]);
                T cen[NV][WV];
                hwin(row_ref(pl[H], y), cr[(ry + H) % NC], cen);
                T nz[2 * H][V];  // row y of planes z-H..z-1 then z+1..z+H
#pragma unroll
                for (int d = 1; d <= H; d++) {
                  load_vals(row_ref(pl[H - d], y), nz[H - d]);
                  load_vals(row_ref(pl[H + d], y), nz[H + d - 1]);
                }
                T o[V], c[V];
                if constexpr (sizeof(T) == 4 && !FAST && SHAPE == PERKS_3D7PT) {
                  // FP32 reference order: two adjacent cells per packed
                  // instruction (f32x2.cuh); every result bit as per cell.
                  // 3d7pt only: 3d13pt measured slower in pairs at 512^3
                  // (462 against 484-494 GCells/s), 3d7pt faster (747-749
                  // against 736)
                  const F2 one2(p.one), mone2(-p.one);
#pragma unroll
                  for (int i = 0; i < V; i += 2) {
                    const int kk = i / V16, e = i % V16;
                    auto u2 = [&](int dz, int dy, int dx) -> F2 {
                      if (dz != 0) {
                        const T* a = nz[dz < 0 ? H + dz : H + dz - 1];
                        return F2::pack(a[i], a[i + 1]);
                      }
                      if (dy != 0) return F2::pack(cr[(ry + H + dy) % NC][i], cr[(ry + H + dy) % NC][i + 1]);
                      return F2::pack(cen[kk][H + e + dx], cen[kk][H + e + 1 + dx]);
                    };
                    star3d_ref<F2, SHAPE>(
                        u2, [one2](F2 a, F2 b) { return RN<F2>::fma(b, one2, a); },
                        [mone2](F2 a, F2 b) { return RN<F2>::fma(b, mone2, a); })
                        .unpack(o[i], o[i + 1]);
                    c[i] = cen[kk][H + e];
                    c[i + 1] = cen[kk][H + e + 1];
                  }
                } else {
#pragma unroll
                  for (int i = 0; i < V; i++) {
                    const int kk = i / V16, e = i % V16;
                    auto u = [&](int dz, int dy, int dx) -> T {
                      if (dz != 0) return nz[dz < 0 ? H + dz : H + dz - 1][i];
                      if (dy != 0) return cr[(ry + H + dy) % NC][i];
                      return cen[kk][H + e + dx];
                    };
                    o[i] = stencil_point<T, SHAPE, FAST>(u);
                    c[i] = cen[kk][H + e];
                  }
                }
                finish(y, o, c);
              });
            }
          };
          if constexpr (Cf::RES) {
            if (rj >= 0) do_plane(std::true_type{});
            else do_plane(std::false_type{});
          } else {
            do_plane(std::false_type{});
          }
          // plane at position q-H is not read by later outputs
          __syncwarp();
          if (lane == 0) mbar_arrive(&empty[slot_index(q - H)]);
        }
        if (ok) {  // the segment's last 2H positions are released without an output
          __syncwarp();
          if (lane == 0)
            for (int q = ZN - H; q < ZN + H; q++) mbar_arrive(&empty[slot_index(q)]);
        }
      }
      pc += ZN + 2 * H;
    }
    if (it + 1 < p.steps && p.persistent) {
      fence_proxy_async_global();
      if (!gbar.sync()) ok = false;
    }
  }
  if (Cf::RES && ok && rn > 0 && !producer) {
    // the resident planes into the launch's output field (each lane reads
    // what it stored; the barrier keeps these loads behind those stores)
    __syncwarp();
    asm volatile("" ::: "memory");
    T* fo = static_cast<T*>(p.f[(p.t0 + p.steps) & 1]);
    const int x0 = (rtile % p.gx) * SW, y0 = (rtile / p.gx) * TY;
    for (int j = 0; j < rn; j++) {
      for (int r = wid * RY; r < wid * RY + RY; r++) {
        if (y0 + r >= wy) break;
        const T* src = resb + (size_t(j) * TY + r) * SW + lane * V16;
        T* dst = fo + (size_t(rz0 + j) * wy + y0 + r) * px + x0 + lane * V16;
#pragma unroll
        for (int k2 = 0; k2 < NV; k2++) {
          if (x0 + k2 * 32 * V16 + lane * V16 < px) {
            T v[V16];
            vec16_load(src + k2 * 32 * V16, v);
            vec16_store(dst + k2 * 32 * V16, v);
          }
        }
      }
    }
  }
  if (!ok && producer && lane == 0) {
    // leave no bulk copy in flight into this CTA's shared memory: the last NR
    // issued positions are the only ones whose copies may still be running
    // (a budget of its own, independent of p.ctl: copies end by themselves,
    // and a shortened test budget must not cut this wait short)
    for (long long P = max(0ll, issued - NR); P < issued; P++) {
      const int s = int(P % NR);
      const unsigned par = unsigned((P / NR) & 1);
      const long long t0 = clock64();
      while (!mbar_try_wait(&full[s], par)) {
        if (clock64() - t0 > (1ll << 30)) break;
      }
    }
  }
}

}  // namespace perks
