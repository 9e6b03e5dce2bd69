// 2D Jacobi time loop for sm_103a: persistent cooperative kernel with
// shared-memory-resident rows and a bulk-copy (TMA) row pipeline.
//
// Work decomposition (one CTA per SM):
//   The internal field is row-major with a padded pitch (gx * TX columns).
//   CTA (ti, tj) owns the tile of columns [tj*TX, tj*TX+TX) and rows
//   [r0, r1) (balanced split of width_y over gy tile rows).
//   Each step the CTA sweeps its rows in groups of R output rows. Input rows
//   arrive in a ring of NR shared-memory slots, one cp.async.bulk per row
//   covering the tile plus HP pad columns on each side, completing on a
//   per-slot mbarrier. The first and last H rows of every tile always live
//   in global memory, so neighbouring tiles read their halos straight from
//   the field.
//   PERKS caching: tile rows [r0+H, r0+H+C) stay in shared memory for the
//   whole launch ("resident rows"). They are updated in place with a skew:
//   the output of a row goes into the slot of the row R+H positions behind it
//   in the sweep (dead by then), so no extra buffer or barrier is needed. The
//   resident rows' first and last HP columns are also stored to the field so
//   that the left/right neighbour tiles can load them as pads.
//   Steps are separated by a bounded grid barrier.
//   With `alternate`, odd steps sweep bottom-up so that the rows written last
//   are read first (still in L2), and input lines that are dead after their
//   last read are dropped from L2 without write-back.
//
// Boundary: clamp-to-edge as the reference. Rows outside the domain alias the
// edge row's slot; columns outside the domain are filled in shared memory
// from the edge column ("fixups") before the rows are read.
#pragma once
#include <cstdint>
#include "ptx.cuh"
#include "shapes.cuh"

namespace perks {

struct Stencil2DParams {
  void* f[2];         // internal fields, pitch elements per row
  int wy, wx, pitch;  // domain and padded row pitch (elements)
  int gx, gy;         // tile grid
  int steps;          // steps run by this launch
  int t0;             // global index of this launch's first step
  int C;              // resident rows per tile (upper bound; tiles clamp to TY-2H)
  int M;              // resident slots (C + R + H), 0 when C == 0
  int dirichlet;      // hold the outer H cells fixed instead of clamping
  int alternate;      // alternate sweep direction + L2 line dropping
  int persistent;     // grid barrier between steps (cooperative launch)
  unsigned* bar;      // grid barrier words [2]
  unsigned* status;   // error word
};

template <class T, int SHAPE, int NT_>
struct Cfg2D {
  static constexpr int H = ShapeInfo<SHAPE>::H;
  static constexpr bool BOX = ShapeInfo<SHAPE>::box;
  static constexpr int NT = NT_;
  static constexpr int V = 16 / sizeof(T);            // elements per 16-byte vector
  static constexpr int TX = NT * V;                    // tile width
  static constexpr int HP = ((H + V - 1) / V) * V;     // pad columns (16-byte multiple)
  static constexpr int RW = TX + 2 * HP;               // shared-memory row width
  static constexpr int R = BOX ? 4 : 8;                // output rows per group
  static constexpr int NR = 2 * R + 2 * H + (BOX ? 8 : 4);  // ring slots (>= 2R + 2H)
  static constexpr int NVW = (V + 2 * HP) / V;         // vectors per full window row
  static_assert(NR <= 64, "phase mask holds 64 slots");
  static constexpr size_t ring_bytes = size_t(NR) * RW * sizeof(T);
  static constexpr size_t row_bytes = size_t(RW) * sizeof(T);
  static constexpr size_t bar_bytes = (NR + 2) * sizeof(uint64_t);
};

template <class T>
struct Vec;
template <>
struct Vec<float> {
  using type = float4;
};
template <>
struct Vec<double> {
  using type = double2;
};

template <class T, int SHAPE, bool FAST, int NT>
__global__ void __launch_bounds__(NT, 1) stencil2d_kernel(const __grid_constant__ Stencil2DParams p) {
  using Cf = Cfg2D<T, SHAPE, NT>;
  using VT = typename Vec<T>::type;
  constexpr int H = Cf::H, V = Cf::V, TX = Cf::TX, HP = Cf::HP, RW = Cf::RW, R = Cf::R, NR = Cf::NR;
  constexpr int WROWS = R + 2 * H;     // window rows per group
  constexpr int NVW = Cf::NVW;
  constexpr int WW = V + 2 * HP;       // window width (elements)

  extern __shared__ __align__(128) unsigned char smem_raw[];
  T* ring = reinterpret_cast<T*>(smem_raw);
  T* res = ring + NR * RW;
  uint64_t* bars = reinterpret_cast<uint64_t*>(res + size_t(p.M) * RW);
  uint64_t* bar_res = bars + NR;

  const int tid = threadIdx.x;
  const int ti = blockIdx.x / p.gx, tj = blockIdx.x % p.gx;
  const int r0 = int((long long)ti * p.wy / p.gy);
  const int r1 = int((long long)(ti + 1) * p.wy / p.gy);
  const int TY = r1 - r0;
  const int x0 = tj * TX;
  const int C = (p.M > 0) ? max(0, min(p.C, TY - 2 * H)) : 0;
  const int rres0 = r0 + H;
  const int M = p.M;
  const int wy = p.wy, wx = p.wx, pitch = p.pitch;
  const bool left_edge = (tj == 0) && !p.dirichlet;
  const bool right_edge = (tj == p.gx - 1) && !p.dirichlet;
  const int lw = wx - 1 - x0;  // tile-local index of the last domain column (right edge tile)
  // Source window of one row copy: [x0-HP, x0+TX+HP) clipped to the pitch.
  const int src_lo = max(x0 - HP, 0);
  const int src_hi = min(x0 + TX + HP, pitch);
  const int dst_off = src_lo - (x0 - HP);
  const unsigned copy_bytes = unsigned(src_hi - src_lo) * sizeof(T);
  const bool has_w = x0 - HP >= 0, has_e = x0 + TX + HP <= pitch;

  GridBarrier gbar{p.bar, p.status, gridDim.x * gridDim.y * gridDim.z};
  const uint64_t pol = policy_evict_normal();
  const uint64_t pol_first = policy_evict_first();

  if (tid == 0) {
    for (int i = 0; i < NR + 1; i++) mbar_init(&bars[i], 1);
    fence_mbar_init();
  }
  __syncthreads();

  uint64_t phase = 0ull;    // per ring slot parity (identical in every thread)
  uint32_t res_phase = 0u;
  int off = 0;             // resident skew (mod M)
  bool ok = true;
  int issued = 0, waited = 0;  // sweep positions issued / waited this step (drain on error)
  bool fwd = true;

  auto slot_of_res = [&](int r) -> T* {
    int s = (r - rres0 + off) % M;
    if (s < 0) s += M;
    return res + size_t(s) * RW;
  };
  auto fixup_row = [&](T* slot, int which) {
    // which 0: left edge, 1: right edge. Columns outside the domain take the
    // value of the edge column.
    if (which == 0) {
      const T v = slot[HP];
#pragma unroll
      for (int k = 1; k <= H; k++) slot[HP - k] = v;
    } else {
      const T v = slot[HP + lw];
#pragma unroll
      for (int k = 1; k <= H; k++) slot[HP + lw + k] = v;
    }
  };

  // ---------------------------------------------------------------- prologue
  // Bring the resident rows in from the field once per launch.
  if (C > 0) {
    const T* fin = static_cast<const T*>(p.f[p.t0 & 1]);
    if (tid == 0) {
      mbar_arrive_expect_tx(bar_res, copy_bytes * unsigned(C));
      for (int r = rres0; r < rres0 + C; r++)
        bulk_g2s(slot_of_res(r) + dst_off, fin + size_t(r) * pitch + src_lo, copy_bytes, bar_res, pol);
    }
    if (!mbar_wait(bar_res, res_phase & 1u)) {
      atomicOr(p.status, kErrCopyTimeout);
      ok = false;
    }
    res_phase ^= 1u;
    ok = __syncthreads_and(ok);
  }

  for (int it = 0; it < p.steps && ok; it++) {
    const int t = p.t0 + it;
    const T* fin = static_cast<const T*>(p.f[t & 1]);
    T* fout = static_cast<T*>(p.f[(t + 1) & 1]);
    fwd = !p.alternate || ((t & 1) == 0);
    // Row of sweep position s (positions -H..TY+H-1 include the halo rows).
    auto row_of = [&](int s) { return fwd ? r0 + s : r1 - 1 - s; };
    auto is_res = [&](int r) { return C > 0 && r >= rres0 && r < rres0 + C; };
    auto loaded = [&](int s) {
      const int r = row_of(s);
      return r >= 0 && r < wy && !is_res(r);
    };
    auto pos_of = [&](int r) { return fwd ? r - r0 : r1 - 1 - r; };
    auto slot_of = [&](int r) -> T* {
      // shared-memory slot holding input row r (clamped to the domain)
      r = min(max(r, 0), wy - 1);
      if (is_res(r)) return slot_of_res(r);
      const int s = pos_of(r);
      return ring + size_t((s + H) % NR) * RW;
    };

    issued = -H;  // next sweep position the producer will issue
    auto produce = [&](int upto) {
      // thread 0 only: issue row copies for positions < upto
      const int lim = min(upto, TY + H);
      for (; issued < lim; issued++) {
        if (!loaded(issued)) continue;
        const int r = row_of(issued);
        uint64_t* b = &bars[(issued + H) % NR];
        T* dst = ring + size_t((issued + H) % NR) * RW + dst_off;
        mbar_arrive_expect_tx(b, copy_bytes);
        // interior rows are read only by this CTA: evict them first from L2
        const bool interior = r >= r0 + H && r < r1 - H;
        bulk_g2s(dst, fin + size_t(r) * pitch + src_lo, copy_bytes, b,
                 (p.alternate && interior) ? pol_first : pol);
      }
    };

    if (tid == 0) {
      fence_proxy_async_global();
      produce(NR - H);
      if (C > 0 && it > 0 && (has_w || has_e)) {
        // refresh the resident rows' pad columns from the neighbours' stores
        const unsigned pb = HP * sizeof(T);
        mbar_arrive_expect_tx(bar_res, pb * unsigned(C) * unsigned(has_w + has_e));
        for (int r = rres0; r < rres0 + C; r++) {
          T* s = slot_of_res(r);
          if (has_w) bulk_g2s(s, fin + size_t(r) * pitch + x0 - HP, pb, bar_res, pol);
          if (has_e) bulk_g2s(s + HP + TX, fin + size_t(r) * pitch + x0 + TX, pb, bar_res, pol);
        }
      }
    }
    if (C > 0 && it > 0 && (has_w || has_e)) {
      if (!mbar_wait(bar_res, res_phase & 1u)) {
        atomicOr(p.status, kErrCopyTimeout);
        ok = false;
      }
      res_phase ^= 1u;
      ok = __syncthreads_and(ok);
      if (!ok) break;
    }
    if (C > 0 && (left_edge || right_edge)) {
      for (int k = tid; k < C; k += NT) {
        T* s = slot_of_res(rres0 + k);
        if (left_edge) fixup_row(s, 0);
        if (right_edge) fixup_row(s, 1);
      }
    }

    waited = -H;
    for (int lo = 0; lo < TY && ok; lo += R) {
      const int hi = min(lo + R, TY);
      const int need_hi = hi + H;
      for (; waited < need_hi; waited++) {
        if (!loaded(waited)) continue;
        const int q = (waited + H) % NR;
        if (!mbar_wait(&bars[q], unsigned(phase >> q) & 1u)) {
          atomicOr(p.status, kErrCopyTimeout);
          ok = false;
          break;
        }
        phase ^= (1ull << q);
        T* slot = ring + size_t(q) * RW;
        if (left_edge && tid == (waited & 31)) fixup_row(slot, 0);
        if (right_edge && tid == 32 + (waited & 31)) fixup_row(slot, 1);
      }
      ok = __syncthreads_and(ok);
      if (!ok) break;
      if (tid == 0) produce(lo - H + NR);

      // rows of this group in increasing row order
      const int ra = fwd ? r0 + lo : r1 - hi;   // first output row
      const int nrows = hi - lo;
      const int c0 = tid * V;  // window start in slot coordinates (= column x0 + c0 - HP)
      // Star shapes: the middle V columns of every window row stay in
      // registers; the full-width window of each centre row is loaded just
      // before its outputs are computed. Box shapes keep full windows.
      constexpr int WCOL = Cf::BOX ? WW : V;
      constexpr int WOFF = Cf::BOX ? 0 : HP;   // slot column of w[.][0] relative to c0
      T w[WROWS][WCOL];
#pragma unroll
      for (int i = 0; i < WROWS; i++) {
        if (i < nrows + 2 * H) {
          const T* s = slot_of(ra - H + i) + c0 + WOFF;
#pragma unroll
          for (int v = 0; v < WCOL / V; v++) {
            VT x = reinterpret_cast<const VT*>(s)[v];
            const T* xe = reinterpret_cast<const T*>(&x);
#pragma unroll
            for (int e = 0; e < V; e++) w[i][v * V + e] = xe[e];
          }
        }
      }
#pragma unroll
      for (int k = 0; k < R; k++) {
        if (k < nrows) {
          const int y = ra + k;
          T cw[Cf::BOX ? 1 : WW];
          if constexpr (!Cf::BOX) {
            const T* s = slot_of(y) + c0;
#pragma unroll
            for (int v = 0; v < NVW; v++) {
              VT x = reinterpret_cast<const VT*>(s)[v];
              const T* xe = reinterpret_cast<const T*>(&x);
#pragma unroll
              for (int e = 0; e < V; e++) cw[v * V + e] = xe[e];
            }
          }
          T o[V];
#pragma unroll
          for (int e = 0; e < V; e++) {
            auto u = [&](int, int dy, int dx) -> T {
              if constexpr (Cf::BOX) return w[k + H + dy][HP + e + dx];
              else return dy == 0 ? cw[HP + e + dx] : w[k + H + dy][e];
            };
            o[e] = stencil_point<T, SHAPE, FAST>(u);
          }
          if (p.dirichlet) {
            const bool row_fixed = (y < H) || (y >= wy - H);
#pragma unroll
            for (int e = 0; e < V; e++) {
              const int x = x0 + c0 + e;
              const T old = Cf::BOX ? w[k + H][HP + e] : w[k + H][e];
              if (row_fixed || x < H || x >= wx - H) o[e] = old;
            }
          }
          VT ov;
          T* oe = reinterpret_cast<T*>(&ov);
#pragma unroll
          for (int e = 0; e < V; e++) oe[e] = o[e];
          if (is_res(y)) {
            // in-place update with skew: the slot of the row R+H positions behind
            const int tr = fwd ? y - (R + H) : y + (R + H);
            int s = (tr - rres0 + off) % M;
            if (s < 0) s += M;
            *reinterpret_cast<VT*>(res + size_t(s) * RW + HP + c0) = ov;
            if (c0 < HP || c0 >= TX - HP)
              *reinterpret_cast<VT*>(fout + size_t(y) * pitch + x0 + c0) = ov;
          } else {
            *reinterpret_cast<VT*>(fout + size_t(y) * pitch + x0 + c0) = ov;
          }
        }
      }
    }
    if (!ok) break;
    // Every issued copy has been waited for (positions up to TY+H-1).
    off = fwd ? off - (R + H) : off + (R + H);
    off %= (M > 0 ? M : 1);
    if (off < 0) off += M;
    if (it + 1 < p.steps) {
      fence_proxy_async_global();
      if (p.persistent) {
        if (!gbar.sync()) { ok = false; break; }
      }
    }
  }
  // ---------------------------------------------------------------- epilogue
  if (ok && C > 0) {
    __syncthreads();
    T* fnew = static_cast<T*>(p.f[(p.t0 + p.steps) & 1]);
    for (int k = 0; k < C; k++) {
      const int r = rres0 + k;
      *reinterpret_cast<VT*>(fnew + size_t(r) * pitch + x0 + tid * V) =
          *reinterpret_cast<const VT*>(slot_of_res(r) + HP + tid * V);
    }
  }
  if (!ok) {
    // Leave no bulk copy in flight into this CTA's shared memory: thread 0
    // waits (bounded) for every position it issued that was not yet waited.
    __syncthreads();
    if (tid == 0) {
      uint64_t ph = phase;
      for (int s = waited; s < issued; s++) {
        const int r = fwd ? r0 + s : r1 - 1 - s;
        if (r < 0 || r >= wy || (C > 0 && r >= rres0 && r < rres0 + C)) continue;
        const int q = (s + H) % NR;
        long long tw = clock64();
        while (!mbar_try_wait(&bars[q], unsigned(ph >> q) & 1u)) {
          if (clock64() - tw > (1ll << 28)) break;
        }
        ph ^= (1ull << q);
      }
    }
  }
}

}  // namespace perks
