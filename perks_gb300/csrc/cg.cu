// Conjugate gradient for sm_103a: one persistent cooperative launch per
// solve (or one launch per phase, as the comparator), CSR or DIA matrices,
// FP64, FP32 (the reference's float build) or mixed precision.
//
// Iteration (cpuConjugateGrad, conjugateGradient/cg_cpu.cpp:40-81, with the
// stop test of the reference GPU kernel, conjugateGradient/cg_kernels.cuh:834):
//   p = r (first) or p = r + beta p;  Ap = A p;  alpha = rr / p.Ap;
//   x += alpha p;  r -= alpha Ap;  rr' = r.r;  beta = rr' / rr
// FP64: three grid barriers per iteration: after p (the SpMV gathers it),
// after the p.Ap reduction, after the r.r reduction. FP32 and the FP32 inner
// iteration of mixed precision form p on the fly in the SpMV gather instead
// (p_j = beta*p_old_j + r_j, the same fma its owner applies, so the values are
// identical) with p double-buffered, saving the p pass and one barrier; for
// FP64 the extra fma per nonzero would cost more FP64 issue than it saves
// (GB300 runs FP64 at 1/64 of FP32). Dot products are reduced
// deterministically: each CTA writes one partial sum, and after the barrier
// every CTA adds all partials in the same fixed order, so all CTAs derive
// identical alpha / beta without atomics.
//
// CSR rows are split between CTAs by a merge-path split of rows + nonzeros,
// so irregular rows are balanced. A CSR matrix with sorted, unique columns
// whose entries lie on at most 32 diagonals (DIA padding <= 25%) is copied at
// the start of the solve into the DIA layout (diagonals ascending = columns
// ascending, the CSR entry order). Otherwise, a CSR matrix whose longest row has at most
// 64 entries and whose rows are near that length (ELL padding <= 25%, e.g.
// the Laplacians) is copied at the start of the solve into a column-major ELL
// layout (entry k of row i at k*n + i, short rows padded with column i and
// value 0): the SpMV then reads it coalesced, four rows per thread, in the
// CSR entry order. The running sum is never -0 (it starts at +0 and exact
// cancellation rounds to +0), so a padding term fma(0, x_i, acc) leaves it
// unchanged and the results equal the CSR ones for finite values.
//
// Mixed precision (reliable updates, Sleijpen & van der Vorst 1996): the
// Krylov iteration runs in FP32 (FP32 copy of the matrix values and FP32
// vectors, dot products accumulated in FP64); the solution is accumulated in
// FP64 and whenever the FP32 recursive residual has dropped by `delta` since
// the last update (or claims convergence), x += x_s in FP64 and the true
// residual r = b - A x is recomputed with the FP64 matrix and re-injected.
// Convergence is only declared on an FP64 true residual.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include "ptx.cuh"
#include "runtime.cuh"

namespace perks {

constexpr int kCgThreads = 1024;
constexpr int kCgResidentKB = 160;  // default shared-memory residency budget per CTA (DIA / ELL layouts)
constexpr int kMaxDiag = 32;

// SELL-C-sigma (Kreutzer et al., "A unified sparse matrix data format for
// efficient general sparse matrix-vector multiplication on modern processors
// with wide SIMD units", SIAM J. Sci. Comput. 36(5), 2014) with C = 32: rows
// sorted by length (longest first) within windows of kSellWindow rows, cut
// into slices of 32 rows; a slice stores its entries column-major, entry k of
// slot l at sl_ptr[slice] + 32 k + l, padded to its longest row with column =
// the slot's own row and value 0. One lane computes one row in CSR entry
// order, so a warp's loads of values and columns are coalesced and rows of
// similar length share a warp.
constexpr int kSellWindow = 1024;

struct CgMat {
  int n, nnz, fmt;        // fmt 0 = CSR, 1 = DIA, 2 = ELL (column-major, ew entries per row), 3 = SELL
  const int* rp;          // CSR
  const int* ci;
  const void* val;        // CSR values or DIA data (dtype of the solve, FP64 for mixed)
  int ndiag;
  int off[kMaxDiag];
  const int* eci;         // ELL column indices [ew][n]; SELL column indices
  int ew;
  int grp;                // CSR: lanes per row in the SpMV phase (4, 8, 16 or 32)
  const int* sl_ptr;      // SELL: [nslices + 1] first entry of each slice
  const int* sl_row;      // SELL: [nslices * 32] row of each slot (n: an empty padding slot)
  int nslices;
};

struct CgParams {
  CgMat A;                // the working-precision SpMV (may be the ELL copy)
  CgMat A64;              // mixed precision: the FP64 matrix as given (true residual)
  const void* b;
  void* x;                // in: x0, out: solution (FP64 for FP64/mixed, FP32 for FP32)
  void* r;                // working vectors, working precision
  void* p[2];             // p; FP32 and mixed alternate the two buffers between iterations
  void* Ap;
  // mixed precision extras
  float* val32;           // FP32 copy of the matrix values, in A's layout (built before the launch)
  float* xs;              // FP32 solution increment
  double* part;           // [4][gridDim] partial sums
  double tol;
  int stop, max_iter, static_iter, replace_every;
  double delta2;          // reliable-update threshold (squared)
  int* out_iter;          // iterations done
  int* out_outer;         // reliable updates done
  double* out_rr;         // final r.r, then r.r one iteration earlier, then b.b
  // rows per CTA kept in shared memory for the whole solve (multiples of 4;
  // 0 = streamed): r (or, mixed, its FP32 r), x (mixed: x_s), Ap
  int cap_r, cap_x, cap_ap;
  int cluster;            // CTAs per thread-block cluster of the launch (1 = no cluster combine)
  // resume from a checkpoint: r and p already in place, scalars here
  int resume, k0;         // k0 = iterations completed before this launch
  double rr0, rrp0, bb0;
  double maxrr0;          // mixed: r.r at the last reliable update
  int outer0, since0;     // mixed: reliable updates done, iterations since the last one
  int keep_state;         // a checkpoint takes the final state
  unsigned* bar;
  unsigned* status;
  WaitCtl ctl;
};

// SELL: first slice of CTA `c`, splitting the slices by their padded
// entries + rows. The SpMV of a CTA then writes rows that other CTAs own in
// the row-wise phases (those are split evenly), so r and Ap of a SELL solve
// stay in global memory.
__device__ __forceinline__ int sell_split(const CgMat& A, int c, int ncta) {
  const long long total = (long long)A.sl_ptr[A.nslices] + 32ll * A.nslices;
  const long long target = total * c / ncta;
  int lo = 0, hi = A.nslices;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if ((long long)A.sl_ptr[mid] + 32ll * mid < target) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// First row of CTA `c` in the row-wise phases: CSR by a merge-path split
// (row + row_ptr[row] >= c*(n+nnz)/ncta), the other layouts evenly.
__device__ __forceinline__ int cg_split(const CgMat& A, int c, int ncta) {
  if (A.fmt != 0) return int((long long)A.n * c / ncta);
  const long long target = (long long)(A.n + (long long)A.nnz) * c / ncta;
  int lo = 0, hi = A.n;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if ((long long)mid + A.rp[mid] < target) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// SELL SpMV over slices [s0, s1); lane l computes the row of slot l in CSR
// entry order (padding entries add fma(0, x_row, acc) = acc: the sum is
// never -0) and runs epi(row, sum) for a slot that holds a row. The slices of
// a window are sorted longest first, so with one warp per slice of a window
// (32 warps, 32 slices per window) warp w takes slice w of even windows and
// slice 31 - w of odd ones: every warp gets long and short slices alike (a
// plain round-robin gave warp 0 the longest slice of every window, and the
// CTA waited for it). Fixed assignment, so the partial sums are reproducible.
template <class XV, class MV, class XF, class Epi>
__device__ __forceinline__ void sell_rows(const CgMat& A, const MV* __restrict__ val, int s0, int s1, const XF& xv,
                                          Epi&& epi) {
  constexpr int SPW = kSellWindow / 32;  // slices per window
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5, w = threadIdx.x >> 5;
  const bool snake = nw == SPW;
  const int first = snake ? s0 / SPW : s0 + w, last = snake ? (s1 - 1) / SPW : s1 - 1, stride = snake ? 1 : nw;
  for (int it = first; it <= last; it += stride) {
    const int s = snake ? it * SPW + ((it & 1) ? SPW - 1 - w : w) : it;
    if (s < s0 || s >= s1) continue;
    const int e0 = __ldg(A.sl_ptr + s), e1 = __ldg(A.sl_ptr + s + 1);
    const int row = __ldg(A.sl_row + s * 32 + lane);
    XV acc = XV(0);
    // batches of U entries: all column and value loads, then all gathers,
    // then the multiply-adds in entry order (the chain column -> x -> fma
    // would otherwise leave one gather per lane in flight)
    constexpr int U = 8;
    int e = e0 + lane;
    for (; e + 32 * (U - 1) < e1; e += 32 * U) {
      int c[U];
      MV a[U];
      XV g[U];
#pragma unroll
      for (int u = 0; u < U; u++) c[u] = __ldg(A.eci + e + 32 * u);
#pragma unroll
      for (int u = 0; u < U; u++) a[u] = __ldg(val + e + 32 * u);
#pragma unroll
      for (int u = 0; u < U; u++) g[u] = xv(c[u]);
#pragma unroll
      for (int u = 0; u < U; u++) acc = fma(XV(a[u]), g[u], acc);
    }
    for (; e < e1; e += 32) acc = fma(XV(__ldg(val + e)), xv(__ldg(A.eci + e)), acc);
    if (row < A.n) epi(row, acc);
  }
}

// Row i of A times a vector given by xv(column). Accumulates in the working
// precision XV (double for FP64, float for FP32).
// FMT >= 0 fixes the format at compile time (the other paths drop out).
template <class XV, int FMT = -1, class MV, class XF>
__device__ __forceinline__ XV spmv_row_f(const CgMat& A, const MV* __restrict__ val, const XF& xv, int i) {
  const int fmt = FMT >= 0 ? FMT : A.fmt;
  XV acc = XV(0);
  if (fmt == 0) {
    const int j0 = __ldg(A.rp + i), j1 = __ldg(A.rp + i + 1);
    int j = j0;
    // four independent gathers in flight per row
    for (; j + 4 <= j1; j += 4) {
      const int c0 = __ldg(A.ci + j), c1 = __ldg(A.ci + j + 1), c2 = __ldg(A.ci + j + 2), c3 = __ldg(A.ci + j + 3);
      const XV v0 = XV(__ldg(val + j)), v1 = XV(__ldg(val + j + 1)), v2 = XV(__ldg(val + j + 2)), v3 = XV(__ldg(val + j + 3));
      const XV x0 = xv(c0), x1 = xv(c1), x2 = xv(c2), x3 = xv(c3);
      acc = fma(v0, x0, acc);
      acc = fma(v1, x1, acc);
      acc = fma(v2, x2, acc);
      acc = fma(v3, x3, acc);
    }
    for (; j < j1; j++) acc = fma(XV(__ldg(val + j)), xv(__ldg(A.ci + j)), acc);
  } else if (fmt == 2) {
    for (int k = 0; k < A.ew; k++) {
      const size_t e = (size_t)k * A.n + i;
      acc = fma(XV(__ldg(val + e)), xv(__ldg(A.eci + e)), acc);
    }
  } else {
#pragma unroll 8
    for (int k = 0; k < A.ndiag; k++) {
      const int c = i + A.off[k];
      const XV a = XV(__ldg(val + (size_t)k * A.n + i));
      if (c >= 0 && c < A.n) acc = fma(a, xv(c), acc);
    }
  }
  return acc;
}
template <int FMT = -1, class MV, class XV>
__device__ __forceinline__ XV spmv_row(const CgMat& A, const MV* __restrict__ val, const XV* __restrict__ x, int i) {
  return spmv_row_f<XV, FMT>(A, val, [x](int c) { return x[c]; }, i);
}

// Block-wide sum of two doubles; result valid in every thread.
__device__ __forceinline__ void block_sum2(double& a, double& b) {
  __shared__ double sa[32], sb[32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  __syncthreads();
  if (lane == 0) {
    sa[w] = a;
    sb[w] = b;
  }
  __syncthreads();
  const int nw = blockDim.x >> 5;
  a = lane < nw ? sa[lane] : 0.0;
  b = lane < nw ? sb[lane] : 0.0;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
}

// Block-wide sum of NV doubles, valid in thread 0 only: warps reduce by
// shuffles, then warp 0 alone adds the warp sums (FP64 issue is scarce).
// WARP_DONE: lane 0 of every warp already holds its warp's sum.
template <int NV, bool WARP_DONE = false>
__device__ __forceinline__ void block_sum_t0(double (&v)[NV]) {
  __shared__ double sw[NV][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if constexpr (!WARP_DONE) {
#pragma unroll
    for (int k = 0; k < NV; k++)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  }
  __syncthreads();  // the previous call's readers are done with sw
  if (lane == 0)
#pragma unroll
    for (int k = 0; k < NV; k++) sw[k][w] = v[k];
  __syncthreads();
  if (w == 0) {
    const int nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NV; k++) {
      v[k] = lane < nw ? sw[k][lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    }
  }
}

constexpr int kMaxCluster = 16;

// Grid-wide deterministic sum: every CTA stores its partials, one barrier,
// then every CTA adds all partials in the same order.
// With thread-block clusters (cl > 1, the launch's cluster size) the CTAs of
// a cluster first combine their partials in the leader CTA's shared memory
// over DSMEM (fixed rank order); only the leaders store partials and arrive
// at the grid barrier (gb.nblocks = clusters), the leader adds the clusters'
// partials in cluster order and hands the total back to its CTAs over DSMEM.
// Every CTA of a cluster passes the same cluster barriers in the same order
// (all decisions below depend only on values the whole cluster shares), so
// no CTA waits on a cluster barrier that a peer skips; a failed wait ends the
// kernel in every CTA after one more cluster barrier, so that no CTA leaves
// while a peer still reads its shared memory.
struct GridSum {
  double* part;  // [slot][2][gridDim]
  GridBarrier gb;
  int cl = 1;
  // every CTA of the cluster: the leader's flag, `ok`, after the grid barrier
  __device__ bool cluster_barrier() {
    __shared__ unsigned cl_ok;
    gb.epoch++;
    if (threadIdx.x == 0) __threadfence();  // this CTA's global writes, before the leader arrives
    cluster_sync_all();
    if (cluster_ctarank() == 0 && threadIdx.x < 32) {
      unsigned ok = 0;
      if (threadIdx.x == 0) ok = gb.arrive_wait(int(cluster_index_x())) ? 1u : 0u;
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (threadIdx.x == 0) cl_ok = ok;
    }
    cluster_sync_all();
    __shared__ unsigned my_ok;
    if (threadIdx.x == 0) my_ok = dsmem_ld_u32(dsmem_addr(&cl_ok, 0));
    cluster_sync_all();  // the leader's cl_ok is read before it may change or the leader may leave
    return my_ok != 0;
  }
  __device__ bool bar() { return cl > 1 ? cluster_barrier() : gb.sync(); }
  // `fin(totals)` runs on thread 0 of every CTA before the totals are
  // broadcast: scalars derived from them (the CG quotients) are computed once
  // per CTA and published in shared memory by the same barrier. A double
  // division is a long FP64 sequence, and FP64 issue on this GPU is 2 lanes
  // per clock per SM: all 1024 threads dividing would take microseconds.
  struct NoFin {
    __device__ void operator()(const double*) const {}
  };
  template <int NV, class Fin>
  __device__ bool sum_cluster(int slot, double (&v)[NV], const Fin& fin) {
    __shared__ double cl_part[kMaxCluster][NV];
    __shared__ double cl_tot[NV];
    __shared__ unsigned cl_ok;
    const unsigned rank = cluster_ctarank();
    if (threadIdx.x == 0) {
#pragma unroll
      for (int k = 0; k < NV; k++) dsmem_st_f64(dsmem_addr(&cl_part[rank][k], 0), v[k]);
      __threadfence();  // this CTA's global writes, before the leader arrives
    }
    gb.epoch++;
    cluster_sync_all();
    if (rank == 0 && threadIdx.x < 32) {
      const int ncl = int(cluster_count_x());
      double* ps = part + size_t(slot) * 2 * gridDim.x;
      unsigned ok = 0;
      if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
          double c = 0.0;
          for (int r = 0; r < cl; r++) c += cl_part[r][k];
          ps[k * ncl + int(cluster_index_x())] = c;
        }
        ok = gb.arrive_wait(int(cluster_index_x())) ? 1u : 0u;
      }
      ok = __shfl_sync(0xffffffffu, ok, 0);
      if (ok) {
#pragma unroll
        for (int k = 0; k < NV; k++) {
          double acc = 0.0;
#pragma unroll 8
          for (int i = threadIdx.x; i < ncl; i += 32) acc += __ldcg(ps + k * ncl + i);
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
          if (threadIdx.x == 0) cl_tot[k] = acc;
        }
      }
      if (threadIdx.x == 0) cl_ok = ok;
    }
    cluster_sync_all();
    __shared__ double rs[NV];
    __shared__ unsigned my_ok;
    if (threadIdx.x == 0) {
      my_ok = dsmem_ld_u32(dsmem_addr(&cl_ok, 0));
#pragma unroll
      for (int k = 0; k < NV; k++) rs[k] = dsmem_ld_f64(dsmem_addr(&cl_tot[k], 0));
      if (my_ok) fin(rs);
    }
    cluster_sync_all();  // the leader's results are read before they may change or the leader may leave
    if (my_ok == 0) return false;
#pragma unroll
    for (int k = 0; k < NV; k++) v[k] = rs[k];
    return true;
  }
  template <int NV, bool WARP_DONE = false, class Fin = NoFin>
  __device__ bool sum(int slot, double (&v)[NV], const Fin& fin = Fin{}) {
    block_sum_t0<NV, WARP_DONE>(v);
    if (cl > 1) return sum_cluster<NV>(slot, v, fin);
    const int G = gridDim.x;
    double* ps = part + size_t(slot) * 2 * G;
    if (threadIdx.x == 0)
#pragma unroll
      for (int k = 0; k < NV; k++) ps[k * G + blockIdx.x] = v[k];
    if (!gb.sync()) return false;
    __shared__ double rs[NV];
    if (threadIdx.x < 32) {
#pragma unroll
      for (int k = 0; k < NV; k++) {
        // independent loads, then a fixed-order sum
        double acc = 0.0;
#pragma unroll 8
        for (int i = threadIdx.x; i < G; i += 32) acc += __ldcg(ps + k * G + i);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) rs[k] = acc;
      }
      if (threadIdx.x == 0) fin(rs);
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; k++) v[k] = rs[k];
    return true;
  }
  template <class Fin = NoFin>
  __device__ bool sum2(int slot, double& a, double& b, const Fin& fin = Fin{}) {
    double v[2] = {a, b};
    if (!sum<2>(slot, v, fin)) return false;
    a = v[0];
    b = v[1];
    return true;
  }
  template <class Fin = NoFin>
  __device__ bool sum1(int slot, double& a, const Fin& fin = Fin{}) {
    double v[1] = {a};
    if (!sum<1>(slot, v, fin)) return false;
    a = v[0];
    return true;
  }
  // An FP32 per-thread partial: summed across the warp in FP32 (FP64 issue
  // is 1/64 of FP32 here), then across warps and CTAs in FP64.
  template <class Fin = NoFin>
  __device__ bool sum1f(int slot, float a, double& out, const Fin& fin = Fin{}) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    double v[1] = {double(a)};
    if (!sum<1, true>(slot, v, fin)) return false;
    out = v[0];
    return true;
  }
};

// ---------------------------------------------------------------------------
// Row loops: each thread takes kU rows per pass (rows i, i+nt, ..., so warps
// stay coalesced) and issues all of their loads before any use.
constexpr int kU = 4;
#define CG_ROWS(i, BODY)                                                   \
  for (int base_ = row0 + tid; base_ < row1; base_ += nt * kU) {           \
    _Pragma("unroll") for (int u_ = 0; u_ < kU; u_++) {                    \
      const int i = base_ + u_ * nt;                                       \
      if (i < row1) { BODY }                                               \
    }                                                                      \
  }

// Streaming row loops: 4 consecutive rows per thread with 16-byte vector
// accesses over the 4-aligned part of [row0, row1), the ragged ends (and
// everything when `vec` is false, e.g. a caller's vector that is not 16-byte
// aligned) one row per thread.
template <class F4, class F1>
__device__ __forceinline__ void cg_rows4(int row0, int row1, bool vec, F4&& f4, F1&& f1) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int a0 = vec ? min(row1, (row0 + 3) & ~3) : row1;
  const int a1 = vec ? max(a0, row1 & ~3) : row1;
#pragma unroll 2
  for (int i = a0 + 4 * tid; i < a1; i += 4 * nt) f4(i);
  for (int i = row0 + tid; i < a0; i += nt) f1(i);
  for (int i = a1 + tid; i < row1; i += nt) f1(i);
}
// CSR rows by groups of G = A.grp lanes: lane l of a group takes entries
// j0+l, j0+l+G, ... of its row, so a group reads the row's columns and values
// as one contiguous run. Each group works on R rows per pass and steps through
// their entries together, so up to R gathers per lane are in flight (the
// dependent row pointer -> column -> x loads would otherwise leave the memory
// system idle). The group adds its partial sums by shuffles and its first
// lane runs epi(i, row sum). Every lane of the CTA runs the same number of
// passes (the shuffles need whole warps).
template <class XV, class MV, class XF, class Epi>
__device__ __forceinline__ void csr_rows_grouped(const CgMat& A, const MV* __restrict__ val, int row0, int row1,
                                                 const XF& xv, Epi&& epi) {
  constexpr int R = 4;  // rows per group and pass (the reduction below is written for 4)
  const int G = A.grp;
  const int gl = threadIdx.x & (G - 1);
  const int g = threadIdx.x / G, ng = blockDim.x / G;
  for (int i0 = row0; i0 < row1; i0 += R * ng) {
    int j[R], j1[R];
    XV acc[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
      const int i = i0 + g + r * ng;
      acc[r] = XV(0);
      j[r] = 0;
      j1[r] = 0;
      if (i < row1) {
        j[r] = __ldg(A.rp + i) + gl;
        j1[r] = __ldg(A.rp + i + 1);
      }
    }
    for (bool more = true; more;) {
      more = false;
#pragma unroll
      for (int r = 0; r < R; r++) {
        if (j[r] < j1[r]) {
          acc[r] = fma(XV(__ldg(val + j[r])), xv(__ldg(A.ci + j[r])), acc[r]);
          j[r] += G;
          more |= j[r] < j1[r];
        }
      }
    }
    // Transposing reduction of the four row sums over the group (G >= 4):
    // the first two exchanges halve the values a lane holds, so a lane adds
    // 2 + 1 + log2(G/4) values instead of 4 log2(G) (FP64 adds are scarce on
    // this GPU). Afterwards lane gl < 4 holds the sum of row 2(gl&1) + (gl>>1).
    constexpr unsigned kFull = 0xffffffffu;
    const bool b0 = gl & 1, b1 = gl & 2;
    const XV s0 = __shfl_xor_sync(kFull, b0 ? acc[0] : acc[2], 1);
    const XV s1 = __shfl_xor_sync(kFull, b0 ? acc[1] : acc[3], 1);
    const XV p0 = (b0 ? acc[2] : acc[0]) + s0;  // row 0 (or 2)
    const XV p1 = (b0 ? acc[3] : acc[1]) + s1;  // row 1 (or 3)
    XV t = (b1 ? p1 : p0) + __shfl_xor_sync(kFull, b1 ? p0 : p1, 2);
    for (int o = 4; o < G; o <<= 1) t += __shfl_xor_sync(kFull, t, o);
    const int i = i0 + g + (2 * (gl & 1) + (gl >> 1)) * ng;
    if (gl < 4 && i < row1) epi(i, t);
  }
}

// SpMV phase rows: DIA and ELL in groups of four rows per thread (f4; the
// ragged ends row by row), CSR by lane groups, SELL by slices (the CTA's
// slice range sr; rows in slot order). e1(i, row sum) finishes a row.
template <int FMT, class XV, class MV, class XF, class F4, class E1>
__device__ __forceinline__ void cg_rows_spmv(const CgMat& A, const MV* __restrict__ val, const XF& xv, int row0,
                                             int row1, int2 sr, F4&& f4, E1&& e1) {
  static_assert(FMT >= 0, "format fixed at compile time");
  if constexpr (FMT == 3)
    sell_rows<XV>(A, val, sr.x, sr.y, xv, e1);
  else if constexpr (FMT == 0)
    csr_rows_grouped<XV>(A, val, row0, row1, xv, e1);
  else
    cg_rows4(row0, row1, true, f4, [&](int i) { e1(i, spmv_row_f<XV, FMT>(A, val, xv, i)); });
}
// The CTA's SELL slice range (unused for other formats).
template <int FMT>
__device__ __forceinline__ int2 cta_slices(const CgMat& A) {
  if constexpr (FMT == 3) return make_int2(sell_split(A, blockIdx.x, gridDim.x), sell_split(A, blockIdx.x + 1, gridDim.x));
  else return make_int2(0, 0);
}
__device__ __forceinline__ void ld4(const float* p, float (&v)[4]) {
  const float4 t = *reinterpret_cast<const float4*>(p);
  v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
}
__device__ __forceinline__ void ld4(const double* p, double (&v)[4]) {
  const double2 a = reinterpret_cast<const double2*>(p)[0], b = reinterpret_cast<const double2*>(p)[1];
  v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}
__device__ __forceinline__ void st4(float* p, const float (&v)[4]) {
  *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void st4(double* p, const double (&v)[4]) {
  reinterpret_cast<double2*>(p)[0] = make_double2(v[0], v[1]);
  reinterpret_cast<double2*>(p)[1] = make_double2(v[2], v[3]);
}
__device__ __forceinline__ bool aligned16(const void* a) { return (reinterpret_cast<uintptr_t>(a) & 15) == 0; }

// Rows i..i+3 of A times the vector xv(column), each row in the same order as
// spmv_row_f. DIA runs diagonal-major over the four rows: one 16-byte load of
// the diagonal's values (when every diagonal starts 16-byte aligned) and four
// independent gathers per diagonal, so a thread keeps many loads in flight.
template <class XV, int FMT = -1, class MV, class XF>
__device__ __forceinline__ void spmv4(const CgMat& A, const MV* __restrict__ val, bool v4, const XF& xv, int i,
                                      XV (&acc)[4]) {
  const int fmt = FMT >= 0 ? FMT : A.fmt;
  if (fmt == 0) {
#pragma unroll
    for (int u = 0; u < 4; u++) acc[u] = spmv_row_f<XV, FMT>(A, val, xv, i + u);
  } else if (fmt == 2) {
#pragma unroll
    for (int u = 0; u < 4; u++) acc[u] = XV(0);
#pragma unroll 2
    for (int k = 0; k < A.ew; k++) {
      const size_t e = (size_t)k * A.n + i;
      MV a[4];
      int c[4];
      if (v4) {
        ld4(val + e, a);
        const int4 t = *reinterpret_cast<const int4*>(A.eci + e);
        c[0] = t.x; c[1] = t.y; c[2] = t.z; c[3] = t.w;
      } else {
#pragma unroll
        for (int u = 0; u < 4; u++) {
          a[u] = val[e + u];
          c[u] = A.eci[e + u];
        }
      }
#pragma unroll
      for (int u = 0; u < 4; u++) acc[u] = fma(XV(a[u]), xv(c[u]), acc[u]);
    }
  } else {
#pragma unroll
    for (int u = 0; u < 4; u++) acc[u] = XV(0);
#pragma unroll 2
    for (int k = 0; k < A.ndiag; k++) {
      const MV* vk = val + (size_t)k * A.n + i;
      MV a[4];
      if (v4) {
        ld4(vk, a);
      } else {
#pragma unroll
        for (int u = 0; u < 4; u++) a[u] = vk[u];
      }
      const int c = i + A.off[k];
#pragma unroll
      for (int u = 0; u < 4; u++)
        if (c + u >= 0 && c + u < A.n) acc[u] = fma(XV(a[u]), xv(c + u), acc[u]);
    }
  }
}

// A vector of which this CTA keeps rows [base, cut) in shared memory for the
// whole solve, the rest (and every row of other CTAs) in global memory
// (PERKS: the CTA's share of the domain stays on chip across iterations and
// only the remainder streams). base = row0 rounded down to 4 and cut - base is
// a multiple of 4, so a four-row group is entirely on one side and 16-byte
// aligned there. at() checks both ends: a SELL SpMV writes rows of other
// CTAs, below base as well as above cut.
template <class T>
struct RowVec {
  T* g;
  T* s;
  int base, cut;
  __device__ __forceinline__ T* at(int i) const {
    return unsigned(i - base) < unsigned(cut - base) ? s + (i - base) : g + i;
  }
  // global -> shared (rows [lo, hi) of the CTA), or back
  __device__ __forceinline__ void load(int lo, int hi) const {
    for (int i = lo + threadIdx.x; i < min(hi, cut); i += blockDim.x) s[i - base] = g[i];
  }
  __device__ __forceinline__ void store(int lo, int hi) const {
    for (int i = lo + threadIdx.x; i < min(hi, cut); i += blockDim.x) g[i] = s[i - base];
  }
};
// Shared-memory rows of the resident vectors, in the order of `caps` (rows,
// multiples of 4; 0 = not resident). Dynamic shared memory of the CG kernels.
extern __shared__ __align__(16) unsigned char cg_smem[];
template <class T>
__device__ __forceinline__ RowVec<T> row_vec(T* g, int cap, int row0, int row1, int& off) {
  const int base = row0 & ~3;
  const int span = (row1 - base + 3) & ~3;
  RowVec<T> v{g, reinterpret_cast<T*>(cg_smem) + off, base, base + min(cap, max(span, 0))};
  off += cap;
  return v;
}

// Plain CG in one precision T (double, or float with the reference's float
// build rounding of the scalars r.r, p.Ap, alpha and beta). Vectors that
// only the owning CTA touches (r unless the SpMV gathers it, x, Ap) keep the
// CTA's rows in shared memory as far as P.cap_* allow.
template <class T, int FMT>
__global__ void __launch_bounds__(kCgThreads, 1) cg_persistent(const __grid_constant__ CgParams P) {
  // FP32 forms p where the SpMV gathers it, except for CSR/SELL: there the
  // random gathers dominate, and gathering p_old and r instead of p doubles
  // them. Then r is gathered and stays in global memory.
  constexpr bool FUSE = sizeof(T) == 4 && FMT != 0 && FMT != 3;
  const CgMat& A = P.A;
  const T* __restrict__ val = static_cast<const T*>(A.val);
  const T* __restrict__ b = static_cast<const T*>(P.b);
  T* __restrict__ r = static_cast<T*>(P.r);  // global r (gathered when FUSE)
  const int G = gridDim.x;
  const int row0 = cg_split(A, blockIdx.x, G), row1 = cg_split(A, blockIdx.x + 1, G);
  const int2 sr = cta_slices<FMT>(A);
  GridSum gs{P.part, GridBarrier{P.bar, P.status, unsigned(P.cluster > 1 ? G / P.cluster : G), P.ctl}, P.cluster};
  const int tid = threadIdx.x, nt = blockDim.x;
  const bool xvec = aligned16(P.x);  // the caller's solution vector
  const bool v4 = A.fmt != 0 && (A.n & 3) == 0 && aligned16(val) && aligned16(A.eci);  // DIA/ELL columns 16-byte aligned
  int off = 0;
  // SELL: the SpMV writes rows of other CTAs (r at the start, Ap): global
  const RowVec<T> R = row_vec<T>(r, (FUSE || FMT == 3) ? 0 : P.cap_r, row0, row1, off);
  const RowVec<T> X = row_vec<T>(static_cast<T*>(P.x), P.cap_x, row0, row1, off);
  const RowVec<T> AP = row_vec<T>(static_cast<T*>(P.Ap), FMT == 3 ? 0 : P.cap_ap, row0, row1, off);
  X.load(row0, row1);

  T r1, r0;
  double bb;
  int k;
  // alpha and beta, divided once per CTA by thread 0 in the finishing step of
  // the reduction that produces their denominator or numerator
  __shared__ T s_alpha, s_beta;
  if (P.resume) {  // r and the last p were restored by the host
    R.load(row0, row1);
    r1 = T(P.rr0);
    r0 = T(P.rrp0);
    if (tid == 0) s_beta = r1 / r0;
    __syncthreads();
    bb = P.bb0;
    k = P.k0 + 1;
  } else {
    __syncthreads();  // x in shared memory
    // r = b - A x ; rr = r.r ; bb = b.b  (per-thread sums in T, then double)
    T rr_t = T(0), bb_t = T(0);
    auto init_row = [&](int i, T ax) {
      const T bi = b[i];
      const T ri = T(-1) * ax + bi;
      *R.at(i) = ri;
      rr_t = fma(ri, ri, rr_t);
      bb_t = fma(bi, bi, bb_t);
    };
    const T* __restrict__ xg = static_cast<const T*>(P.x);  // gathered: the global copy (x0)
    if constexpr (FMT == 3) {
      sell_rows<T>(A, val, sr.x, sr.y, [xg](int c) { return xg[c]; }, init_row);
    } else {
      CG_ROWS(i, { init_row(i, spmv_row<FMT>(A, val, xg, i)); })
    }
    double rr = double(rr_t);
    bb = double(bb_t);
    if (!gs.sum2(0, rr, bb)) return;
    r1 = T(rr);  // float build: r.r rounded to float (cg_cpu.cpp:52)
    r0 = T(0);
    k = 1;
  }
  const double tol2 = (P.stop == PERKS_STOP_REL) ? P.tol * P.tol * bb : P.tol * P.tol;
  const T tol2t = T(P.tol) * T(P.tol);
  while (true) {
    if (!P.static_iter) {
      const bool done = (P.stop == PERKS_STOP_REL) ? (double(r1) < tol2) : (r1 < tol2t);
      if (done) break;
    }
    if (k > P.max_iter) break;
    T* __restrict__ p = static_cast<T*>(P.p[FUSE ? (k & 1) : 0]);
    T pap_t = T(0);
    if constexpr (FUSE) {
      // p = r (first) or beta p_old + r, formed where it is gathered
      if (k > 1) {
        const T beta = s_beta;
        const T* __restrict__ po = static_cast<const T*>(P.p[(k + 1) & 1]);
        auto pg = [&](int c) { return fma(beta, po[c], r[c]); };
        cg_rows_spmv<FMT, T>(A, val, pg, row0, row1, sr, [&](int i) {
          T av[4], pov[4], rv[4], pv[4];
          spmv4<T, FMT>(A, val, v4, pg, i, av);
          ld4(po + i, pov);
          ld4(r + i, rv);
#pragma unroll
          for (int u = 0; u < 4; u++) {
            pv[u] = fma(beta, pov[u], rv[u]);
            pap_t = fma(pv[u], av[u], pap_t);
          }
          st4(p + i, pv);
          st4(AP.at(i), av);
        }, [&](int i, T api) {
          const T pi = fma(beta, po[i], r[i]);
          p[i] = pi;
          *AP.at(i) = api;
          pap_t = fma(pi, api, pap_t);
        });
      } else {
        auto rg = [&](int c) { return r[c]; };
        cg_rows_spmv<FMT, T>(A, val, rg, row0, row1, sr, [&](int i) {
          T av[4], rv[4];
          spmv4<T, FMT>(A, val, v4, rg, i, av);
          ld4(r + i, rv);
#pragma unroll
          for (int u = 0; u < 4; u++) pap_t = fma(rv[u], av[u], pap_t);
          st4(p + i, rv);
          st4(AP.at(i), av);
        }, [&](int i, T api) {
          const T pi = r[i];
          p[i] = pi;
          *AP.at(i) = api;
          pap_t = fma(pi, api, pap_t);
        });
      }
    } else {
      if (k > 1) {
        const T beta = s_beta;
        cg_rows4(row0, row1, true, [&](int i) {
          T pv[4], rv[4];
          ld4(p + i, pv);
          ld4(R.at(i), rv);
#pragma unroll
          for (int u = 0; u < 4; u++) pv[u] = fma(beta, pv[u], rv[u]);
          st4(p + i, pv);
        }, [&](int i) { p[i] = fma(beta, p[i], *R.at(i)); });
      } else {
        cg_rows4(row0, row1, true, [&](int i) {
          T rv[4];
          ld4(R.at(i), rv);
          st4(p + i, rv);
        }, [&](int i) { p[i] = *R.at(i); });
      }
      if (!gs.bar()) return;
      auto pg = [&](int c) { return p[c]; };
      cg_rows_spmv<FMT, T>(A, val, pg, row0, row1, sr, [&](int i) {
        T av[4], pv[4];
        spmv4<T, FMT>(A, val, v4, pg, i, av);
        ld4(p + i, pv);
#pragma unroll
        for (int u = 0; u < 4; u++) pap_t = fma(pv[u], av[u], pap_t);
        st4(AP.at(i), av);
      }, [&](int i, T api) {
        *AP.at(i) = api;
        pap_t = fma(p[i], api, pap_t);
      });
    }
    double pap;
    T* const sa = &s_alpha;
    auto fin_alpha = [r1, sa](const double* t) { *sa = r1 / T(t[0]); };
    if constexpr (FUSE) {
      if (!gs.sum1f(1 + (k & 1), float(pap_t), pap, fin_alpha)) return;
    } else {
      pap = double(pap_t);
      if (!gs.sum1(1 + (k & 1), pap, fin_alpha)) return;
    }
    const T dot = T(pap);
    if (!(dot > T(0)) || !isfinite(double(dot))) {
      if (tid == 0 && blockIdx.x == 0) atomicOr(P.status, kErrBreakdown);
      return;
    }
    const T alpha = s_alpha;
    T rrn_t = T(0);
    cg_rows4(row0, row1, xvec, [&](int i) {
      T xv[4], pv[4], av[4], rv[4];
      T* const xi = X.at(i);
      T* const ri = R.at(i);
      ld4(xi, xv);
      ld4(p + i, pv);
      ld4(AP.at(i), av);
      ld4(ri, rv);
#pragma unroll
      for (int u = 0; u < 4; u++) {
        xv[u] = fma(alpha, pv[u], xv[u]);
        rv[u] = fma(-alpha, av[u], rv[u]);
        rrn_t = fma(rv[u], rv[u], rrn_t);
      }
      st4(xi, xv);
      st4(ri, rv);
    }, [&](int i) {
      T* const xi = X.at(i);
      *xi = fma(alpha, p[i], *xi);
      T* const rp = R.at(i);
      const T rn = fma(-alpha, *AP.at(i), *rp);
      *rp = rn;
      rrn_t = fma(rn, rn, rrn_t);
    });
    double rrn;
    T* const sb = &s_beta;
    auto fin_beta = [r1, sb](const double* t) { *sb = T(t[0]) / r1; };  // the next iteration's r1 / r0
    if constexpr (FUSE) {
      if (!gs.sum1f(3, float(rrn_t), rrn, fin_beta)) return;
    } else {
      rrn = double(rrn_t);
      if (!gs.sum1(3, rrn, fin_beta)) return;
    }
    r0 = r1;
    r1 = T(rrn);
    k++;
  }
  // the resident rows back to global memory: x (the caller's solution) and r
  // (read by a checkpoint)
  X.store(row0, row1);
  R.store(row0, row1);
  if (blockIdx.x == 0 && tid == 0) {
    *P.out_iter = k - 1;
    P.out_rr[0] = double(r1);
    P.out_rr[1] = double(r0);
    P.out_rr[2] = bb;
    *P.out_outer = 0;
  }
}

// ---------------------------------------------------------------------------
// Single-reduction CG (Chronopoulos & Gear, "s-step iterative methods for
// symmetric linear systems", J. Comput. Appl. Math. 25, 1989): the same
// iterates as plain CG in exact arithmetic, with s = A p and w = A r carried
// by recurrences, so one iteration needs one row pass, one grid barrier and
// one reduction of two dot products instead of two passes, a barrier and
// two reductions:
//   p = r + beta p;  s = w + beta s;  x += alpha p;  r -= alpha s   (rows)
//   -- barrier --
//   w = A r;  gamma = r.r;  delta = w.r                              (SpMV)
//   -- reduction --
//   beta' = gamma / gamma_old;  alpha' = gamma / (delta - beta' gamma / alpha)
// Rounding differs from plain CG: r is updated with the recurred s instead of
// A p, and alpha comes from delta = (A r).r. The stop test is plain CG's, on
// gamma = r.r. FP64 or FP32 (scalars formed in FP64, rounded to T). p, s and
// x are touched only by their owning CTA and keep rows in shared memory as far
// as P.cap_* allow (cap_r: p, cap_x: x, cap_ap: s); r is gathered by the
// SpMV and w (SELL) written by other CTAs, so both stay in global memory.
template <class T, int FMT>
__global__ void __launch_bounds__(kCgThreads, 1) cg_single_red(const __grid_constant__ CgParams P) {
  const CgMat& A = P.A;
  const T* __restrict__ val = static_cast<const T*>(A.val);
  const T* __restrict__ b = static_cast<const T*>(P.b);
  T* __restrict__ r = static_cast<T*>(P.r);
  T* __restrict__ w = static_cast<T*>(P.p[1]);  // w = A r
  const int G = gridDim.x;
  const int row0 = cg_split(A, blockIdx.x, G), row1 = cg_split(A, blockIdx.x + 1, G);
  const int2 sr = cta_slices<FMT>(A);
  GridSum gs{P.part, GridBarrier{P.bar, P.status, unsigned(P.cluster > 1 ? G / P.cluster : G), P.ctl}, P.cluster};
  const int tid = threadIdx.x, nt = blockDim.x;
  const bool xvec = aligned16(P.x);
  const bool v4 = A.fmt != 0 && (A.n & 3) == 0 && aligned16(val) && aligned16(A.eci);
  int off = 0;
  const RowVec<T> PV = row_vec<T>(static_cast<T*>(P.p[0]), P.cap_r, row0, row1, off);
  const RowVec<T> X = row_vec<T>(static_cast<T*>(P.x), P.cap_x, row0, row1, off);
  const RowVec<T> S = row_vec<T>(static_cast<T*>(P.Ap), P.cap_ap, row0, row1, off);
  X.load(row0, row1);
  __syncthreads();

  // r = b - A x, r.r, b.b
  T rr_t = T(0), bb_t = T(0);
  {
    const T* __restrict__ xg = static_cast<const T*>(P.x);
    auto init_row = [&](int i, T ax) {
      const T bi = b[i];
      const T ri = T(-1) * ax + bi;
      r[i] = ri;
      rr_t = fma(ri, ri, rr_t);
      bb_t = fma(bi, bi, bb_t);
    };
    if constexpr (FMT == 3) {
      sell_rows<T>(A, val, sr.x, sr.y, [xg](int c) { return xg[c]; }, init_row);
    } else {
      CG_ROWS(i, { init_row(i, spmv_row<FMT>(A, val, xg, i)); })
    }
  }
  double gamma = double(rr_t), bb = double(bb_t);
  if (!gs.sum2(0, gamma, bb)) return;
  // w = A r, delta = w.r (the rows of r this CTA's SpMV produces)
  auto spmv_w = [&](T& g_t, T& d_t) {
    auto rg = [&](int c) { return r[c]; };
    cg_rows_spmv<FMT, T>(A, val, rg, row0, row1, sr, [&](int i) {
      T wv[4], rv[4];
      spmv4<T, FMT>(A, val, v4, rg, i, wv);
      ld4(r + i, rv);
#pragma unroll
      for (int u = 0; u < 4; u++) {
        g_t = fma(rv[u], rv[u], g_t);
        d_t = fma(wv[u], rv[u], d_t);
      }
      st4(w + i, wv);
    }, [&](int i, T wi) {
      const T ri = r[i];
      w[i] = wi;
      g_t = fma(ri, ri, g_t);
      d_t = fma(wi, ri, d_t);
    });
  };
  T g0 = T(0), d0 = T(0);
  spmv_w(g0, d0);
  double delta = double(d0), unused = double(g0);
  if (!gs.sum2(1, delta, unused)) return;
  const double tol2 = (P.stop == PERKS_STOP_REL) ? P.tol * P.tol * bb : P.tol * P.tol;
  if (!(delta > 0.0) || !isfinite(delta)) {
    if (!(gamma < tol2)) {  // a zero residual needs no step
      if (tid == 0 && blockIdx.x == 0) atomicOr(P.status, kErrBreakdown);
      return;
    }
  }
  double alpha = gamma / delta, beta = 0.0, gamma_old = gamma;
  int k = 1;
  while (true) {
    if (!P.static_iter && gamma < tol2) break;
    if (k > P.max_iter) break;
    const T a = T(alpha), be = T(beta);
    const bool first = k == 1;
    cg_rows4(row0, row1, xvec, [&](int i) {
      T pv[4], sv[4], xv[4], rv[4], wv[4];
      T* const pi = PV.at(i);
      T* const si = S.at(i);
      T* const xi = X.at(i);
      ld4(r + i, rv);
      ld4(w + i, wv);
      ld4(xi, xv);
      if (!first) {
        ld4(pi, pv);
        ld4(si, sv);
      }
#pragma unroll
      for (int u = 0; u < 4; u++) {
        pv[u] = first ? rv[u] : fma(be, pv[u], rv[u]);
        sv[u] = first ? wv[u] : fma(be, sv[u], wv[u]);
        xv[u] = fma(a, pv[u], xv[u]);
        rv[u] = fma(-a, sv[u], rv[u]);
      }
      st4(pi, pv);
      st4(si, sv);
      st4(xi, xv);
      st4(r + i, rv);
    }, [&](int i) {
      T* const pi = PV.at(i);
      T* const si = S.at(i);
      T* const xi = X.at(i);
      const T pn = first ? r[i] : fma(be, *pi, r[i]);
      const T sn = first ? w[i] : fma(be, *si, w[i]);
      *pi = pn;
      *si = sn;
      *xi = fma(a, pn, *xi);
      r[i] = fma(-a, sn, r[i]);
    });
    if (!gs.bar()) return;
    T g_t = T(0), d_t = T(0);
    spmv_w(g_t, d_t);
    double gn = double(g_t), dn = double(d_t);
    // beta, the denominator and alpha, divided once per CTA by thread 0
    __shared__ double s_q[3];
    double* const q = s_q;
    if (!gs.sum2(1 + (k & 1), gn, dn, [gamma_old, alpha, q](const double* t) {
          const double bq = t[0] / gamma_old;
          const double den_q = t[1] - bq * t[0] / alpha;
          q[0] = bq;
          q[1] = den_q;
          q[2] = t[0] / den_q;
        }))
      return;
    beta = s_q[0];
    const double den = s_q[1];
    gamma_old = gn;
    gamma = gn;
    k++;
    if (!P.static_iter && gamma < tol2) break;
    if (!(den > 0.0) || !isfinite(den)) {
      if (tid == 0 && blockIdx.x == 0) atomicOr(P.status, kErrBreakdown);
      return;
    }
    alpha = s_q[2];
  }
  X.store(row0, row1);
  if (blockIdx.x == 0 && tid == 0) {
    *P.out_iter = k - 1;
    P.out_rr[0] = gamma;
    P.out_rr[1] = 0.0;
    P.out_rr[2] = bb;
    *P.out_outer = 0;
  }
}

// ---------------------------------------------------------------------------
// Mixed precision: FP32 Krylov iteration, FP64 solution and true residual.
// Shared-memory residency as in cg_persistent: the FP32 r (unless the SpMV
// gathers it), the FP32 increment x_s and Ap keep the CTA's rows on chip.
template <int FMT, int FMT64>  // FMT64: the format of the FP64 matrix as given (CSR or DIA)
__global__ void __launch_bounds__(kCgThreads, 1) cg_mixed(const __grid_constant__ CgParams P) {
  constexpr bool FUSE = FMT != 0 && FMT != 3;  // p formed where the SpMV gathers it (r gathered)
  const CgMat& A = P.A;      // FP32 iteration (values in val32)
  const CgMat& A64 = P.A64;  // FP64 true residual
  const double* __restrict__ val64 = static_cast<const double*>(A64.val);
  float* __restrict__ val32 = P.val32;
  const double* __restrict__ b = static_cast<const double*>(P.b);
  double* __restrict__ x = static_cast<double*>(P.x);
  float* __restrict__ r = static_cast<float*>(P.r);  // global r (gathered when FUSE)
  const int G = gridDim.x;
  const int row0 = cg_split(A, blockIdx.x, G), row1 = cg_split(A, blockIdx.x + 1, G);
  const int2 sr = cta_slices<FMT>(A);
  GridSum gs{P.part, GridBarrier{P.bar, P.status, unsigned(P.cluster > 1 ? G / P.cluster : G), P.ctl}, P.cluster};
  const int tid = threadIdx.x, nt = blockDim.x;
  const bool v4 = A.fmt != 0 && (A.n & 3) == 0 && aligned16(A.eci);  // val32 (workspace) is aligned
  int off = 0;
  // SELL: the SpMV writes rows of other CTAs (Ap): global
  const RowVec<float> R = row_vec<float>(r, FUSE ? 0 : P.cap_r, row0, row1, off);
  const RowVec<float> XS = row_vec<float>(P.xs, P.cap_x, row0, row1, off);
  const RowVec<float> AP = row_vec<float>(static_cast<float*>(P.Ap), FMT == 3 ? 0 : P.cap_ap, row0, row1, off);

  // body(i, (A64 x)_i) for every row of this CTA: CSR by lane groups, else
  // one row per thread (rows split as for A: A64 has the same rows)
  auto true_rows = [&](auto&& body) {
    if constexpr (FMT64 == 0) {
      csr_rows_grouped<double>(A64, val64, row0, row1, [&](int c) { return x[c]; }, body);
    } else {
      CG_ROWS(i, { body(i, spmv_row<FMT64>(A64, val64, x, i)); })
    }
  };
  double rr, bb, maxrr, rr0;
  int k, outer, since;
  // alpha and beta, divided once per CTA by thread 0 in the finishing step of
  // the reduction that produces their denominator or numerator
  __shared__ float s_alpha, s_beta;
  if (P.resume) {  // r, x_s and the last p restored by the host
    R.load(row0, row1);
    XS.load(row0, row1);
    if (tid == 0) s_beta = float(P.rr0 / P.rrp0);
    __syncthreads();
    rr = P.rr0;
    rr0 = P.rrp0;
    bb = P.bb0;
    maxrr = P.maxrr0;
    k = P.k0 + 1;
    outer = P.outer0;
    since = P.since0;
  } else {
    // true residual in FP64
    rr = 0.0;
    bb = 0.0;
    true_rows([&](int i, double ax) {
      const double bi = b[i];
      const double ri = bi - ax;
      *R.at(i) = float(ri);
      *XS.at(i) = 0.0f;
      rr = fma(ri, ri, rr);
      bb = fma(bi, bi, bb);
    });
    if (!gs.sum2(0, rr, bb)) return;
    maxrr = rr;
    rr0 = 0.0;
    k = 1;
    outer = 0;
    since = 0;
  }
  const double tol2 = (P.stop == PERKS_STOP_REL) ? P.tol * P.tol * bb : P.tol * P.tol;
  while (true) {
    if (!P.static_iter && rr < tol2) break;
    if (k > P.max_iter) break;
    // p = r (first) or beta p_old + r; iteration k writes P.p[k & 1]
    float* __restrict__ p = static_cast<float*>(P.p[k & 1]);
    float pap_t = 0.0f;
    if constexpr (!FUSE) {
      // CSR / SELL: p in its own pass (same values as the fused form), so
      // that the SpMV gathers one vector instead of two
      const float beta = k > 1 ? s_beta : 0.0f;
      const float* __restrict__ po = static_cast<const float*>(P.p[(k + 1) & 1]);
      cg_rows4(row0, row1, true, [&](int i) {
        float pv[4], rv[4];
        ld4(R.at(i), rv);
        if (k > 1) {
          ld4(po + i, pv);
#pragma unroll
          for (int u = 0; u < 4; u++) pv[u] = fmaf(beta, pv[u], rv[u]);
        } else {
#pragma unroll
          for (int u = 0; u < 4; u++) pv[u] = rv[u];
        }
        st4(p + i, pv);
      }, [&](int i) { p[i] = k > 1 ? fmaf(beta, po[i], *R.at(i)) : *R.at(i); });
      if (!gs.bar()) return;
      auto pgat = [&](int c) { return p[c]; };
      cg_rows_spmv<FMT, float>(A, val32, pgat, row0, row1, sr, [&](int) {}, [&](int i, float api) {
        *AP.at(i) = api;
        pap_t = fmaf(p[i], api, pap_t);
      });
    } else if (k > 1) {
      // formed where it is gathered (the values its owner stores are the same fma)
      const float beta = s_beta;
      const float* __restrict__ po = static_cast<const float*>(P.p[(k + 1) & 1]);
      auto pg = [&](int c) { return fmaf(beta, po[c], r[c]); };
      cg_rows_spmv<FMT, float>(A, val32, pg, row0, row1, sr, [&](int i) {
        float av[4], pov[4], rv[4], pv[4];
        spmv4<float, FMT>(A, val32, v4, pg, i, av);
        ld4(po + i, pov);
        ld4(r + i, rv);
#pragma unroll
        for (int u = 0; u < 4; u++) {
          pv[u] = fmaf(beta, pov[u], rv[u]);
          pap_t = fmaf(pv[u], av[u], pap_t);
        }
        st4(p + i, pv);
        st4(AP.at(i), av);
      }, [&](int i, float api) {
        const float pi = fmaf(beta, po[i], r[i]);
        p[i] = pi;
        *AP.at(i) = api;
        pap_t = fmaf(pi, api, pap_t);
      });
    } else {
      auto rg = [&](int c) { return r[c]; };
      cg_rows_spmv<FMT, float>(A, val32, rg, row0, row1, sr, [&](int i) {
        float av[4], rv[4];
        spmv4<float, FMT>(A, val32, v4, rg, i, av);
        ld4(r + i, rv);
#pragma unroll
        for (int u = 0; u < 4; u++) pap_t = fmaf(rv[u], av[u], pap_t);
        st4(p + i, rv);
        st4(AP.at(i), av);
      }, [&](int i, float api) {
        const float pi = r[i];
        p[i] = pi;
        *AP.at(i) = api;
        pap_t = fmaf(pi, api, pap_t);
      });
    }
    double pap;
    float* const sa = &s_alpha;
    if (!gs.sum1f(1 + (k & 1), pap_t, pap, [rr, sa](const double* t) { *sa = float(rr / t[0]); })) return;
    if (!(pap > 0.0) || !isfinite(pap)) {
      if (tid == 0 && blockIdx.x == 0) atomicOr(P.status, kErrBreakdown);
      return;
    }
    const float alpha = s_alpha;
    float rrn_t = 0.0f;
    cg_rows4(row0, row1, true, [&](int i) {
      float xv[4], pv[4], av[4], rv[4];
      float* const xi = XS.at(i);
      float* const ri = R.at(i);
      ld4(xi, xv);
      ld4(p + i, pv);
      ld4(AP.at(i), av);
      ld4(ri, rv);
#pragma unroll
      for (int u = 0; u < 4; u++) {
        xv[u] = fmaf(alpha, pv[u], xv[u]);
        rv[u] = fmaf(-alpha, av[u], rv[u]);
        rrn_t = fmaf(rv[u], rv[u], rrn_t);
      }
      st4(xi, xv);
      st4(ri, rv);
    }, [&](int i) {
      float* const xi = XS.at(i);
      *xi = fmaf(alpha, p[i], *xi);
      float* const rp = R.at(i);
      const float rn = fmaf(-alpha, *AP.at(i), *rp);
      *rp = rn;
      rrn_t = fmaf(rn, rn, rrn_t);
    });
    double rrn;
    // the next iteration's rr / rr0 (replaced below after a reliable update)
    float* const sb = &s_beta;
    auto fin_beta = [rr, sb](const double* t) { *sb = float(t[0] / rr); };
    if (!gs.sum1f(3, rrn_t, rrn, fin_beta)) return;
    since++;
    // the last allowed iteration folds x_s into x, unless a checkpoint takes
    // the state (then x_s is saved with it and the resumed solve continues
    // exactly as an uninterrupted one)
    const bool update = rrn < P.delta2 * maxrr || rrn < tol2 || (P.replace_every > 0 && since >= P.replace_every) ||
                        (k == P.max_iter && !P.keep_state);
    if (update) {
      // x += xs in FP64; true residual with the FP64 matrix
      CG_ROWS(i, {
        float* const xi = XS.at(i);
        x[i] += double(*xi);
        *xi = 0.0f;
      })
      if (!gs.bar()) return;
      double rt = 0.0;
      true_rows([&](int i, double ax) {
        const double ri = b[i] - ax;
        *R.at(i) = float(ri);
        rt = fma(ri, ri, rt);
      });
      if (!gs.sum1(0, rt, fin_beta)) return;
      rrn = rt;
      maxrr = rt;
      outer++;
      since = 0;
    }
    rr0 = rr;
    rr = rrn;
    k++;
  }
  // resident rows back to global memory (read by a checkpoint)
  R.store(row0, row1);
  XS.store(row0, row1);
  if (blockIdx.x == 0 && tid == 0) {
    *P.out_iter = k - 1;
    P.out_rr[0] = rr;
    P.out_rr[1] = rr0;
    P.out_rr[2] = bb;
    P.out_rr[3] = maxrr;
    P.out_rr[4] = double(since);
    *P.out_outer = outer;
  }
}

// ---------------------------------------------------------------------------
// One-launch-per-phase comparator kernels (plain CG, FP64 or FP32). Scalars
// live on the device: s[0] = r1 (r.r), s[1] = r0, s[2] = p.Ap, s[3] = bb,
// s[4] = done flag, s[5] = iterations.
template <class T>
__global__ void cg_phase_init(const __grid_constant__ CgParams P, double* part) {
  const CgMat& A = P.A;
  const T* val = static_cast<const T*>(A.val);
  const T* b = static_cast<const T*>(P.b);
  const T* x = static_cast<const T*>(P.x);
  T* r = static_cast<T*>(P.r);
  double rr = 0.0, bb = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += gridDim.x * blockDim.x) {
    const T ri = T(-1) * T(spmv_row(A, val, x, i)) + b[i];
    r[i] = ri;
    rr += double(ri * ri);
    bb += double(b[i] * b[i]);
  }
  block_sum2(rr, bb);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = rr;
    part[gridDim.x + blockIdx.x] = bb;
  }
}

// Reduce the partials of the previous kernel into scalar slot `which`
// (0: r.r at init, 2: p.Ap, 1: new r.r) and update the iteration state.
template <class T>
__global__ void cg_phase_reduce(const __grid_constant__ CgParams P, double* part, int nparts, double* s, int which) {
  double a = 0.0, bsum = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
    a += part[i];
    bsum += part[nparts + i];
  }
  block_sum2(a, bsum);
  if (threadIdx.x != 0) return;
  if (which != 0 && s[4] != 0.0) return;  // converged or broken down: keep the final state
  if (which == 0) {
    s[0] = double(T(a));
    s[3] = bsum;
    s[5] = 0.0;
  } else if (which == 2) {
    s[2] = double(T(a));
    if (!(s[2] > 0.0)) {
      s[4] = 1.0;
      atomicOr(P.status, kErrBreakdown);
    }
  } else {
    s[1] = s[0];
    s[0] = double(T(a));
    s[5] += 1.0;
  }
  if (which != 2) {
    const double tol2 = (P.stop == PERKS_STOP_REL) ? P.tol * P.tol * s[3] : double(T(P.tol) * T(P.tol));
    if ((!P.static_iter && s[0] < tol2) || s[5] >= P.max_iter) s[4] = 1.0;
  }
}

template <class T>
__global__ void cg_phase_p(const __grid_constant__ CgParams P, const double* s) {
  if (s[4] != 0.0) return;
  T* p = static_cast<T*>(P.p[0]);
  const T* r = static_cast<const T*>(P.r);
  const bool first = s[5] == 0.0;
  const T beta = first ? T(0) : T(s[0]) / T(s[1]);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.A.n; i += gridDim.x * blockDim.x)
    p[i] = first ? r[i] : fma(beta, p[i], r[i]);
}

template <class T>
__global__ void cg_phase_spmv(const __grid_constant__ CgParams P, const double* s, double* part) {
  if (s[4] != 0.0) return;
  const T* val = static_cast<const T*>(P.A.val);
  const T* p = static_cast<const T*>(P.p[0]);
  T* Ap = static_cast<T*>(P.Ap);
  double pap = 0.0, u = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.A.n; i += gridDim.x * blockDim.x) {
    const T api = T(spmv_row(P.A, val, p, i));
    Ap[i] = api;
    pap += double(p[i] * api);
  }
  block_sum2(pap, u);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = pap;
    part[gridDim.x + blockIdx.x] = 0.0;
  }
}

template <class T>
__global__ void cg_phase_update(const __grid_constant__ CgParams P, const double* s, double* part) {
  if (s[4] != 0.0) return;
  T* x = static_cast<T*>(P.x);
  T* r = static_cast<T*>(P.r);
  const T* p = static_cast<const T*>(P.p[0]);
  const T* Ap = static_cast<const T*>(P.Ap);
  const T alpha = T(s[0]) / T(s[2]);
  double rr = 0.0, u = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P.A.n; i += gridDim.x * blockDim.x) {
    x[i] = fma(alpha, p[i], x[i]);
    const T ri = fma(-alpha, Ap[i], r[i]);
    r[i] = ri;
    rr += double(ri * ri);
  }
  block_sum2(rr, u);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = rr;
    part[gridDim.x + blockIdx.x] = 0.0;
  }
}

// True relative residual ||b - A x|| / ||b|| in FP64 (reported, not used for stopping).
template <class T>
__global__ void cg_true_residual(CgMat A, const void* bv, const void* xv, double* part) {
  const T* val = static_cast<const T*>(A.val);
  const T* b = static_cast<const T*>(bv);
  const T* x = static_cast<const T*>(xv);
  double rr = 0.0, bb = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += gridDim.x * blockDim.x) {
    double acc = 0.0;
    if (A.fmt == 0) {
      for (int j = A.rp[i]; j < A.rp[i + 1]; j++) acc = fma(double(val[j]), double(x[A.ci[j]]), acc);
    } else {
      for (int k = 0; k < A.ndiag; k++) {
        const int c = i + A.off[k];
        if (c >= 0 && c < A.n) acc = fma(double(val[(size_t)k * A.n + i]), double(x[c]), acc);
      }
    }
    const double ri = double(b[i]) - acc;
    rr += ri * ri;
    bb += double(b[i]) * double(b[i]);
  }
  block_sum2(rr, bb);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = rr;
    part[gridDim.x + blockIdx.x] = bb;
  }
}

__global__ void sum_partials(const double* part, int n, double* out) {
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    a += part[i];
    b += part[n + i];
  }
  block_sum2(a, b);
  if (threadIdx.x == 0) {
    out[0] = a;
    out[1] = b;
  }
}

template <class T>
__global__ void spmv_kernel(CgMat A, const T* x, T* y) {
  const T* val = static_cast<const T*>(A.val);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += gridDim.x * blockDim.x)
    y[i] = T(spmv_row(A, val, x, i));
}

// Longest CSR row (setup for the ELL choice).
__global__ void csr_max_row(const int* rp, int n, int* out) {
  int m = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) m = max(m, rp[i + 1] - rp[i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}
// CSR -> column-major ELL with ew entries per row, values converted to DV.
template <class SV, class DV>
__global__ void ell_build(const int* rp, const int* ci, const SV* val, int n, int ew, int* eci, DV* ev) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int j0 = rp[i], len = rp[i + 1] - j0;
    for (int k = 0; k < ew; k++) {
      const size_t e = (size_t)k * n + i;
      eci[e] = k < len ? ci[j0 + k] : i;
      ev[e] = k < len ? DV(val[j0 + k]) : DV(0);
    }
  }
}
// Distinct diagonal offsets of a CSR matrix into a 64-slot open-addressing
// table (kEmpty = unused); flags[0]: more than 64 distinct, flags[1]: a row
// whose columns are not strictly increasing.
constexpr int kEmpty = 0x7fffffff;
__global__ void csr_diag_scan(const int* rp, const int* ci, int n, int* tab, int* flags) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (*((volatile int*)flags)) return;  // table full: not a DIA matrix, stop scanning
    const int j0 = rp[i], j1 = rp[i + 1];
    int prev = -1;
    for (int j = j0; j < j1; j++) {
      const int c = ci[j];
      if (c <= prev) flags[1] = 1;
      prev = c;
      const int d = c - i;
      int h = (d * 40503) & 63, probes = 0;
      for (; probes < 64; probes++, h = (h + 1) & 63) {
        const int t = *((volatile int*)(tab + h));
        if (t == d) break;
        if (t == kEmpty) {
          const int old = atomicCAS(tab + h, kEmpty, d);
          if (old == kEmpty || old == d) break;
        }
      }
      if (probes == 64) {
        flags[0] = 1;
        return;
      }
    }
  }
}
// CSR -> DIA (data zeroed beforehand), values converted to DV.
template <class SV, class DV>
__global__ void dia_build(CgMat D, const int* rp, const int* ci, const SV* val, DV* data) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < D.n; i += gridDim.x * blockDim.x) {
    int k = 0;
    for (int j = rp[i]; j < rp[i + 1]; j++) {
      const int d = ci[j] - i;
      while (k < D.ndiag - 1 && D.off[k] != d) k++;  // columns ascend, so diagonals do too
      data[(size_t)k * D.n + i] = DV(val[j]);
    }
  }
}
// SELL setup (kSellWindow threads per window of rows): sort the window's rows
// by length, longest first, ties by row (a bitonic sort of 64-bit keys in
// shared memory); write each slot's row (n for the slots after the last row)
// and each slice's width, the length of its first, longest row.
__global__ void __launch_bounds__(kSellWindow) sell_sort(const int* rp, int n, int* sl_row, int* width) {
  __shared__ unsigned long long key[kSellWindow];
  const int t = threadIdx.x, base = blockIdx.x * kSellWindow;
  const int len = base + t < n ? rp[base + t + 1] - rp[base + t] : -1;
  const unsigned inv = len < 0 ? 0xffffffffu : 0x7fffffffu - unsigned(len);  // ascending = longest first
  key[t] = (static_cast<unsigned long long>(inv) << 32) | unsigned(t);
  __syncthreads();
  for (int k = 2; k <= kSellWindow; k <<= 1) {
    for (int j = k >> 1; j > 0; j >>= 1) {
      const int o = t ^ j;
      if (o > t) {
        const unsigned long long a = key[t], b = key[o];
        if ((a > b) == ((t & k) == 0)) {
          key[t] = b;
          key[o] = a;
        }
      }
      __syncthreads();
    }
  }
  const int row = base + int(key[t] & 0xffffffffu);
  const bool real = row < n;
  sl_row[base + t] = real ? row : n;
  if ((t & 31) == 0) width[blockIdx.x * (kSellWindow / 32) + (t >> 5)] = real ? rp[row + 1] - rp[row] : 0;
}
// sl_ptr[s] = 32 * (width[0] + ... + width[s-1]) for s <= ns; *total = the
// sum in 64 bits (the caller rejects layouts past int32). One CTA.
__global__ void __launch_bounds__(1024) sell_scan(const int* width, int ns, int* sl_ptr, long long* total) {
  __shared__ long long sh[1024];
  const int t = threadIdx.x, per = (ns + 1023) / 1024;
  const int a = min(ns, t * per), b = min(ns, a + per);
  long long s = 0;
  for (int i = a; i < b; i++) s += 32ll * width[i];
  sh[t] = s;
  __syncthreads();
  for (int d = 1; d < 1024; d <<= 1) {  // inclusive scan (Hillis-Steele)
    const long long v = t >= d ? sh[t - d] : 0;
    __syncthreads();
    sh[t] += v;
    __syncthreads();
  }
  long long off = sh[t] - s;
  for (int i = a; i < b; i++) {
    sl_ptr[i] = int(min(off, 0x7fffffffll));
    off += 32ll * width[i];
  }
  if (t == 1023) {
    sl_ptr[ns] = int(min(sh[1023], 0x7fffffffll));
    *total = sh[1023];
  }
}
// SELL entries from CSR, one warp per slice: entry k of slot l at
// sl_ptr[s] + 32 k + l; short rows padded with their own column and 0.
template <class SV, class DV>
__global__ void sell_fill(CgMat S, const int* rp, const int* ci, const SV* val, int* eci, DV* ev) {
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < S.nslices; s += nwarps) {
    const int e0 = S.sl_ptr[s], w = (S.sl_ptr[s + 1] - e0) >> 5;
    const int row = S.sl_row[s * 32 + lane];
    const bool real = row < S.n;
    const int j0 = real ? rp[row] : 0, len = real ? rp[row + 1] - j0 : 0;
    for (int k = 0; k < w; k++) {
      const int e = e0 + 32 * k + lane;
      eci[e] = k < len ? ci[j0 + k] : (real ? row : 0);
      ev[e] = k < len ? DV(val[j0 + k]) : DV(0);
    }
  }
}

__global__ void to_f32(const double* src, size_t n, float* dst) {
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    dst[i] = float(src[i]);
}

// ---------------------------------------------------------------------------
// Host side
static int cg_solve(CgMat A, const void* b, void* x, const perks_cg_opts* o, perks_cg_result* res) {
  if (!o) return fail(PERKS_ERR_INVALID_ARG, "opts is NULL");
  if (o->dtype != PERKS_FP64 && o->dtype != PERKS_FP32 && o->dtype != PERKS_MIXED)
    return fail(PERKS_ERR_INVALID_ARG, "unknown CG dtype");
  if (o->stop != PERKS_STOP_ABS_RR && o->stop != PERKS_STOP_REL) return fail(PERKS_ERR_INVALID_ARG, "unknown stop rule");
  if (o->max_iter < 0 || !(o->tol >= 0)) return fail(PERKS_ERR_INVALID_ARG, "bad max_iter or tol");
  if (o->kernel != PERKS_KERNEL_PERSISTENT && o->kernel != PERKS_KERNEL_PER_STEP)
    return fail(PERKS_ERR_INVALID_ARG, "unknown kernel kind");
  if (o->dtype == PERKS_MIXED && o->kernel != PERKS_KERNEL_PERSISTENT)
    return fail(PERKS_ERR_UNSUPPORTED, "mixed precision runs in the persistent kernel only");
  if (o->algorithm != PERKS_CG_PLAIN && o->algorithm != PERKS_CG_SINGLE_REDUCTION)
    return fail(PERKS_ERR_INVALID_ARG, "unknown CG algorithm");
  const bool single_red = o->algorithm == PERKS_CG_SINGLE_REDUCTION;
  if (single_red && (o->kernel != PERKS_KERNEL_PERSISTENT || o->dtype == PERKS_MIXED || o->checkpoint))
    return fail(PERKS_ERR_UNSUPPORTED,
                "the single-reduction CG runs in the persistent kernel, FP64 or FP32, without a checkpoint");
  perks_cg_state* ck = o->checkpoint;
  if (ck) {
    if (!ck->d_r || !ck->d_p || ck->k < 0) return fail(PERKS_ERR_INVALID_ARG, "bad checkpoint");
    if (o->dtype == PERKS_MIXED && !ck->d_xs)
      return fail(PERKS_ERR_INVALID_ARG, "a mixed-precision checkpoint needs d_xs");
    if (ck->k > 0 && ck->kernel != o->kernel)
      return fail(PERKS_ERR_INVALID_ARG, "checkpoint was written by the other kernel kind");
    // d_r and d_p hold n elements of the writer's working type: a different
    // dtype or size would read and write them out of bounds
    if (ck->k > 0 && ck->dtype != o->dtype)
      return fail(PERKS_ERR_INVALID_ARG, "checkpoint was written by a solve of another dtype");
    if (ck->k > 0 && ck->n != A.n)
      return fail(PERKS_ERR_INVALID_ARG, "checkpoint was written by a solve of " + std::to_string(ck->n) +
                                             " rows, this one has " + std::to_string(A.n));
  }
  const bool resume = ck && ck->k > 0;
  const DeviceInfo* dev = device_info();
  if (!dev) return PERKS_ERR_NO_DEVICE;
  cudaStream_t s = static_cast<cudaStream_t>(o->stream);
  const int n = A.n;
  const bool f32 = o->dtype == PERKS_FP32;
  const size_t ws = f32 || o->dtype == PERKS_MIXED ? 4 : 8;  // working precision bytes
  int st = PERKS_OK;
  const int ctas = o->ctas > 0 ? std::min(o->ctas, dev->sms) : dev->sms;
  const int cl = o->cluster > 1 ? o->cluster : 1;
  if (cl > kMaxCluster || (cl & (cl - 1)) != 0)
    return fail(PERKS_ERR_INVALID_ARG, "cluster must be 1, 2, 4, 8 or 16");
  if (cl > 1 && o->kernel != PERKS_KERNEL_PERSISTENT)
    return fail(PERKS_ERR_INVALID_ARG, "clusters are an option of the persistent kernel");
  int ctas_used = ctas;
  const size_t vbytes = (size_t(n) * ws + 255) & ~size_t(255);
  const size_t nval = A.fmt == 0 ? size_t(A.nnz) : size_t(A.ndiag) * n;
  constexpr size_t kTail = 80 * 1024;   // partial sums (4 slots x 2 x 1024 CTAs) + scalars
  size_t need = 4 * vbytes + kTail;     // r, p (two buffers), Ap + tail
  if (o->dtype == PERKS_MIXED) need += vbytes + ((nval * 4 + 255) & ~size_t(255));  // x_s, FP32 values
  unsigned char* w = static_cast<unsigned char*>(workspace(kWsCgVec, need, &st));
  if (!w) return st;
  SyncWords sw;
  if ((st = sync_words(&sw, s)) != PERKS_OK) return st;
  CgParams P{};
  P.A = A;
  P.b = b;
  P.x = x;
  P.r = w;
  P.p[0] = w + vbytes;
  P.p[1] = w + 3 * vbytes;
  P.Ap = w + 2 * vbytes;
  unsigned char* tail = w + 4 * vbytes;
  P.part = reinterpret_cast<double*>(tail);          // 4 slots x 2 x (<= 1024 CTAs)
  double* scal = P.part + 8 * 1024;                    // device scalars / results (32 doubles)
  unsigned char* more = tail + kTail;
  if (o->dtype == PERKS_MIXED) {
    P.xs = reinterpret_cast<float*>(more);
    P.val32 = reinterpret_cast<float*>(more + vbytes);
  }
  P.tol = o->tol;
  P.stop = o->stop;
  P.max_iter = o->max_iter;
  P.static_iter = o->static_iter;
  P.replace_every = o->replace_every;
  P.delta2 = 0.1 * 0.1;
  P.out_iter = reinterpret_cast<int*>(scal + 16);
  P.out_outer = reinterpret_cast<int*>(scal + 17);
  P.out_rr = scal + 18;  // [18..22]
  P.keep_state = ck != nullptr;
  if (resume) {
    P.resume = 1;
    P.k0 = ck->k;
    P.rr0 = ck->rr;
    P.rrp0 = ck->rr_prev;
    P.bb0 = ck->bb;
    P.maxrr0 = ck->maxrr;
    P.outer0 = ck->outer;
    P.since0 = ck->since;
  }
  P.bar = sw.bar;
  P.status = sw.status;
  P.ctl = wait_ctl();
  PERKS_CUDA(cudaMemsetAsync(scal, 0, 32 * sizeof(double), s));

  // The timed region includes the matrix setup below.
  cudaEvent_t e0, e1;
  PERKS_CUDA(cudaEventCreate(&e0));
  PERKS_CUDA(cudaEventCreate(&e1));
  PERKS_CUDA(cudaEventRecord(e0, s));

  // Working matrix of the persistent kernels: CSR with bounded rows -> ELL.
  P.A64 = A;
  const bool mixed = o->dtype == PERKS_MIXED;
  bool as_dia = false;
  if (A.fmt == 0 && o->kernel == PERKS_KERNEL_PERSISTENT && n > 0) {
    // 64 table slots + 2 flags in the CG vector workspace's spare tail
    int* tab = reinterpret_cast<int*>(scal + 32);
    int* flags = tab + 64;
    std::vector<int> init(66, kEmpty);
    init[64] = init[65] = 0;
    PERKS_CUDA(cudaMemcpyAsync(tab, init.data(), 66 * sizeof(int), cudaMemcpyHostToDevice, s));
    csr_diag_scan<<<dev->sms * 8, 256, 0, s>>>(A.rp, A.ci, n, tab, flags);
    std::vector<int> got(66);
    PERKS_CUDA(cudaMemcpyAsync(got.data(), tab, 66 * sizeof(int), cudaMemcpyDeviceToHost, s));
    PERKS_CUDA(cudaStreamSynchronize(s));
    count_launch(1);
    std::vector<int> offs;
    for (int h = 0; h < 64; h++)
      if (got[h] != kEmpty) offs.push_back(got[h]);
    std::sort(offs.begin(), offs.end());
    if (!got[64] && !got[65] && !offs.empty() && int(offs.size()) <= kMaxDiag &&
        4ll * (long long)offs.size() * n <= 5ll * std::max(A.nnz, 1)) {
      const size_t evb = (f32 || mixed) ? 4 : 8;
      const size_t bytes = offs.size() * size_t(n) * evb;
      void* data = workspace(kWsCgMat, bytes, &st);
      if (!data) return st;
      PERKS_CUDA(cudaMemsetAsync(data, 0, bytes, s));
      CgMat D{};
      D.n = n;
      D.fmt = 1;
      D.ndiag = int(offs.size());
      for (int k = 0; k < D.ndiag; k++) D.off[k] = offs[k];
      const int g = dev->sms * 8;
      if (f32)
        dia_build<float, float><<<g, 256, 0, s>>>(D, A.rp, A.ci, static_cast<const float*>(A.val), static_cast<float*>(data));
      else if (mixed)
        dia_build<double, float><<<g, 256, 0, s>>>(D, A.rp, A.ci, static_cast<const double*>(A.val), static_cast<float*>(data));
      else
        dia_build<double, double><<<g, 256, 0, s>>>(D, A.rp, A.ci, static_cast<const double*>(A.val), static_cast<double*>(data));
      PERKS_CUDA(cudaGetLastError());
      count_launch(1);
      D.val = mixed ? nullptr : data;
      P.A = D;
      if (mixed) P.val32 = static_cast<float*>(data);
      as_dia = true;
    }
  }
  if (A.fmt == 0 && o->kernel == PERKS_KERNEL_PERSISTENT && n > 0 && !as_dia) {
    int* mx = reinterpret_cast<int*>(scal + 24);
    csr_max_row<<<dev->sms * 4, 256, 0, s>>>(A.rp, n, mx);
    int ew = 0;
    PERKS_CUDA(cudaMemcpyAsync(&ew, mx, sizeof(int), cudaMemcpyDeviceToHost, s));
    PERKS_CUDA(cudaStreamSynchronize(s));
    count_launch(1);
    if (ew >= 1 && ew <= 64 && 4ll * ew * n <= 5ll * std::max(A.nnz, 1)) {
      const size_t evb = (f32 || mixed) ? 4 : 8;
      const size_t ci_bytes = (size_t(ew) * n * 4 + 255) & ~size_t(255);
      unsigned char* m = static_cast<unsigned char*>(workspace(kWsCgMat, ci_bytes + size_t(ew) * n * evb, &st));
      if (!m) return st;
      int* eci = reinterpret_cast<int*>(m);
      void* ev = m + ci_bytes;
      const int g = dev->sms * 8;
      if (f32)
        ell_build<float, float><<<g, 256, 0, s>>>(A.rp, A.ci, static_cast<const float*>(A.val), n, ew, eci,
                                                   static_cast<float*>(ev));
      else if (mixed)
        ell_build<double, float><<<g, 256, 0, s>>>(A.rp, A.ci, static_cast<const double*>(A.val), n, ew, eci,
                                                    static_cast<float*>(ev));
      else
        ell_build<double, double><<<g, 256, 0, s>>>(A.rp, A.ci, static_cast<const double*>(A.val), n, ew, eci,
                                                     static_cast<double*>(ev));
      PERKS_CUDA(cudaGetLastError());
      count_launch(1);
      P.A.fmt = 2;
      P.A.ew = ew;
      P.A.eci = eci;
      P.A.val = mixed ? nullptr : ev;
      if (mixed) P.val32 = static_cast<float*>(ev);
    }
  }
  if (A.fmt == 0 && o->kernel == PERKS_KERNEL_PERSISTENT && n > 0 && P.A.fmt == 0) {
    // Irregular CSR: SELL-32 copy with rows sorted by length within windows,
    // kept when its padding stays below 30% of the entries
    const int nwin = (n + kSellWindow - 1) / kSellWindow, ns = nwin * (kSellWindow / 32);
    const size_t rows_b = (size_t(ns) * 32 * 4 + 255) & ~size_t(255);
    const size_t wid_b = (size_t(ns) * 4 + 255) & ~size_t(255);
    const size_t ptr_b = (size_t(ns + 1) * 4 + 255) & ~size_t(255);
    unsigned char* mw = static_cast<unsigned char*>(workspace(kWsCgSell, rows_b + wid_b + ptr_b + 256, &st));
    if (!mw) return st;
    int* sl_row = reinterpret_cast<int*>(mw);
    int* width = reinterpret_cast<int*>(mw + rows_b);
    int* sl_ptr = reinterpret_cast<int*>(mw + rows_b + wid_b);
    long long* tot = reinterpret_cast<long long*>(mw + rows_b + wid_b + ptr_b);
    sell_sort<<<nwin, kSellWindow, 0, s>>>(A.rp, n, sl_row, width);
    sell_scan<<<1, 1024, 0, s>>>(width, ns, sl_ptr, tot);
    long long total = 0;
    PERKS_CUDA(cudaMemcpyAsync(&total, tot, sizeof(total), cudaMemcpyDeviceToHost, s));
    PERKS_CUDA(cudaStreamSynchronize(s));
    count_launch(2);
    if (total < 0x7fffffffll && 10 * total <= 13ll * std::max(A.nnz, 1)) {
      const size_t evb = (f32 || mixed) ? 4 : 8;
      const size_t ci_bytes = (size_t(total) * 4 + 255) & ~size_t(255);
      unsigned char* m = static_cast<unsigned char*>(workspace(kWsCgMat, ci_bytes + size_t(total) * evb + 16, &st));
      if (!m) return st;
      int* eci = reinterpret_cast<int*>(m);
      void* ev = m + ci_bytes;
      CgMat S = A;
      S.fmt = 3;
      S.eci = eci;
      S.sl_ptr = sl_ptr;
      S.sl_row = sl_row;
      S.nslices = ns;
      const int g = dev->sms * 8;
      if (f32)
        sell_fill<float, float><<<g, 256, 0, s>>>(S, A.rp, A.ci, static_cast<const float*>(A.val), eci,
                                                   static_cast<float*>(ev));
      else if (mixed)
        sell_fill<double, float><<<g, 256, 0, s>>>(S, A.rp, A.ci, static_cast<const double*>(A.val), eci,
                                                    static_cast<float*>(ev));
      else
        sell_fill<double, double><<<g, 256, 0, s>>>(S, A.rp, A.ci, static_cast<const double*>(A.val), eci,
                                                     static_cast<double*>(ev));
      PERKS_CUDA(cudaGetLastError());
      count_launch(1);
      S.val = mixed ? nullptr : ev;
      P.A = S;
      if (mixed) P.val32 = static_cast<float*>(ev);
    }
  }
  if (A.fmt == 0) {  // CSR SpMV: lanes per row, about half the mean row length
    const long long avg = (A.nnz + std::max(n, 1) - 1) / std::max(n, 1);
    int g = 4;
    while (g < 32 && 2ll * g < avg) g *= 2;
    P.A64.grp = g;  // the FP64 true residual of mixed precision uses the matrix as given
    if (P.A.fmt == 0) P.A.grp = g;
  }
  if (mixed && P.A.fmt == A.fmt) {  // no converted copy: FP32 copy of the given values
    to_f32<<<dev->sms * 8, 256, 0, s>>>(static_cast<const double*>(A.val), nval, P.val32);
    PERKS_CUDA(cudaGetLastError());
    count_launch(1);
  }

  // the iterate's p: FP32 persistent iterations that form p in the gather
  // (DIA, ELL) alternate two buffers (iteration k writes P.p[k & 1]); the
  // others keep p in P.p[0]
  auto p_of = [&](int k) {
    const bool fused32 = f32 && o->kernel == PERKS_KERNEL_PERSISTENT && P.A.fmt != 0 && P.A.fmt != 3;
    return (fused32 || mixed) ? P.p[k & 1] : P.p[0];
  };
  if (resume) {
    PERKS_CUDA(cudaMemcpyAsync(P.r, ck->d_r, size_t(n) * ws, cudaMemcpyDeviceToDevice, s));
    PERKS_CUDA(cudaMemcpyAsync(p_of(ck->k), ck->d_p, size_t(n) * ws, cudaMemcpyDeviceToDevice, s));
    if (mixed) PERKS_CUDA(cudaMemcpyAsync(P.xs, ck->d_xs, size_t(n) * 4, cudaMemcpyDeviceToDevice, s));
  }
  int launches = 0;
  if (o->kernel == PERKS_KERNEL_PERSISTENT) {
    const int f = P.A.fmt;
    const void* kern =
        single_red
            ? (f32 ? (f == 0 ? (const void*)cg_single_red<float, 0> : f == 1 ? (const void*)cg_single_red<float, 1>
                      : f == 2 ? (const void*)cg_single_red<float, 2> : (const void*)cg_single_red<float, 3>)
                   : (f == 0 ? (const void*)cg_single_red<double, 0> : f == 1 ? (const void*)cg_single_red<double, 1>
                      : f == 2 ? (const void*)cg_single_red<double, 2> : (const void*)cg_single_red<double, 3>))
        : o->dtype == PERKS_MIXED
            ? (f == 0 ? (const void*)cg_mixed<0, 0>
               : f == 2 ? (const void*)cg_mixed<2, 0>
               : f == 3 ? (const void*)cg_mixed<3, 0>
               : A.fmt == 1 ? (const void*)cg_mixed<1, 1> : (const void*)cg_mixed<1, 0>)
        : f32 ? (f == 0 ? (const void*)cg_persistent<float, 0> : f == 1 ? (const void*)cg_persistent<float, 1>
                 : f == 2 ? (const void*)cg_persistent<float, 2> : (const void*)cg_persistent<float, 3>)
              : (f == 0 ? (const void*)cg_persistent<double, 0> : f == 1 ? (const void*)cg_persistent<double, 1>
                 : f == 2 ? (const void*)cg_persistent<double, 2> : (const void*)cg_persistent<double, 3>);
    // Shared memory for the vectors that only their owning CTA touches, in
    // order of accesses saved per iteration: r (3, unless the SpMV gathers
    // it or, SELL, writes rows of other CTAs), x or the mixed increment x_s
    // (2), Ap (2, not SELL). Each takes its CTA's rows up to what is left of
    // the budget; rows past a cap stream through global memory. The budget
    // is taken from the L1 cache (one 256 KB store per SM), on which the
    // SpMV gathers depend. Measured on GB300 (2D Laplacian 2048^2, us per
    // iteration, FP64 / mixed / FP32): none 110.6 / 61.4 / 54.0, 160 KB
    // 102.8 / 56.0 / 48.9, the whole ~220 KB 130.3 / 66.5 / 63.8; no effect
    // on the SELL layout (only x can stay). Default: 160 KB for DIA and ELL.
    cudaFuncAttributes fa{};
    PERKS_CUDA(cudaFuncGetAttributes(&fa, kern));
    const bool gathered_r = ((f32 || mixed) && (f == 1 || f == 2)) || f == 3;
    const size_t es = ws;  // FP64 / FP32; mixed: the FP32 r, x_s, Ap
    const long long most = (long long)dev->smem_optin - (long long)fa.sharedSizeBytes - 256;
    const int kb = o->cache_vectors >= 0 ? o->cache_vectors : ((f == 1 || f == 2) ? kCgResidentKB : 0);
    long long budget = std::min<long long>(most, 1024ll * kb);
    // rows of the CTA with the most: DIA/ELL split evenly; CSR (merge path)
    // and SELL (whole 1024-row windows) vary around n / ctas
    const long long even = (n + ctas - 1) / ctas;
    const long long span = (f == 1 || f == 2) ? even + 4 : std::min<long long>(n + 4, even + even / 4 + 1028);
    auto take = [&](bool allowed) {
      if (!allowed || budget <= 0) return 0;
      const long long rows = std::min<long long>((budget / (long long)es) & ~3ll, (span + 3) & ~3ll);
      budget -= rows * (long long)es;
      return int(rows);
    };
    // the single-reduction kernel keeps p, x and s (= A p) instead: all three
    // are touched by their owning CTA only
    P.cap_r = take(single_red || !gathered_r);
    P.cap_x = take(true);
    P.cap_ap = take(single_red || f != 3);
    const size_t dsmem = size_t(P.cap_r + P.cap_x + P.cap_ap) * es;
    PERKS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(dsmem)));
    int per_sm = 0;
    PERKS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kCgThreads, dsmem));
    if (per_sm < 1) return fail(PERKS_ERR_LAUNCH, "CG kernel does not fit on an SM");
    void* args[] = {&P};
    cudaError_t e;
    if (cl > 1) {
      // cooperative launch (every CTA resident, for the grid barrier) in
      // thread-block clusters of `cl` CTAs; the grid is as many whole
      // clusters as can be resident at once
      cudaLaunchAttribute at[2];
      at[0].id = cudaLaunchAttributeCooperative;
      at[0].val.cooperative = 1;
      at[1].id = cudaLaunchAttributeClusterDimension;
      at[1].val.clusterDim.x = unsigned(cl);
      at[1].val.clusterDim.y = 1;
      at[1].val.clusterDim.z = 1;
      cudaLaunchConfig_t cfg{};
      cfg.blockDim = dim3(kCgThreads);
      cfg.dynamicSmemBytes = dsmem;
      cfg.stream = s;
      cfg.attrs = at;
      cfg.numAttrs = 2;
      if (cl > 8) PERKS_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
      cfg.gridDim = dim3(unsigned(ctas / cl * cl));
      int maxcl = 0;
      e = cudaOccupancyMaxActiveClusters(&maxcl, kern, &cfg);
      if (e != cudaSuccess) return cuda_fail(e, "cudaOccupancyMaxActiveClusters(cg)");
      const int grid = std::min(ctas / cl, maxcl) * cl;
      if (grid < cl) return fail(PERKS_ERR_UNSUPPORTED, "no cluster of " + std::to_string(cl) + " CTAs fits");
      cfg.gridDim = dim3(unsigned(grid));
      P.cluster = cl;
      e = cudaLaunchKernelExC(&cfg, kern, args);
      if (e != cudaSuccess) return cuda_fail(e, "cudaLaunchKernelExC(cg, cooperative clusters)");
      ctas_used = grid;
    } else {
      P.cluster = 1;
      e = cudaLaunchCooperativeKernel(kern, dim3(ctas), dim3(kCgThreads), args, dsmem, s);
      if (e != cudaSuccess) return cuda_fail(e, "cudaLaunchCooperativeKernel(cg)");
    }
    launches = 1;
  } else {
    // one launch per phase; scalars on the device; the host checks the
    // convergence flag every `chunk` iterations
    double* sv = scal;  // s[0..5]
    const int grid = dev->sms * 2, bt = 512;
    double* part = P.part;
    double flag = 0.0;
    if (resume) {  // scalars of the checkpoint, with the stop test of cg_phase_reduce
      const double tol2 = o->stop == PERKS_STOP_REL ? o->tol * o->tol * ck->bb
                          : f32 ? double(float(o->tol) * float(o->tol)) : o->tol * o->tol;
      const double hs0[6] = {ck->rr, ck->rr_prev, 0.0, ck->bb,
                             ((!o->static_iter && ck->rr < tol2) || ck->k >= o->max_iter) ? 1.0 : 0.0,
                             double(ck->k)};
      PERKS_CUDA(cudaMemcpyAsync(sv, hs0, sizeof(hs0), cudaMemcpyHostToDevice, s));
      flag = hs0[4];
    } else if (f32) {
      cg_phase_init<float><<<grid, bt, 0, s>>>(P, part);
      cg_phase_reduce<float><<<1, 1024, 0, s>>>(P, part, grid, sv, 0);
      launches = 2;
    } else {
      cg_phase_init<double><<<grid, bt, 0, s>>>(P, part);
      cg_phase_reduce<double><<<1, 1024, 0, s>>>(P, part, grid, sv, 0);
      launches = 2;
    }
    const int chunk = 32;
    for (int it = 0; it < o->max_iter + 1 && flag == 0.0; it += chunk) {
      for (int c = 0; c < chunk; c++) {
        if (f32) {
          cg_phase_p<float><<<grid, bt, 0, s>>>(P, sv);
          cg_phase_spmv<float><<<grid, bt, 0, s>>>(P, sv, part);
          cg_phase_reduce<float><<<1, 1024, 0, s>>>(P, part, grid, sv, 2);
          cg_phase_update<float><<<grid, bt, 0, s>>>(P, sv, part);
          cg_phase_reduce<float><<<1, 1024, 0, s>>>(P, part, grid, sv, 1);
        } else {
          cg_phase_p<double><<<grid, bt, 0, s>>>(P, sv);
          cg_phase_spmv<double><<<grid, bt, 0, s>>>(P, sv, part);
          cg_phase_reduce<double><<<1, 1024, 0, s>>>(P, part, grid, sv, 2);
          cg_phase_update<double><<<grid, bt, 0, s>>>(P, sv, part);
          cg_phase_reduce<double><<<1, 1024, 0, s>>>(P, part, grid, sv, 1);
        }
        launches += 5;
      }
      PERKS_CUDA(cudaMemcpyAsync(&flag, sv + 4, sizeof(double), cudaMemcpyDeviceToHost, s));
      PERKS_CUDA(cudaStreamSynchronize(s));
    }
    PERKS_CUDA(cudaGetLastError());
  }
  PERKS_CUDA(cudaEventRecord(e1, s));
  count_launch(launches);
  int rc = check_status(sw, s);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != PERKS_OK) return rc;
  // results
  double hs[24] = {0};
  PERKS_CUDA(cudaMemcpyAsync(hs, scal, sizeof(hs), cudaMemcpyDeviceToHost, s));
  PERKS_CUDA(cudaStreamSynchronize(s));
  int iters = 0, outer = 0;
  double rr = 0.0, rr_prev = 0.0, bbs = 0.0, maxrr = 0.0, since = 0.0;
  if (o->kernel == PERKS_KERNEL_PERSISTENT) {
    std::memcpy(&iters, &hs[16], sizeof(int));
    std::memcpy(&outer, &hs[17], sizeof(int));
    rr = hs[18];
    rr_prev = hs[19];
    bbs = hs[20];
    maxrr = hs[21];
    since = hs[22];
  } else {
    iters = int(hs[5]);
    rr = hs[0];
    rr_prev = hs[1];
    bbs = hs[3];
  }
  if (ck) {  // state for a later resume
    PERKS_CUDA(cudaMemcpyAsync(ck->d_r, P.r, size_t(n) * ws, cudaMemcpyDeviceToDevice, s));
    PERKS_CUDA(cudaMemcpyAsync(ck->d_p, p_of(iters), size_t(n) * ws, cudaMemcpyDeviceToDevice, s));
    if (mixed) PERKS_CUDA(cudaMemcpyAsync(ck->d_xs, P.xs, size_t(n) * 4, cudaMemcpyDeviceToDevice, s));
    ck->rr = rr;
    ck->rr_prev = rr_prev;
    ck->bb = bbs;
    ck->maxrr = maxrr;
    ck->outer = outer;
    ck->since = int(since);
    ck->k = iters;
    ck->kernel = o->kernel;
    ck->dtype = o->dtype;
    ck->n = n;
  }
  // true relative residual in FP64
  double* tpart = P.part;
  const int tg = dev->sms * 2;
  const bool val_f32 = f32;
  if (val_f32) cg_true_residual<float><<<tg, 512, 0, s>>>(A, b, x, tpart);
  else cg_true_residual<double><<<tg, 512, 0, s>>>(A, b, x, tpart);
  sum_partials<<<1, 1024, 0, s>>>(tpart, tg, scal + 28);
  count_launch(2);
  double tr[2];
  PERKS_CUDA(cudaMemcpyAsync(tr, scal + 28, sizeof(tr), cudaMemcpyDeviceToHost, s));
  PERKS_CUDA(cudaStreamSynchronize(s));
  if (res) {
    res->iterations = iters;
    res->outer = outer;
    res->rr = rr;
    res->true_rel_res = tr[1] > 0 ? std::sqrt(tr[0] / tr[1]) : std::sqrt(tr[0]);
    res->ms = ms;
    res->launches = launches;
    res->layout = P.A.fmt;
    res->ctas = ctas_used;
  }
  const double thr = o->stop == PERKS_STOP_REL ? o->tol * o->tol * tr[1] : o->tol * o->tol;
  if (!o->static_iter && iters >= o->max_iter && !(rr < thr))
    return fail(PERKS_ERR_NOT_CONVERGED, "CG reached max_iter=" + std::to_string(o->max_iter) +
                                             " (r.r = " + std::to_string(rr) + ")");
  return PERKS_OK;
}

}  // namespace perks

using namespace perks;

extern "C" {

void perks_cg_default_opts(perks_cg_opts* o) {
  if (!o) return;
  *o = perks_cg_opts{};
  o->dtype = PERKS_FP64;
  o->stop = PERKS_STOP_REL;
  o->tol = 1e-10;
  o->max_iter = 100000;
  o->static_iter = 0;
  o->kernel = PERKS_KERNEL_PERSISTENT;
  o->replace_every = 0;
  o->ctas = 0;
  o->stream = nullptr;
  o->checkpoint = nullptr;
  o->cache_vectors = -1;
  o->cluster = 1;
  o->algorithm = PERKS_CG_PLAIN;
}

int perks_cg_csr(int n, int nnz, const int* rp, const int* ci, const void* val, const void* b, void* x,
                 const perks_cg_opts* o, perks_cg_result* res) {
  if (n <= 0 || nnz < 0 || !rp || !ci || !val || !b || !x) return fail(PERKS_ERR_INVALID_ARG, "bad CSR arguments");
  CgMat A{};
  A.n = n;
  A.nnz = nnz;
  A.fmt = 0;
  A.rp = rp;
  A.ci = ci;
  A.val = val;
  return cg_solve(A, b, x, o, res);
}

int perks_cg_dia(int n, int ndiag, const int* off, const void* data, const void* b, void* x, const perks_cg_opts* o,
                 perks_cg_result* res) {
  if (n <= 0 || ndiag <= 0 || ndiag > kMaxDiag || !off || !data || !b || !x)
    return fail(PERKS_ERR_INVALID_ARG, "bad DIA arguments (at most 32 diagonals)");
  CgMat A{};
  A.n = n;
  A.fmt = 1;
  A.ndiag = ndiag;
  for (int k = 0; k < ndiag; k++) {
    if (off[k] <= -n || off[k] >= n) return fail(PERKS_ERR_INVALID_ARG, "DIA offset out of range");
    A.off[k] = off[k];
  }
  A.val = data;
  return cg_solve(A, b, x, o, res);
}

int perks_spmv_csr(int dtype, int n, int nnz, const int* rp, const int* ci, const void* val, const void* x, void* y,
                   void* stream) {
  if (n <= 0 || !rp || !ci || !val || !x || !y) return fail(PERKS_ERR_INVALID_ARG, "bad CSR arguments");
  if (dtype != PERKS_FP32 && dtype != PERKS_FP64) return fail(PERKS_ERR_INVALID_ARG, "dtype");
  const DeviceInfo* dev = device_info();
  if (!dev) return PERKS_ERR_NO_DEVICE;
  CgMat A{};
  A.n = n;
  A.nnz = nnz;
  A.fmt = 0;
  A.rp = rp;
  A.ci = ci;
  A.val = val;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (dtype == PERKS_FP32)
    spmv_kernel<float><<<dev->sms * 4, 256, 0, s>>>(A, static_cast<const float*>(x), static_cast<float*>(y));
  else
    spmv_kernel<double><<<dev->sms * 4, 256, 0, s>>>(A, static_cast<const double*>(x), static_cast<double*>(y));
  count_launch(1);
  PERKS_CUDA(cudaGetLastError());
  PERKS_CUDA(cudaStreamSynchronize(s));
  return PERKS_OK;
}

int perks_spmv_dia(int dtype, int n, int ndiag, const int* off, const void* data, const void* x, void* y,
                   void* stream) {
  if (n <= 0 || ndiag <= 0 || ndiag > kMaxDiag || !off || !data || !x || !y)
    return fail(PERKS_ERR_INVALID_ARG, "bad DIA arguments");
  if (dtype != PERKS_FP32 && dtype != PERKS_FP64) return fail(PERKS_ERR_INVALID_ARG, "dtype");
  const DeviceInfo* dev = device_info();
  if (!dev) return PERKS_ERR_NO_DEVICE;
  CgMat A{};
  A.n = n;
  A.fmt = 1;
  A.ndiag = ndiag;
  for (int k = 0; k < ndiag; k++) A.off[k] = off[k];
  A.val = data;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (dtype == PERKS_FP32)
    spmv_kernel<float><<<dev->sms * 4, 256, 0, s>>>(A, static_cast<const float*>(x), static_cast<float*>(y));
  else
    spmv_kernel<double><<<dev->sms * 4, 256, 0, s>>>(A, static_cast<const double*>(x), static_cast<double*>(y));
  count_launch(1);
  PERKS_CUDA(cudaGetLastError());
  PERKS_CUDA(cudaStreamSynchronize(s));
  return PERKS_OK;
}

}  // extern "C"
