// Batched uneven workload in one persistent launch.
//
// The jobs (independent stencil time loops and CG solves of different sizes
// and precisions) are ordered largest first. A stencil job larger than the
// balancing unit (total work / (2 x SMs)) is cut into row slices, the rest is
// one work item each; the items go into a device queue in that order. Every
// CTA of one launch repeatedly takes the next item from an atomic counter. A
// single-item job needs only CTA barriers; the CTAs holding the slices of one
// job meet at a job barrier (monotonic counter, bounded wait) after every
// time step and read neighbouring rows through L2 (ld.global.cg). This cannot
// deadlock: the grid is fully resident, and a job's slices are consecutive in
// the queue, so by the time any later job's item is taken every slice of every
// earlier job is held by a running CTA.
//   * Stencil job: if both fields fit in the CTA's shared memory they stay
//     there for every time step (the PERKS idea taken to the whole domain);
//     otherwise the CTA ping-pongs between the output and a scratch field in
//     global memory (L2-resident for these sizes). Clamp boundary, reference
//     evaluation order: results are bit-identical to the single-instance path
//     and to the reference CPU code.
//   * CG job: CSR, x0 = 0, CTA-wide reductions, stop at ||r|| <= tol ||b||;
//     FP64, FP32, or mixed precision (the FP32 iteration with FP64 reliable
//     updates of the single-instance solver, so that the job reaches an FP64
//     tolerance).
// A run is a CUDA graph of {reset the counter, launch}; the launch shape
// (threads per CTA, CTAs per SM, hence shared memory per CTA) is chosen by
// timing each candidate once when the plan is created.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>
#include "ptx.cuh"
#include "runtime.cuh"
#include "shapes.cuh"

namespace perks {

struct BJob {  // one job, in queue order
  int kind, dtype, shape, h, wy, wx, steps;
  const void* in;
  void* out;
  void* scratch;  // stencil: second field; CG: r, p, Ap
  int n, nnz;
  const int* rp;
  const int* ci;
  const void* val;
  const void* b;
  void* x;
  double tol;
  int max_iter;
};
struct BRes {
  int iterations, status;
  double rel_res;
};
struct BItem {  // one work item: a job, or one row slice of a stencil job
  int job, slice, nslices, row_lo, row_hi;
};

// Barrier of the nslices CTAs working on one job: monotonic counter, target
// = (steps done) x nslices. False when the wait ran out its budget. `skip`
// (test hook, WaitCtl::skip_cta): this CTA does not arrive, so the wait of
// every slice of the job runs out.
__device__ __forceinline__ bool job_barrier(unsigned* bar, unsigned target, long long budget, bool skip) {
  __shared__ unsigned s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned ok = 1, old = 0u;
    __threadfence();
    if (!skip) asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], 1;" : "=r"(old) : "l"(bar) : "memory");
    if (skip || int(old + 1u - target) < 0) {
      const long long t0 = clock64();
      while (int(ld_acquire_gpu(bar) - target) < 0) {
        if (clock64() - t0 > budget) {
          ok = 0;
          break;
        }
      }
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// CTA-wide sum of one double, valid in every thread (`red`: kRed doubles).
// Warp 0 adds the warp sums and thread 0 publishes the total, with `fin`
// run on it: quotients derived from the total (alpha, beta) are divided once
// per CTA and read from red[33..34] after the same barrier. FP64 issue is 2
// lanes per clock per SM, so a second shuffle tree in every warp, or every
// thread dividing, would cost microseconds per iteration.
constexpr int kRed = 35;
struct NoFin {
  __device__ void operator()(double) const {}
};
template <class Fin = NoFin>
__device__ __forceinline__ double cta_sum(double v, double* red, const Fin& fin = Fin{}) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = lane < nw ? red[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) {
      red[32] = v;
      fin(v);
    }
  }
  __syncthreads();
  return red[32];
}

// One time step over rows [r_lo, r_hi) of the job's (h*wy) rows. L2 = true
// reads through L2 only (other CTAs wrote the source).
template <class T, int SHAPE, bool L2>
__device__ __forceinline__ void stencil_rows(const BJob& J, const T* __restrict__ src, T* __restrict__ dst, int r_lo,
                                             int r_hi) {
  const int h = J.h, wy = J.wy, wx = J.wx;
  const int nt = blockDim.x, tid = threadIdx.x;
  // threads per row (whole warps), rows in parallel
  const int tpr = min(nt, ((wx + 31) / 32) * 32);
  const int rpar = nt / tpr;
  const int r_off = tid / tpr, c0 = tid % tpr;
  if (r_off >= rpar) return;
  for (int row = r_lo + r_off; row < r_hi; row += rpar) {
    const int z = row / wy, y = row - z * wy;
    for (int x = c0; x < wx; x += tpr) {
      auto u = [&](int dz, int dy, int dx) -> T {
        const int zz = min(max(z + dz, 0), h - 1), yy = min(max(y + dy, 0), wy - 1), xx = min(max(x + dx, 0), wx - 1);
        const T* a = src + ((size_t)zz * wy + yy) * wx + xx;
        if constexpr (L2) return __ldcg(a);
        else return *a;
      };
      // FP32: the branch-free short finish of the exact division (divconst.cuh, form 3)
      dst[((size_t)z * wy + y) * wx + x] = stencil_point<T, SHAPE, false, sizeof(T) == 4 ? 3 : 0>(u);
    }
  }
}

// A stencil job cut into nslices row slices, this CTA holding one of them.
template <class T, int SHAPE>
__device__ void batch_stencil_slice(const BJob& J, const BItem& I, unsigned* bar, BRes* res, const WaitCtl& ctl) {
  const int steps = J.steps;
  const T* src = static_cast<const T*>(J.in);
  T* out = static_cast<T*>(J.out);
  T* scratch = static_cast<T*>(J.scratch);
  int done = 0;
  for (int t = 0; t < steps; t++) {
    T* dst = ((steps - 1 - t) & 1) == 0 ? out : scratch;  // the last step writes `out`
    stencil_rows<T, SHAPE, true>(J, src, dst, I.row_lo, I.row_hi);
    if (!job_barrier(bar, unsigned(t + 1) * unsigned(I.nslices), ctl.budget, t == 0 && I.slice == ctl.skip_cta)) break;
    src = dst;
    done = t + 1;
  }
  if (I.slice == 0 && threadIdx.x == 0) {
    res->iterations = done;
    res->status = done == steps ? PERKS_OK : PERKS_ERR_TIMEOUT;
    res->rel_res = 0.0;
  }
}

template <class T, int SHAPE>
__device__ void batch_stencil(const BJob& J, unsigned char* smem, unsigned smem_bytes, BRes* res) {
  const int h = J.h, wy = J.wy, wx = J.wx, steps = J.steps;
  const long long cells = (long long)h * wy * wx;
  const int nt = blockDim.x, tid = threadIdx.x;
  const int rows = h * wy;
  auto sweep = [&](const T* __restrict__ src, T* __restrict__ dst) { stencil_rows<T, SHAPE, false>(J, src, dst, 0, rows); };
  const T* in = static_cast<const T*>(J.in);
  T* out = static_cast<T*>(J.out);
  if (steps == 0) {
    for (long long i = tid; i < cells; i += nt) out[i] = in[i];
  } else if (2 * cells * (long long)sizeof(T) <= (long long)smem_bytes) {
    T* A = reinterpret_cast<T*>(smem);
    T* B = A + cells;
    for (long long i = tid; i < cells; i += nt) A[i] = in[i];
    __syncthreads();
    for (int t = 0; t < steps; t++) {
      sweep(A, B);
      __syncthreads();
      T* tmp = A;
      A = B;
      B = tmp;
    }
    for (long long i = tid; i < cells; i += nt) out[i] = A[i];
  } else {
    T* scratch = static_cast<T*>(J.scratch);
    const T* src = in;
    for (int t = 0; t < steps; t++) {
      T* dst = ((steps - 1 - t) & 1) == 0 ? out : scratch;  // the last step writes `out`
      sweep(src, dst);
      __syncthreads();  // this CTA's global writes are visible to it after the barrier
      src = dst;
    }
  }
  if (tid == 0) {
    res->iterations = steps;
    res->status = PERKS_OK;
    res->rel_res = 0.0;
  }
}

template <class T>
__device__ void batch_cg(const BJob& J, double* red, BRes* res) {
  const int n = J.n, nt = blockDim.x, tid = threadIdx.x;
  const int* __restrict__ rp = J.rp;
  const int* __restrict__ ci = J.ci;
  const T* __restrict__ val = static_cast<const T*>(J.val);
  const T* __restrict__ b = static_cast<const T*>(J.b);
  T* __restrict__ x = static_cast<T*>(J.x);
  T* __restrict__ r = static_cast<T*>(J.scratch);
  T* __restrict__ p = r + ((n + 63) & ~63);
  T* __restrict__ Ap = p + ((n + 63) & ~63);
  double rr = 0.0;
  for (int i = tid; i < n; i += nt) {
    const T bi = b[i];
    x[i] = T(0);
    r[i] = bi;
    p[i] = bi;
    rr += double(bi) * double(bi);
  }
  rr = cta_sum(rr, red);
  const double bb = rr, stop2 = J.tol * J.tol * bb;
  int k = 0, status = PERKS_OK;
  while (k < J.max_iter && rr > stop2) {
    __syncthreads();  // p complete before the SpMV gathers it
    double pap = 0.0;
    for (int i = tid; i < n; i += nt) {
      T acc = T(0);
      for (int j = rp[i]; j < rp[i + 1]; j++) acc = fma(val[j], p[ci[j]], acc);
      Ap[i] = acc;
      pap += double(p[i]) * double(acc);
    }
    pap = cta_sum(pap, red, [rr, red](double t) { red[33] = double(T(rr / t)); });
    if (!(pap > 0.0) || !isfinite(pap)) {
      status = PERKS_ERR_BREAKDOWN;
      break;
    }
    const T alpha = T(red[33]);
    double rrn = 0.0;
    for (int i = tid; i < n; i += nt) {
      x[i] = fma(alpha, p[i], x[i]);
      const T ri = fma(-alpha, Ap[i], r[i]);
      r[i] = ri;
      rrn += double(ri) * double(ri);
    }
    rrn = cta_sum(rrn, red, [rr, red](double t) { red[34] = double(T(t / rr)); });
    const T beta = T(red[34]);
    for (int i = tid; i < n; i += nt) p[i] = fma(beta, p[i], r[i]);
    rr = rrn;
    k++;
  }
  if (status == PERKS_OK && rr > stop2) status = PERKS_ERR_NOT_CONVERGED;
  if (tid == 0) {
    res->iterations = k;
    res->status = status;
    res->rel_res = bb > 0.0 ? sqrt(rr / bb) : sqrt(rr);
  }
}

// Mixed-precision CG job in one CTA (the reliable-update scheme of the
// single-instance cg_mixed: Sleijpen & van der Vorst 1996): the Krylov
// iteration runs in FP32 on an FP32 copy of the values (products summed in
// FP32 per row, dot products in FP64); the solution x is accumulated in FP64,
// and whenever the recursive r.r has dropped by delta^2 = 0.01 since the last
// update (or claims convergence, or the iteration cap is reached) x += x_s and
// r = b - A x is recomputed with the FP64 values. Convergence is declared on
// that FP64 true residual only. Scratch: FP32 r, p, Ap, x_s and the values.
__device__ void batch_cg_mixed(const BJob& J, double* red, BRes* res) {
  const int n = J.n, nt = blockDim.x, tid = threadIdx.x;
  const int* __restrict__ rp = J.rp;
  const int* __restrict__ ci = J.ci;
  const double* __restrict__ val = static_cast<const double*>(J.val);
  const double* __restrict__ b = static_cast<const double*>(J.b);
  double* __restrict__ x = static_cast<double*>(J.x);
  const size_t np = size_t((n + 63) & ~63);
  float* __restrict__ r = static_cast<float*>(J.scratch);
  float* __restrict__ p = r + np;
  float* __restrict__ Ap = p + np;
  float* __restrict__ xs = Ap + np;
  float* __restrict__ v32 = xs + np;
  for (int j = tid; j < J.nnz; j += nt) v32[j] = float(val[j]);
  double rr = 0.0;
  for (int i = tid; i < n; i += nt) {
    const double bi = b[i];
    x[i] = 0.0;
    r[i] = float(bi);
    xs[i] = 0.0f;
    rr += bi * bi;
  }
  rr = cta_sum(rr, red);  // also orders the writes above before the reads below
  const double bb = rr, stop2 = J.tol * J.tol * bb;
  double maxrr = rr, rr0 = 0.0;
  int k = 0, status = PERKS_OK;
  while (k < J.max_iter && rr > stop2) {
    const float beta = k > 0 ? float(red[34]) : 0.0f;  // rr / rr0, divided by thread 0 below
    for (int i = tid; i < n; i += nt) p[i] = k > 0 ? fmaf(beta, p[i], r[i]) : r[i];
    __syncthreads();  // p complete before the SpMV gathers it
    double pap = 0.0;
    for (int i = tid; i < n; i += nt) {
      float acc = 0.0f;
      for (int j = rp[i]; j < rp[i + 1]; j++) acc = fmaf(v32[j], p[ci[j]], acc);
      Ap[i] = acc;
      pap += double(p[i] * acc);
    }
    pap = cta_sum(pap, red, [rr, red](double t) { red[33] = double(float(rr / t)); });
    if (!(pap > 0.0) || !isfinite(pap)) {
      status = PERKS_ERR_BREAKDOWN;
      break;
    }
    const float alpha = float(red[33]);
    double rrn = 0.0;
    for (int i = tid; i < n; i += nt) {
      xs[i] = fmaf(alpha, p[i], xs[i]);
      const float ri = fmaf(-alpha, Ap[i], r[i]);
      r[i] = ri;
      rrn += double(ri * ri);
    }
    // the next iteration's rr / rr0 (replaced after a reliable update)
    auto fin_beta = [rr, red](double t) { red[34] = double(float(t / rr)); };
    rrn = cta_sum(rrn, red, fin_beta);
    k++;
    if (rrn < 0.01 * maxrr || rrn <= stop2 || k == J.max_iter) {
      // reliable update: x += x_s in FP64, true residual with the FP64 values
      for (int i = tid; i < n; i += nt) {
        x[i] += double(xs[i]);
        xs[i] = 0.0f;
      }
      __syncthreads();  // x complete before the SpMV gathers it
      double rt = 0.0;
      for (int i = tid; i < n; i += nt) {
        double acc = 0.0;
        for (int j = rp[i]; j < rp[i + 1]; j++) acc = fma(val[j], x[ci[j]], acc);
        const double ri = b[i] - acc;
        r[i] = float(ri);
        rt += ri * ri;
      }
      rrn = cta_sum(rt, red, fin_beta);
      maxrr = rrn;
    }
    rr0 = rr;
    rr = rrn;
  }
  if (status == PERKS_OK && rr > stop2) status = PERKS_ERR_NOT_CONVERGED;
  if (tid == 0) {
    res->iterations = k;
    res->status = status;
    res->rel_res = bb > 0.0 ? sqrt(rr / bb) : sqrt(rr);
  }
}

// counter[0]: the queue; counter[1 + job]: the job barriers (all zero at launch)
__global__ void __launch_bounds__(1024, 1)
    batch_kernel(const BJob* __restrict__ jobs, const BItem* __restrict__ items, int nitems, BRes* res,
                 unsigned* counter, unsigned smem_bytes, const WaitCtl ctl) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ int sq;
  __shared__ double red[kRed];
  while (true) {
    if (threadIdx.x == 0) sq = int(atomicAdd(counter, 1u));
    __syncthreads();
    const int q = sq;
    if (q >= nitems) break;
    const BItem I = items[q];
    const int j = I.job;
    const BJob& J = jobs[j];
    const bool f64 = J.dtype == PERKS_FP64;
    if (I.nslices > 1) {
      unsigned* bar = counter + 1 + j;
      switch (J.shape) {
        case PERKS_2D5PT:
          if (f64) batch_stencil_slice<double, PERKS_2D5PT>(J, I, bar, res + j, ctl);
          else batch_stencil_slice<float, PERKS_2D5PT>(J, I, bar, res + j, ctl);
          break;
        case PERKS_2DS9PT:
          if (f64) batch_stencil_slice<double, PERKS_2DS9PT>(J, I, bar, res + j, ctl);
          else batch_stencil_slice<float, PERKS_2DS9PT>(J, I, bar, res + j, ctl);
          break;
        case PERKS_2D9PT:
          if (f64) batch_stencil_slice<double, PERKS_2D9PT>(J, I, bar, res + j, ctl);
          else batch_stencil_slice<float, PERKS_2D9PT>(J, I, bar, res + j, ctl);
          break;
        default:
          if (f64) batch_stencil_slice<double, PERKS_3D7PT>(J, I, bar, res + j, ctl);
          else batch_stencil_slice<float, PERKS_3D7PT>(J, I, bar, res + j, ctl);
          break;
      }
    } else if (J.kind == PERKS_JOB_CG) {
      if (J.dtype == PERKS_MIXED) batch_cg_mixed(J, red, res + j);
      else if (f64) batch_cg<double>(J, red, res + j);
      else batch_cg<float>(J, red, res + j);
    } else {
      switch (J.shape) {
        case PERKS_2D5PT:
          if (f64) batch_stencil<double, PERKS_2D5PT>(J, smem, smem_bytes, res + j);
          else batch_stencil<float, PERKS_2D5PT>(J, smem, smem_bytes, res + j);
          break;
        case PERKS_2DS9PT:
          if (f64) batch_stencil<double, PERKS_2DS9PT>(J, smem, smem_bytes, res + j);
          else batch_stencil<float, PERKS_2DS9PT>(J, smem, smem_bytes, res + j);
          break;
        case PERKS_2D9PT:
          if (f64) batch_stencil<double, PERKS_2D9PT>(J, smem, smem_bytes, res + j);
          else batch_stencil<float, PERKS_2D9PT>(J, smem, smem_bytes, res + j);
          break;
        default:  // PERKS_3D7PT (validated on the host)
          if (f64) batch_stencil<double, PERKS_3D7PT>(J, smem, smem_bytes, res + j);
          else batch_stencil<float, PERKS_3D7PT>(J, smem, smem_bytes, res + j);
          break;
      }
    }
    __syncthreads();  // every thread has read sq before it is overwritten
  }
}

}  // namespace perks

using namespace perks;

struct perks_batch_plan_s {
  int device = -1;
  cudaStream_t stream = nullptr;
  int njobs = 0;
  std::vector<int> order;  // queue position -> caller's index
  std::vector<long long> cells_of;  // per queue position, stencil cells x sizeof (0 for CG)
  BJob* d_jobs = nullptr;
  BItem* d_items = nullptr;
  int nitems = 0, sliced = 0, slicing = 0;
  BRes* d_res = nullptr;
  unsigned* d_counter = nullptr;
  void* d_scratch = nullptr;
  int threads = 0, ctas_per_sm = 0, grid = 0, tuned = 0, resident = 0;
  unsigned smem = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  float last_ms = 0.f;
  WaitCtl ctl;  // wait budget of the plan's launches (taken when the plan is made)
};

namespace {

bool batch_shape_ok(int s) {
  return s == PERKS_2D5PT || s == PERKS_2DS9PT || s == PERKS_2D9PT || s == PERKS_3D7PT;
}

void plan_free(perks_batch_plan p) {
  if (!p) return;
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  if (p->e0) cudaEventDestroy(p->e0);
  if (p->e1) cudaEventDestroy(p->e1);
  cudaFree(p->d_jobs);
  cudaFree(p->d_items);
  cudaFree(p->d_res);
  cudaFree(p->d_counter);
  cudaFree(p->d_scratch);
  delete p;
}

// Shared memory per CTA for a launch shape (dynamic part).
unsigned smem_for(const DeviceInfo* dev, int ctas_per_sm) {
  const size_t per_sm = 228 * 1024;  // GB300 shared memory per SM
  size_t s = per_sm / size_t(ctas_per_sm) - 1024 - 512;  // CTA reservation + static smem
  return unsigned(std::min(s, dev->smem_optin));
}

int launch_once(perks_batch_plan p, cudaStream_t s, int threads, int ctas, unsigned smem, float* ms) {
  PERKS_CUDA(cudaFuncSetAttribute(batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  const int grid = device_info()->sms * ctas;
  PERKS_CUDA(cudaMemsetAsync(p->d_counter, 0, sizeof(unsigned) * (1 + p->njobs), s));
  PERKS_CUDA(cudaEventRecord(p->e0, s));
  batch_kernel<<<grid, threads, smem, s>>>(p->d_jobs, p->d_items, p->nitems, p->d_res, p->d_counter, smem,
                                           p->ctl);
  PERKS_CUDA(cudaGetLastError());
  PERKS_CUDA(cudaEventRecord(p->e1, s));
  PERKS_CUDA(cudaEventSynchronize(p->e1));
  count_launch(1);
  PERKS_CUDA(cudaEventElapsedTime(ms, p->e0, p->e1));
  return PERKS_OK;
}

}  // namespace

extern "C" {

void perks_batch_default_opts(perks_batch_opts* o) {
  if (!o) return;
  *o = perks_batch_opts{};
}

int perks_batch_plan_create(const perks_job* jobs, int njobs, const perks_batch_opts* opts, perks_batch_plan* out) {
  if (!out) return fail(PERKS_ERR_INVALID_ARG, "plan is NULL");
  *out = nullptr;
  if (!jobs || njobs <= 0) return fail(PERKS_ERR_INVALID_ARG, "no jobs");
  perks_batch_opts o{};
  if (opts) o = *opts;
  if (o.threads != 0 && o.threads != 256 && o.threads != 512 && o.threads != 1024)
    return fail(PERKS_ERR_INVALID_ARG, "threads must be 0, 256, 512 or 1024");
  if (o.ctas_per_sm < 0 || o.ctas_per_sm > 2) return fail(PERKS_ERR_INVALID_ARG, "ctas_per_sm must be 0, 1 or 2");
  if (o.slicing != 0 && o.slicing != 1 && o.slicing != 2 && o.slicing != 4 && o.slicing != 8 && o.slicing != 16)
    return fail(PERKS_ERR_INVALID_ARG, "slicing must be 0, 1, 2, 4, 8 or 16");
  const DeviceInfo* dev = device_info();
  if (!dev) return PERKS_ERR_NO_DEVICE;

  // validate; cost estimate for the order
  std::vector<double> cost(njobs);
  std::vector<size_t> scratch_bytes(njobs);
  for (int i = 0; i < njobs; i++) {
    const perks_job& J = jobs[i];
    const std::string at = "job " + std::to_string(i) + ": ";
    const bool mixed = J.dtype == PERKS_MIXED;
    if (J.dtype != PERKS_FP32 && J.dtype != PERKS_FP64 && !(mixed && J.kind == PERKS_JOB_CG))
      return fail(PERKS_ERR_INVALID_ARG, at + "dtype (PERKS_MIXED is for CG jobs)");
    const size_t es = J.dtype == PERKS_FP64 ? 8 : 4;
    if (J.kind == PERKS_JOB_STENCIL) {
      if (!batch_shape_ok(J.shape))
        return fail(PERKS_ERR_UNSUPPORTED, at + "batched stencils are 2d5pt, 2ds9pt, 2d9pt and 3d7pt");
      const bool is3d = J.shape == PERKS_3D7PT;
      if (J.h <= 0 || J.wy <= 0 || J.wx <= 0 || J.steps < 0 || (!is3d && J.h != 1))
        return fail(PERKS_ERR_INVALID_ARG, at + "bad stencil size");
      if (!J.d_in || !J.d_out) return fail(PERKS_ERR_INVALID_ARG, at + "NULL field");
      const double cells = double(J.h) * J.wy * J.wx;
      if (cells > 2e9) return fail(PERKS_ERR_UNSUPPORTED, at + "field too large for one CTA");
      cost[i] = cells * std::max(J.steps, 1) * (J.dtype == PERKS_FP64 ? 8.0 : 1.0);
      scratch_bytes[i] = (size_t(cells) * es + 255) & ~size_t(255);
    } else if (J.kind == PERKS_JOB_CG) {
      if (J.n <= 0 || J.nnz < 0 || !J.d_row_ptr || !J.d_col || !J.d_val || !J.d_b || !J.d_x)
        return fail(PERKS_ERR_INVALID_ARG, at + "bad CSR arguments");
      if (J.max_iter < 0 || !(J.tol >= 0)) return fail(PERKS_ERR_INVALID_ARG, at + "bad max_iter or tol");
      cost[i] = double(J.nnz + J.n) * std::sqrt(double(J.n)) * 4.0 * (J.dtype == PERKS_FP64 ? 4.0 : 1.0);
      // FP64/FP32: r, p, Ap; mixed: FP32 r, p, Ap, x_s (the vectors of 64-row
      // multiples, one after another) and the FP32 values
      scratch_bytes[i] = mixed ? ((size_t((J.n + 63) & ~63) * 16 + size_t(J.nnz) * 4 + 255) & ~size_t(255))
                               : 3 * ((size_t((J.n + 63) & ~63) * es + 255) & ~size_t(255));
    } else {
      return fail(PERKS_ERR_INVALID_ARG, at + "unknown job kind");
    }
  }
  perks_batch_plan p = new perks_batch_plan_s();
  p->ctl = wait_ctl();
  p->device = dev->device;
  p->stream = static_cast<cudaStream_t>(o.stream);
  p->njobs = njobs;
  p->order.resize(njobs);
  for (int i = 0; i < njobs; i++) p->order[i] = i;
  std::stable_sort(p->order.begin(), p->order.end(), [&](int a, int b) { return cost[a] > cost[b]; });

  size_t total = 0;
  std::vector<size_t> offs(njobs);
  for (int q = 0; q < njobs; q++) {
    offs[q] = total;
    total += scratch_bytes[p->order[q]];
  }
  auto bail = [&](int rc) {
    plan_free(p);
    return rc;
  };
  cudaError_t e;
  if ((e = cudaMalloc(&p->d_scratch, std::max<size_t>(total, 256))) != cudaSuccess)
    return bail(cuda_fail(e, "cudaMalloc(batch scratch)"));
  if ((e = cudaMalloc(&p->d_jobs, sizeof(BJob) * njobs)) != cudaSuccess) return bail(cuda_fail(e, "cudaMalloc(jobs)"));
  if ((e = cudaMalloc(&p->d_res, sizeof(BRes) * njobs)) != cudaSuccess) return bail(cuda_fail(e, "cudaMalloc(results)"));
  if ((e = cudaMalloc(&p->d_counter, sizeof(unsigned) * (1 + njobs))) != cudaSuccess)
    return bail(cuda_fail(e, "cudaMalloc(counters)"));
  if ((e = cudaEventCreate(&p->e0)) != cudaSuccess || (e = cudaEventCreate(&p->e1)) != cudaSuccess)
    return bail(cuda_fail(e, "cudaEventCreate"));

  std::vector<BJob> table(njobs);
  p->cells_of.assign(njobs, 0);
  for (int q = 0; q < njobs; q++) {
    const perks_job& J = jobs[p->order[q]];
    BJob& B = table[q];
    B = BJob{};
    B.kind = J.kind;
    B.dtype = J.dtype;
    B.scratch = static_cast<unsigned char*>(p->d_scratch) + offs[q];
    if (J.kind == PERKS_JOB_STENCIL) {
      B.shape = J.shape;
      B.h = J.h;
      B.wy = J.wy;
      B.wx = J.wx;
      B.steps = J.steps;
      B.in = J.d_in;
      B.out = J.d_out;
      p->cells_of[q] = (long long)J.h * J.wy * J.wx * (J.dtype == PERKS_FP64 ? 8 : 4);
    } else {
      B.n = J.n;
      B.nnz = J.nnz;
      B.rp = J.d_row_ptr;
      B.ci = J.d_col;
      B.val = J.d_val;
      B.b = J.d_b;
      B.x = J.d_x;
      B.tol = J.tol;
      B.max_iter = J.max_iter;
    }
  }
  if ((e = cudaMemcpy(p->d_jobs, table.data(), sizeof(BJob) * njobs, cudaMemcpyHostToDevice)) != cudaSuccess)
    return bail(cuda_fail(e, "cudaMemcpy(jobs)"));

  // work items: stencil jobs above the balancing unit, total cost /
  // (slicing x SMs), are cut into row slices (at most one per SM, so every
  // slice of a job can be held at once)
  double total_cost = 0.0;
  for (int i = 0; i < njobs; i++) total_cost += cost[i];
  auto build_items = [&](int slicing, int* sliced) {
    const double unit = total_cost / (double(slicing) * dev->sms);
    std::vector<BItem> items;
    *sliced = 0;
    for (int q = 0; q < njobs; q++) {
      const perks_job& J = jobs[p->order[q]];
      int g = 1;
      if (J.kind == PERKS_JOB_STENCIL && J.steps > 0) {
        const int rows = J.h * J.wy;
        g = int(std::min<double>(std::ceil(cost[p->order[q]] / unit), double(std::min(dev->sms, rows))));
        g = std::max(g, 1);
      }
      if (g > 1) ++*sliced;
      const int rows = J.kind == PERKS_JOB_STENCIL ? J.h * J.wy : 0;
      for (int sl = 0; sl < g; sl++)
        items.push_back(BItem{q, sl, g, int((long long)rows * sl / g), int((long long)rows * (sl + 1) / g)});
    }
    return items;
  };
  // room for the finest granularity's items
  size_t max_items = 0;
  for (int f : {1, 2, 4, 8, 16}) {
    int sl = 0;
    max_items = std::max(max_items, build_items(f, &sl).size());
  }
  if ((e = cudaMalloc(&p->d_items, sizeof(BItem) * max_items)) != cudaSuccess)
    return bail(cuda_fail(e, "cudaMalloc(items)"));
  auto use_items = [&](int slicing) -> cudaError_t {
    const std::vector<BItem> items = build_items(slicing, &p->sliced);
    p->nitems = int(items.size());
    p->slicing = slicing;
    return cudaMemcpy(p->d_items, items.data(), sizeof(BItem) * items.size(), cudaMemcpyHostToDevice);
  };
  if ((e = use_items(o.slicing ? o.slicing : 2)) != cudaSuccess) return bail(cuda_fail(e, "cudaMemcpy(items)"));

  // launch shape: the caller's, or the fastest candidate of one timed run each
  std::vector<std::pair<int, int>> cand;
  for (int t : {256, 512, 1024})
    for (int c : {1, 2})
      if ((o.threads == 0 || o.threads == t) && (o.ctas_per_sm == 0 || o.ctas_per_sm == c) && t * c <= 1024)
        cand.push_back({t, c});  // <= 1024 threads per SM: 64 registers per thread fit
  if (cand.empty()) return bail(fail(PERKS_ERR_INVALID_ARG, "threads x ctas_per_sm must be <= 1024"));
  // every CTA of the grid must be resident (job barriers wait for each other)
  {
    std::vector<std::pair<int, int>> fit;
    for (auto& tc : cand) {
      int nb = 0;
      const unsigned sm = smem_for(dev, tc.second);
      if ((e = cudaFuncSetAttribute(batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sm))) != cudaSuccess)
        return bail(cuda_fail(e, "cudaFuncSetAttribute(batch)"));
      if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_kernel, tc.first, sm)) != cudaSuccess)
        return bail(cuda_fail(e, "occupancy(batch)"));
      if (nb >= tc.second) fit.push_back(tc);
    }
    cand.swap(fit);
    if (cand.empty()) return bail(fail(PERKS_ERR_LAUNCH, "batch launch shape does not fit an SM"));
  }
  float best = 1e30f;
  if (cand.size() > 1) {  // warm-up (module load, cold L2) before the timed candidates
    float ms = 0.f;
    int rc = launch_once(p, p->stream, cand[0].first, cand[0].second, smem_for(dev, cand[0].second), &ms);
    if (rc != PERKS_OK) return bail(rc);
  }
  if (cand.size() == 1) {  // a fixed launch shape: nothing to time
    p->threads = cand[0].first;
    p->ctas_per_sm = cand[0].second;
    best = 0.f;
  } else {
    for (auto& tc : cand) {
      float ms = 0.f;
      int rc = launch_once(p, p->stream, tc.first, tc.second, smem_for(dev, tc.second), &ms);
      if (rc != PERKS_OK) return bail(rc);
      if (ms < best) {
        best = ms;
        p->threads = tc.first;
        p->ctas_per_sm = tc.second;
      }
    }
  }
  // work granularity: the caller's, or (tuning) the fastest of 2, 4, 8 and 16
  // at the chosen launch shape (1, measured twice as slow on the benchmark's
  // workload, only when asked for)
  if (o.slicing == 0) {
    int best_f = p->slicing;
    if (best == 0.f) {  // fixed launch shape: time the default granularity first
      float ms = 0.f;
      int rc = launch_once(p, p->stream, p->threads, p->ctas_per_sm, smem_for(dev, p->ctas_per_sm), &ms);
      if (rc != PERKS_OK) return bail(rc);
      best = ms;
    }
    for (int f : {4, 8, 16}) {
      if ((e = use_items(f)) != cudaSuccess) return bail(cuda_fail(e, "cudaMemcpy(items)"));
      float ms = 0.f;
      int rc = launch_once(p, p->stream, p->threads, p->ctas_per_sm, smem_for(dev, p->ctas_per_sm), &ms);
      if (rc != PERKS_OK) return bail(rc);
      if (ms < best) {
        best = ms;
        best_f = f;
      }
    }
    if ((e = use_items(best_f)) != cudaSuccess) return bail(cuda_fail(e, "cudaMemcpy(items)"));
  }
  p->tuned = cand.size() > 1 || o.slicing == 0;
  p->smem = smem_for(dev, p->ctas_per_sm);
  p->grid = dev->sms * p->ctas_per_sm;
  p->resident = 0;
  {
    std::vector<int> slices(njobs, 1);
    int sl_count = 0;
    for (const BItem& it : build_items(p->slicing, &sl_count)) slices[it.job] = it.nslices;
    for (int q = 0; q < njobs; q++)
      if (slices[q] == 1 && p->cells_of[q] > 0 && 2 * p->cells_of[q] <= (long long)p->smem) p->resident++;
  }

  // the run as a graph: reset the queue counter, launch
  if ((e = cudaFuncSetAttribute(batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(p->smem))) != cudaSuccess)
    return bail(cuda_fail(e, "cudaFuncSetAttribute(batch)"));
  cudaStream_t cs;
  if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess)
    return bail(cuda_fail(e, "cudaStreamCreate"));
  e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    cudaMemsetAsync(p->d_counter, 0, sizeof(unsigned) * (1 + p->njobs), cs);
    batch_kernel<<<p->grid, p->threads, p->smem, cs>>>(p->d_jobs, p->d_items, p->nitems, p->d_res, p->d_counter,
                                                       p->smem, p->ctl);
    e = cudaStreamEndCapture(cs, &p->graph);
  }
  cudaStreamDestroy(cs);
  if (e != cudaSuccess) return bail(cuda_fail(e, "graph capture (batch)"));
  if ((e = cudaGraphInstantiate(&p->exec, p->graph, 0)) != cudaSuccess)
    return bail(cuda_fail(e, "cudaGraphInstantiate(batch)"));
  p->last_ms = best;
  *out = p;
  return PERKS_OK;
}

int perks_batch_plan_run(perks_batch_plan p, void* stream, perks_batch_stats* st) {
  if (!p) return fail(PERKS_ERR_INVALID_ARG, "plan is NULL");
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : p->stream;
  PERKS_CUDA(cudaEventRecord(p->e0, s));
  PERKS_CUDA(cudaGraphLaunch(p->exec, s));
  PERKS_CUDA(cudaEventRecord(p->e1, s));
  PERKS_CUDA(cudaEventSynchronize(p->e1));
  count_launch(1);
  float ms = 0.f;
  PERKS_CUDA(cudaEventElapsedTime(&ms, p->e0, p->e1));
  p->last_ms = ms;
  if (st) {
    st->ms = ms;
    st->threads = p->threads;
    st->ctas_per_sm = p->ctas_per_sm;
    st->grid = p->grid;
    st->resident_jobs = p->resident;
    st->tuned = p->tuned;
    st->sliced_jobs = p->sliced;
    st->slicing = p->slicing;
  }
  return PERKS_OK;
}

int perks_batch_plan_results(perks_batch_plan p, perks_job_result* results) {
  if (!p || !results) return fail(PERKS_ERR_INVALID_ARG, "plan or results is NULL");
  std::vector<BRes> r(p->njobs);
  PERKS_CUDA(cudaMemcpy(r.data(), p->d_res, sizeof(BRes) * p->njobs, cudaMemcpyDeviceToHost));
  for (int q = 0; q < p->njobs; q++) {
    perks_job_result& o = results[p->order[q]];
    o.iterations = r[q].iterations;
    o.status = r[q].status;
    o.rel_res = r[q].rel_res;
  }
  return PERKS_OK;
}

void perks_batch_plan_destroy(perks_batch_plan p) { plan_free(p); }

}  // extern "C"
