// FMA throughput probe: the arithmetic roofline of the FP64 stencils and CG.
//
// On GB300 FP64 runs at a small fraction of the FP32 rate, so FP64 stencils
// and FP64 CG are bound by the FP64 pipe rather than by HBM. This measures
// that pipe (and the FP32 one) with the throughput form of the standard
// micro-benchmark: every thread runs eight independent FMA chains (enough
// independent work per warp to hide the FMA latency), four 256-thread CTAs
// per SM, one launch long enough (~0.1 s) for launch overhead to vanish. The
// chains' results feed a never-true test that keeps the compiler from
// removing them.
#include <cuda_runtime.h>
#include "runtime.cuh"

namespace perks {

template <class T>
__global__ void __launch_bounds__(256) fma_chains(T* out, int iters, T a, T b) {
  T v[8];
#pragma unroll
  for (int k = 0; k < 8; k++) v[k] = T(threadIdx.x + k) * T(0.001);
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++) v[k] = fma(v[k], a, b);
  }
  T s = T(0);
#pragma unroll
  for (int k = 0; k < 8; k++) s += v[k];
  if (s == T(-12345)) out[blockIdx.x] = s;
}

template <class T>
static int probe(int iters, double* fma_per_s, double* ms_out) {
  const DeviceInfo* dev = device_info();
  if (!dev) return PERKS_ERR_NO_DEVICE;
  int st = PERKS_OK;
  const int grid = dev->sms * 4, threads = 256;
  T* out = static_cast<T*>(workspace(kWsCgScalar, sizeof(T) * grid, &st));
  if (!out) return st;
  // a = 1 - 2^-20, b = 2^-10: the chains converge to b / (1 - a), no overflow
  const T a = T(1) - T(1.0 / 1048576.0), b = T(1.0 / 1024.0);
  fma_chains<T><<<grid, threads>>>(out, 64, a, b);  // warm-up
  PERKS_CUDA(cudaGetLastError());
  cudaEvent_t e0, e1;
  PERKS_CUDA(cudaEventCreate(&e0));
  PERKS_CUDA(cudaEventCreate(&e1));
  PERKS_CUDA(cudaEventRecord(e0));
  fma_chains<T><<<grid, threads>>>(out, iters, a, b);
  PERKS_CUDA(cudaEventRecord(e1));
  PERKS_CUDA(cudaEventSynchronize(e1));
  count_launch(2);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *fma_per_s = double(grid) * threads * 8.0 * iters / (double(ms) * 1e-3);
  if (ms_out) *ms_out = ms;
  return PERKS_OK;
}

}  // namespace perks

extern "C" int perks_probe_fma_peak(int dtype, double* fma_per_s, double* ms) {
  if (!fma_per_s) return perks::fail(PERKS_ERR_INVALID_ARG, "fma_per_s is NULL");
  if (dtype == PERKS_FP64) return perks::probe<double>(1 << 16, fma_per_s, ms);
  if (dtype == PERKS_FP32) return perks::probe<float>(1 << 21, fma_per_s, ms);
  return perks::fail(PERKS_ERR_INVALID_ARG, "dtype must be PERKS_FP32 or PERKS_FP64");
}
