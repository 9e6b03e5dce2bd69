// Check of the exact constant division (divconst.cuh) over every FP32 input:
// each of the 2^32 bit patterns divided by the constant in both device forms
// the kernels use (per element, and on packed pairs), compared bit for bit
// with CUDA's IEEE round-to-nearest division (__fdiv_rn); any NaN equals any
// NaN. Finish forms 0 and 1 run the full finish, form 3 the branch-free
// short one; form 2 takes q1 wherever the flag test of its pair (or element)
// is clear and the full finish elsewhere, which checks that a clear flag
// always means a correct q1. A few milliseconds per divisor and finish form
// on one GPU.
#include <cuda_runtime.h>
#include "divconst.cuh"
#include "runtime.cuh"

namespace perks {

__device__ __forceinline__ bool same_result(float a, float b) {
  return (__float_as_uint(a) == __float_as_uint(b)) || (a != a && b != b);
}

template <int B, int FIN>
__global__ void __launch_bounds__(256) div_check_kernel(unsigned long long* bad, unsigned* first) {
  const unsigned long long stride = 2ull * gridDim.x * blockDim.x;
  unsigned long long nb[2] = {0, 0};
  for (unsigned long long i = 2ull * (blockIdx.x * blockDim.x + threadIdx.x); i < (1ull << 32); i += stride) {
    const float x[2] = {__uint_as_float(unsigned(i)), __uint_as_float(unsigned(i + 1))};
    float g[2][2];
    if constexpr (FIN == 2) {
#pragma unroll
      for (int j = 0; j < 2; j++) {
        float ep;
        const float q = div_const_q1<B>(x[j], ep);
        g[0][j] = div_needs_finish4<B>(ep, ep, ep, ep) ? div_const<B, 1>(x[j]) : q;
      }
      F2 ep;
      const F2 q = div_const_q1<B>(F2::pack(x[0], x[1]), ep);
      float ea, eb;
      ep.unpack(ea, eb);
      (div_needs_finish4<B>(ea, eb, ea, eb) ? div_const<B, 1>(F2::pack(x[0], x[1])) : q).unpack(g[1][0], g[1][1]);
    } else {
#pragma unroll
      for (int j = 0; j < 2; j++) g[0][j] = div_const<B, FIN>(x[j]);
      div_const<B, FIN>(F2::pack(x[0], x[1])).unpack(g[1][0], g[1][1]);
    }
#pragma unroll
    for (int j = 0; j < 2; j++) {
      const float ref = __fdiv_rn(x[j], float(B));
#pragma unroll
      for (int v = 0; v < 2; v++) {
        if (!same_result(g[v][j], ref)) {
          nb[v]++;
          atomicMin(&first[v], unsigned(i + j));
        }
      }
    }
  }
#pragma unroll
  for (int v = 0; v < 2; v++)
    if (nb[v]) atomicAdd(&bad[v], nb[v]);
}

template <int B, int FIN>
static int run_check(long long* mismatches, unsigned* first_bad) {
  const DeviceInfo* dev = device_info();
  if (!dev) return PERKS_ERR_NO_DEVICE;
  int st = PERKS_OK;
  void* ws = workspace(kWsCgScalar, 64, &st);
  if (!ws) return st;
  unsigned long long* bad = static_cast<unsigned long long*>(ws);
  unsigned* first = reinterpret_cast<unsigned*>(bad + 2);
  PERKS_CUDA(cudaMemset(bad, 0, 2 * sizeof(unsigned long long)));
  PERKS_CUDA(cudaMemset(first, 0xff, 2 * sizeof(unsigned)));
  div_check_kernel<B, FIN><<<dev->sms * 8, 256>>>(bad, first);
  PERKS_CUDA(cudaGetLastError());
  count_launch(1);
  unsigned long long hb[2];
  unsigned hf[2];
  PERKS_CUDA(cudaMemcpy(hb, bad, sizeof(hb), cudaMemcpyDeviceToHost));
  PERKS_CUDA(cudaMemcpy(hf, first, sizeof(hf), cudaMemcpyDeviceToHost));
  for (int v = 0; v < 2; v++) {
    mismatches[v] = (long long)hb[v];
    if (first_bad) first_bad[v] = hf[v];
  }
  return PERKS_OK;
}

}  // namespace perks

extern "C" int perks_debug_div_check(int divisor, int form, long long* mismatches, unsigned* first_bad) {
  using namespace perks;
  if (!mismatches) return fail(PERKS_ERR_INVALID_ARG, "mismatches is NULL");
  if (form < 0 || form > 3) return fail(PERKS_ERR_INVALID_ARG, "form must be 0, 1, 2 or 3");
  using Fn = int (*)(long long*, unsigned*);
  static const Fn k118[4] = {run_check<118, 0>, run_check<118, 1>, run_check<118, 2>, run_check<118, 3>};
  static const Fn k159[4] = {run_check<159, 0>, run_check<159, 1>, run_check<159, 2>, run_check<159, 3>};
  if (divisor == 118) return k118[form](mismatches, first_bad);
  if (divisor == 159) return k159[form](mismatches, first_bad);
  return fail(PERKS_ERR_INVALID_ARG, "divisor must be 118 or 159");
}
