// Correctly rounded division by a small positive integer constant b, as
// IEEE-754 `x / b` (round to nearest even), without the general division
// sequence.
//
// Normal results: q0 = RN(x * r) with r = RN(1/b), e = fma(-q0, b, x) (exact),
// q1 = fma(e, r, q0) — Markstein's correction (P. Markstein, "Computation of
// elementary functions on the IBM RISC System/6000", IBM J. R&D 34(1), 1990;
// also Muller et al., Handbook of Floating-Point Arithmetic, ch. 4).
// Results that are subnormal (or in the binade just above) are computed
// exactly in integer arithmetic: |x| is an integer multiple M of the smallest
// subnormal, so the quotient is RN_even(M / b) of those units.
//
// The float version for b = 118 and b = 159 is checked against IEEE division
// for all 2^32 inputs on the CPU (oracle-side check) and both
// versions against __fdiv_rn / __ddiv_rn on the GPU (tests/test_divconst_gpu.py).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace perks {

template <int B>
struct DivThreshold;  // below it the quotient is at most 2^-125 (float) / 2^-1021 (double)
template <>
struct DivThreshold<118> {
  static constexpr float f = 0x1p-119f;
  static constexpr double d = 0x1p-1015;
};
template <>
struct DivThreshold<159> {
  static constexpr float f = 0x1p-118f;
  static constexpr double d = 0x1p-1014;
};

template <int B>
__device__ __forceinline__ float div_const(float x) {
  constexpr float b = float(B);
  const float r = __fdiv_rn(1.0f, b);  // folded to a constant
  const float ax = fabsf(x);
  if (ax < DivThreshold<B>::f) {
    const uint32_t M = __float2uint_rz(__fmul_rn(__fmul_rn(ax, 0x1p126f), 0x1p23f));
    uint32_t q = M / uint32_t(B);
    const uint32_t rem = M - q * uint32_t(B);
    if (2u * rem > uint32_t(B) || (2u * rem == uint32_t(B) && (q & 1u))) q++;
    const float res = __fmul_rn(__fmul_rn(__uint2float_rn(q), 0x1p-23f), 0x1p-126f);
    return copysignf(res, x);
  }
  const float q0 = __fmul_rn(x, r);
  const float e = __fmaf_rn(-q0, b, x);
  const float q1 = __fmaf_rn(e, r, q0);
  return isfinite(q0) ? q1 : q0;
}

template <int B>
__device__ __forceinline__ double div_const(double x) {
  constexpr double b = double(B);
  const double r = __ddiv_rn(1.0, b);
  const double ax = fabs(x);
  if (ax < DivThreshold<B>::d) {
    // |x| = M * 2^-1074 with M < 2^60
    const uint64_t M = uint64_t(__double2ull_rz(__dmul_rn(__dmul_rn(ax, 0x1p1022), 0x1p52)));
    uint64_t q = M / uint64_t(B);
    const uint64_t rem = M - q * uint64_t(B);
    if (2ull * rem > uint64_t(B) || (2ull * rem == uint64_t(B) && (q & 1ull))) q++;
    const double res = __dmul_rn(__dmul_rn(__ull2double_rn(q), 0x1p-52), 0x1p-1022);
    return copysign(res, x);
  }
  const double q0 = __dmul_rn(x, r);
  const double e = __fma_rn(-q0, b, x);
  const double q1 = __fma_rn(e, r, q0);
  return isfinite(q0) ? q1 : q0;
}

}  // namespace perks
