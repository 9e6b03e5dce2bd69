// Correctly rounded division by a small positive integer constant b, as
// IEEE-754 `x / b` (round to nearest even), in a few branch-free operations.
//
//   q0 = RN(x * r)            with r = RN(1/b)
//   e  = fma(-q0, b, x)       exact remainder
//   q1 = fma(e, r, q0)        Markstein's correction (P. Markstein, "Computation
//                             of elementary functions on the IBM RISC System/6000",
//                             IBM J. R&D 34(1), 1990; Muller et al., Handbook of
//                             Floating-Point Arithmetic, ch. 4)
//
// For normal quotients q1 is the correctly rounded quotient. For quotients
// on the subnormal grid (spacing g) q0 is within one grid step of x/b, and
// x/b is either exactly on a rounding midpoint or at least g/(2b) away from
// one, far more than the error of e*r; so q1 rounds like x/b except at exact
// midpoints. Those only occur for even b (x/b = (k + 1/2) g when x is an odd
// multiple of (b/2) g); there the remainder is exactly (b/2) g and the even
// neighbour is chosen explicitly. A remainder of exactly (b/2) g is only
// possible while ulp(q0) = g (for larger quotients the remainder is a multiple
// of 2g and b/2 is odd), so the test needs no magnitude check. The quotient
// takes the sign of x, which fixes the sign of zero results.
//
// For even b with b*RN(1/b) > 1 (b = 118 in float) the midpoint fix needs no
// second candidate: the fma then always lands on the neighbour away from q0,
// which is kept when its last bit is even and replaced by q0 otherwise.
//
// FIN = 1 selects an equivalent form without the sign transfer: the remainder
// is formed negated, e' = fma(q0, b, -x), and q1 = fma(e', -r, q0). Then for
// x = -0 (q0 = -0, e' = +0) the correction adds e' * -r = -0 to -0, and a
// quotient that underflows keeps the sign of the nonzero product e' * -r, so
// zero results already carry the sign of x. Both forms give identical
// results; which one ptxas schedules better differs between stencil shapes,
// so the 2D kernels take FIN from their measured tuning table.
//
// FIN = 2 is the FIN = 1 form with the finish taken out of the common path:
// div_const_q1 returns q1 and the negated remainder e', and div_needs_finish
// tells whether any of a set of remainders is exactly (b/2) g (a midpoint on
// the subnormal grid; even b only) or NaN (x infinite or NaN). Where neither
// holds, the finish of FIN = 1 keeps q1, so q1 is the result. The 2D kernels
// test a whole warp row with one vote and redo the row with the full finish
// only when a flag is set; the zero fields that long runs decay to stay on
// the short path (e' = 0).
//
// FIN = 3 is the FIN = 1 form with a branch-free short finish: q0 is kept
// where |e'| is (b/2) g or unordered and q1 is odd, else q1 (odd b: q0 where
// e' is NaN). For x infinite, e' and q1 are NaN and GB300 arithmetic returns
// its NaNs with every mantissa bit set, so q1 counts as odd and q0 = x/b = x
// is kept; the all-inputs check below covers those inputs too.
//
// The float version (all forms, per element and on packed pairs) is checked
// against CUDA's IEEE division for all 2^32 inputs with b = 118 and 159
// (perks_debug_div_check: zero mismatches, signs of zero included), the
// double version through the bit-exact stencil tests on subnormal, tiny,
// huge, infinite and NaN fields.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "f32x2.cuh"

namespace perks {

// The steps after q0, e and q1: the midpoint fix and the sign/non-finite
// handling, for one element.
template <int B>
__device__ __forceinline__ float div_finish(float x, float q0, float e, float q1) {
  if constexpr ((B & 1) == 0) {
    constexpr float half = float(B / 2) * 0x1p-149f;  // b/2 subnormal steps
    const bool tie = fabsf(e) == half;
    // At a midpoint e*r = +-(g/2)(b*r) exactly, so with b*RN(1/b) > 1 the fma
    // lands on the neighbour away from q0: keep it if even, else take q0.
    constexpr bool far_on_tie = double(B) * double(1.0f / float(B)) > 1.0;
    if constexpr (far_on_tie) {
      q1 = (tie && (__float_as_uint(q1) & 1u)) ? q0 : q1;
    } else {
      const float up = __fadd_rn(q0, copysignf(0x1p-149f, e));
      q1 = tie ? ((__float_as_uint(q0) & 1u) ? up : q0) : q1;
    }
  }
  return isfinite(q0) ? copysignf(q1, x) : q0;
}

// FIN = 1: e' = -e and q1 from it; zero results need no sign transfer.
template <int B>
__device__ __forceinline__ float div_finish_neg(float q0, float ep, float q1) {
  bool keep_q0 = !isfinite(q0);  // x infinite or NaN (e' is NaN)
  if constexpr ((B & 1) == 0) {
    constexpr float half = float(B / 2) * 0x1p-149f;
    const bool tie = fabsf(ep) == half;
    constexpr bool far_on_tie = double(B) * double(1.0f / float(B)) > 1.0;
    if constexpr (far_on_tie) {
      keep_q0 = keep_q0 || (tie && (__float_as_uint(q1) & 1u));
    } else {
      const float up = __fsub_rn(q0, copysignf(0x1p-149f, ep));  // neighbour towards x/b
      q1 = tie ? ((__float_as_uint(q0) & 1u) ? up : q0) : q1;
    }
  }
  return keep_q0 ? q0 : q1;
}

// FIN = 3: the short finish of one element.
template <int B>
__device__ __forceinline__ float div_short_finish(float q0, float ep, float q1) {
  float q;
  if constexpr ((B & 1) == 0) {
    constexpr float half = float(B / 2) * 0x1p-149f;
    asm("{\n\t.reg .pred o, p;\n\t.reg .b32 t;\n\t.reg .f32 a;\n\t"
        "and.b32 t, %2, 1;\n\tsetp.ne.b32 o, t, 0;\n\t"
        "abs.f32 a, %3;\n\tsetp.equ.and.f32 p, a, %4, o;\n\t"
        "selp.f32 %0, %1, %2, p;\n\t}"
        : "=f"(q)
        : "f"(q0), "f"(q1), "f"(ep), "f"(half));
  } else {
    asm("{\n\t.reg .pred p;\n\tsetp.nan.f32 p, %3, %3;\n\tselp.f32 %0, %1, %2, p;\n\t}"
        : "=f"(q)
        : "f"(q0), "f"(q1), "f"(ep));
  }
  return q;
}

template <int B, int FIN = 0>
__device__ __forceinline__ float div_const(float x) {
  constexpr float b = float(B);
  const float r = __fdiv_rn(1.0f, b);  // folded to a constant
  const float q0 = __fmul_rn(x, r);
  if constexpr (FIN == 3) {
    const float ep = __fmaf_rn(q0, b, -x);
    return div_short_finish<B>(q0, ep, __fmaf_rn(ep, -r, q0));
  } else if constexpr (FIN != 0) {
    const float ep = __fmaf_rn(q0, b, -x);
    return div_finish_neg<B>(q0, ep, __fmaf_rn(ep, -r, q0));
  } else {
    const float e = __fmaf_rn(-q0, b, x);
    const float q1 = __fmaf_rn(e, r, q0);
    return div_finish<B>(x, q0, e, q1);
  }
}

// Two elements at once: the three rounding steps as packed FP32 pairs (each
// half an IEEE round-to-nearest operation, so each element's result is the
// one above), the finish per element.
template <int B, int FIN = 0>
__device__ __forceinline__ F2 div_const(F2 x) {
  constexpr float b = float(B);
  const float r = __fdiv_rn(1.0f, b);
  const F2 q0 = RN<F2>::mul(x, F2(r));
  float q0a, q0b, ea, eb, q1a, q1b;
  q0.unpack(q0a, q0b);
  if constexpr (FIN != 0) {
    const F2 ep = RN<F2>::fma(q0, F2(b), RN<F2>::mul(x, F2(-1.0f)));  // q0*b - x
    const F2 q1 = RN<F2>::fma(ep, F2(-r), q0);
    ep.unpack(ea, eb);
    q1.unpack(q1a, q1b);
    if constexpr (FIN == 3)
      return F2::pack(div_short_finish<B>(q0a, ea, q1a), div_short_finish<B>(q0b, eb, q1b));
    return F2::pack(div_finish_neg<B>(q0a, ea, q1a), div_finish_neg<B>(q0b, eb, q1b));
  } else {
    const F2 e = RN<F2>::fma(q0, F2(-b), x);  // -q0*b + x, the negation exact
    const F2 q1 = RN<F2>::fma(e, F2(r), q0);
    float xa, xb;
    x.unpack(xa, xb);
    e.unpack(ea, eb);
    q1.unpack(q1a, q1b);
    return F2::pack(div_finish<B>(xa, q0a, ea, q1a), div_finish<B>(xb, q0b, eb, q1b));
  }
}

// FIN = 2, short path: q1 and e' of the negated-remainder form.
template <int B>
__device__ __forceinline__ float div_const_q1(float x, float& ep) {
  constexpr float b = float(B);
  const float r = __fdiv_rn(1.0f, b);
  const float q0 = __fmul_rn(x, r);
  ep = __fmaf_rn(q0, b, -x);
  return __fmaf_rn(ep, -r, q0);
}
template <int B>
__device__ __forceinline__ F2 div_const_q1(F2 x, F2& ep) {
  constexpr float b = float(B);
  const float r = __fdiv_rn(1.0f, b);
  const F2 q0 = RN<F2>::mul(x, F2(r));
  ep = RN<F2>::fma(q0, F2(b), RN<F2>::mul(x, F2(-1.0f)));  // q0*b - x
  return RN<F2>::fma(ep, F2(-r), q0);
}

// Whether the finish could change q1 for any of four remainders e': |e'| equal
// to (b/2) g or unordered (setp.equ), for odd b only NaN. One predicate chain.
template <int B>
__device__ __forceinline__ unsigned div_needs_finish4(float e0, float e1, float e2, float e3) {
  unsigned f;
  if constexpr ((B & 1) == 0) {
    constexpr float half = float(B / 2) * 0x1p-149f;
    asm("{\n\t.reg .pred p;\n\t.reg .f32 a;\n\t"
        "abs.f32 a, %1;\n\tsetp.equ.f32 p, a, %5;\n\t"
        "abs.f32 a, %2;\n\tsetp.equ.or.f32 p, a, %5, p;\n\t"
        "abs.f32 a, %3;\n\tsetp.equ.or.f32 p, a, %5, p;\n\t"
        "abs.f32 a, %4;\n\tsetp.equ.or.f32 p, a, %5, p;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(f)
        : "f"(e0), "f"(e1), "f"(e2), "f"(e3), "f"(half));
  } else {
    asm("{\n\t.reg .pred p;\n\t"
        "setp.nan.f32 p, %1, %2;\n\t"
        "setp.nan.or.f32 p, %3, %4, p;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(f)
        : "f"(e0), "f"(e1), "f"(e2), "f"(e3));
  }
  return f;
}
template <int B, int N>
__device__ __forceinline__ unsigned div_needs_finish(const float (&e)[N]) {
  static_assert(N % 4 == 0, "remainders in groups of four");
  unsigned f = 0;
#pragma unroll
  for (int i = 0; i < N; i += 4) f |= div_needs_finish4<B>(e[i], e[i + 1], e[i + 2], e[i + 3]);
  return f;
}

template <int B, int FIN = 0>
__device__ __forceinline__ double div_const(double x) {
  // FP64 arithmetic is scarce on this GPU: the tie and finiteness
  // tests and the sign transfer use integer operations on the bit patterns.
  constexpr double b = double(B);
  constexpr long long kAbs = 0x7fffffffffffffffll, kExp = 0x7ff0000000000000ll, kSign = (long long)0x8000000000000000ull;
  const double r = __ddiv_rn(1.0, b);
  const double q0 = __dmul_rn(x, r);
  if constexpr (FIN != 0) {  // negated remainder: no sign transfer
    const double ep = __fma_rn(q0, b, -x);
    double q1 = __fma_rn(ep, -r, q0);
    const long long q0b = __double_as_longlong(q0);
    if constexpr ((B & 1) == 0) {
      constexpr double half = double(B / 2) * 0x1p-1074;
      if ((__double_as_longlong(ep) & kAbs) == __double_as_longlong(half)) {
        const double up = __dsub_rn(q0, copysign(0x1p-1074, ep));
        q1 = (q0b & 1ll) ? up : q0;
      }
    }
    return ((q0b & kExp) == kExp) ? q0 : q1;
  }
  const double e = __fma_rn(-q0, b, x);
  double q1 = __fma_rn(e, r, q0);
  const long long xb = __double_as_longlong(x), q0b = __double_as_longlong(q0);
  if constexpr ((B & 1) == 0) {
    constexpr double half = double(B / 2) * 0x1p-1074;
    const long long half_bits = __double_as_longlong(half);
    const bool tie = (__double_as_longlong(e) & kAbs) == half_bits;
    if (tie) {  // rare: exact midpoint on the subnormal grid, take the even neighbour
      const double up = __dadd_rn(q0, copysign(0x1p-1074, e));
      q1 = (q0b & 1ll) ? up : q0;
    }
  }
  if ((q0b & kExp) == kExp) return q0;  // x infinite or NaN
  return __longlong_as_double((__double_as_longlong(q1) & kAbs) | (xb & kSign));
}

}  // namespace perks
