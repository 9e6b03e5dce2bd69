// Packed FP32 pairs for sm_103a: add/mul/fma.rn.f32x2 issue one instruction
// for two independent IEEE round-to-nearest FP32 operations. The reference
// evaluation order is a fixed sequence of separately rounded products and
// sums, so two adjacent cells can go through it together, halving the
// arithmetic instructions without changing any result bit.
//
// ptxas fuses a packed mul.rn followed by a packed add.rn into one fma even
// though both carry explicit rounding (measured on GB300: a third of the pairs
// then differ from separately rounded results), and it also treats fma(a, b,
// -0) as a product. So a sum after a product is written as fma(p, one, acc)
// with `one` = 1.0 read from the kernel parameters: RN(p*1 + acc) = RN(p + acc),
// and ptxas cannot see a product to fuse. RN<F2> has no add for that reason.
#pragma once
#include <cuda_runtime.h>

namespace perks {

struct F2 {
  unsigned long long v;
  F2() = default;
  __device__ __forceinline__ explicit F2(float a) { asm("mov.b64 %0, {%1, %1};" : "=l"(v) : "f"(a)); }
  __device__ __forceinline__ explicit F2(int a) : F2(float(a)) {}
  static __device__ __forceinline__ F2 pack(float a, float b) {
    F2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(a), "f"(b));
    return r;
  }
  __device__ __forceinline__ void unpack(float& a, float& b) const {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
  }
};

template <class T>
struct RN;
template <>
struct RN<F2> {
  static __device__ __forceinline__ F2 mul(F2 a, F2 b) {
    F2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
  }
  static __device__ __forceinline__ F2 fma(F2 a, F2 b, F2 c) {
    F2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return r;
  }
};

}  // namespace perks
