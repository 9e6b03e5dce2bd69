// Stencil shapes of the PERKS reference and their per-point arithmetic.
//
// Two evaluation orders are provided for every shape:
//  * Ref  — the reference CPU gold order, operation by operation, with
//           rounding intrinsics so that nvcc cannot contract a multiply and an
//           add into an FMA, and the final division by 118 / 159 done by the
//           exact constant-division helper (divconst.cuh). Results are bit-identical to the reference's CPU
//           code (stencil/2dstencil/<shape>/jacobi_gold_gen.cpp,
//           stencil/3dstencil/<shape>/<shape>_gold_gen.cpp), including the
//           mid-expression promotion to double that the reference's double
//           literals cause in its float build.
//  * Fast — the same weights folded into one coefficient per point
//           (w/118, w/159) and an FMA chain in the storage type.
//
// A point functor `u(dz, dy, dx)` returns the input value of a neighbour,
// with any domain-edge clamping already applied by the caller.
#pragma once
#include <cuda_runtime.h>
#include "../../include/perks.h"
#include "divconst.cuh"

namespace perks {

template <int SHAPE>
struct ShapeInfo;
#define PERKS_SHAPE_INFO(S, HALO, IS3D, ISBOX) \
  template <>                                  \
  struct ShapeInfo<S> {                        \
    static constexpr int H = HALO;             \
    static constexpr bool is3d = IS3D;         \
    static constexpr bool box = ISBOX;         \
  };
PERKS_SHAPE_INFO(PERKS_2D5PT, 1, false, false)
PERKS_SHAPE_INFO(PERKS_2DS9PT, 2, false, false)
PERKS_SHAPE_INFO(PERKS_2D13PT, 3, false, false)
PERKS_SHAPE_INFO(PERKS_2D17PT, 4, false, false)
PERKS_SHAPE_INFO(PERKS_2D21PT, 5, false, false)
PERKS_SHAPE_INFO(PERKS_2DS25PT, 6, false, false)
PERKS_SHAPE_INFO(PERKS_2D9PT, 1, false, true)
PERKS_SHAPE_INFO(PERKS_2D25PT, 2, false, true)
PERKS_SHAPE_INFO(PERKS_3D7PT, 1, true, false)
PERKS_SHAPE_INFO(PERKS_3D13PT, 2, true, false)
PERKS_SHAPE_INFO(PERKS_3D17PT, 1, true, true)
PERKS_SHAPE_INFO(PERKS_3D27PT, 1, true, true)
PERKS_SHAPE_INFO(PERKS_POISSON, 1, true, true)
#undef PERKS_SHAPE_INFO

// Correctly rounded arithmetic that the compiler may not fuse.
template <>
struct RN<float> {
  static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
  static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
};
template <>
struct RN<double> {
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
};

// 2D star weights by distance (index 0 = nearest): south, west, east, north;
// centre 15, divisor 118 (stencil/2dstencil/2ds25pt/jacobi_gold_gen.cpp:55-86
// holds the full set; lower orders use prefixes).
__host__ __device__ constexpr int star_s(int h) { return h == 0 ? 5 : h == 1 ? 7 : h == 2 ? 5 : h == 3 ? 1 : h == 4 ? 6 : 2; }
__host__ __device__ constexpr int star_w(int h) { return h == 0 ? 12 : h == 1 ? 9 : h == 2 ? 3 : h == 3 ? 2 : h == 4 ? 5 : 6; }
__host__ __device__ constexpr int star_e(int h) { return h == 0 ? 12 : h == 1 ? 9 : h == 2 ? 3 : h == 3 ? 3 : h == 4 ? 4 : 6; }
__host__ __device__ constexpr int star_n(int h) { return h == 0 ? 5 : h == 1 ? 7 : h == 2 ? 5 : h == 3 ? 4 : h == 4 ? 3 : 2; }
// 2D box weights [row from south][column from west]
// (2d9pt/jacobi_gold_gen.cpp:33-36, 2d25pt/jacobi_gold_gen.cpp:35-40).
__host__ __device__ constexpr int box9_w(int r, int c) {
  return (r == 0) ? (c == 0 ? 7 : c == 1 ? 5 : 9) : (r == 1) ? (c == 1 ? 15 : 12) : (c == 0 ? 9 : c == 1 ? 5 : 7);
}
__host__ __device__ constexpr int box25_w(int r, int c) {
  return r == 0 ? 1 + c
       : r == 1 ? (c == 2 ? 5 : c == 4 ? 6 : 7)
       : r == 2 ? (c == 0 ? 8 : c == 2 ? 15 : 12)
       : r == 3 ? (c == 0 || c == 1 ? 9 : c == 2 ? 5 : c == 3 ? 7 : 15)
       : 10 + c;
}
// 3d27pt coefficients [plane b,c,t][row s,c,n][col w,c,e], divisor 159
// (stencil/3dstencil/3d27pt/3d27pt_gold_gen.cpp:30-45).
__host__ __device__ constexpr double c27(int z, int y, int x) {
  return (y == 1 && x == 1) ? (z == 0 ? 1.5 : z == 1 ? 1.51 : 1.52)
       : (y == 1) ? (z == 0 ? 1.2 : z == 1 ? 1.21 : 1.22)
       : (x == 1) ? (z == 0 ? 0.7 : z == 1 ? 0.71 : 0.72)
       : ((y == 0) == (x == 0)) ? (z == 0 ? 0.5 : z == 1 ? 0.51 : 0.52)
                                : (z == 0 ? 0.9 : z == 1 ? 0.91 : 0.92);
}

// ------------------------------------------------------------ Ref order ----
// 2D star, reference order: south (far to near), west (far to near), centre,
// east, north, each term a rounded product added to the rounded running sum,
// then / 118. `add(acc, p)` is the rounded sum (a packed-pair caller passes a
// form ptxas cannot fuse with the product).
template <class T, int SHAPE, class U, class Add>
__device__ __forceinline__ T star2d_sum(const U& u, const Add& add) {
  using O = RN<T>;
  constexpr int H = ShapeInfo<SHAPE>::H;
  T acc = O::mul(T(star_s(H - 1)), u(0, -H, 0));
#pragma unroll
  for (int h = H - 2; h >= 0; h--) acc = add(acc, O::mul(T(star_s(h)), u(0, -1 - h, 0)));
#pragma unroll
  for (int h = H - 1; h >= 0; h--) acc = add(acc, O::mul(T(star_w(h)), u(0, 0, -1 - h)));
  acc = add(acc, O::mul(T(15), u(0, 0, 0)));
#pragma unroll
  for (int h = 0; h < H; h++) acc = add(acc, O::mul(T(star_e(h)), u(0, 0, 1 + h)));
#pragma unroll
  for (int h = 0; h < H; h++) acc = add(acc, O::mul(T(star_n(h)), u(0, 1 + h, 0)));
  return acc;
}
template <class T, int SHAPE, int FIN = 0, class U, class Add>
__device__ __forceinline__ T star2d_ref(const U& u, const Add& add) {
  return div_const<118, FIN>(star2d_sum<T, SHAPE>(u, add));
}

// 3D stars, reference order: e, w, n, s, t, b (3d13pt: each side near then
// far), every product and sum rounded, then minus the rounded centre term;
// float-literal coefficients. `add(acc, p)` / `sub(acc, p)` are the rounded
// sum and difference (a packed-pair caller passes forms ptxas cannot fuse
// with the product).
template <class T, int SHAPE, class U, class Add, class Sub>
__device__ __forceinline__ T star3d_ref(const U& u, const Add& add, const Sub& sub) {
  using O = RN<T>;
  if constexpr (SHAPE == PERKS_3D7PT) {
    T acc = O::mul(T(0.161f), u(0, 0, 1));
    acc = add(acc, O::mul(T(0.162f), u(0, 0, -1)));
    acc = add(acc, O::mul(T(0.163f), u(0, 1, 0)));
    acc = add(acc, O::mul(T(0.164f), u(0, -1, 0)));
    acc = add(acc, O::mul(T(0.165f), u(1, 0, 0)));
    acc = add(acc, O::mul(T(0.166f), u(-1, 0, 0)));
    return sub(acc, O::mul(T(1.67f), u(0, 0, 0)));
  } else {
    static_assert(SHAPE == PERKS_3D13PT, "3D star");
    const T c = T(0.083f);
    T acc = O::mul(c, u(0, 0, 1));
    acc = add(acc, O::mul(c, u(0, 0, 2)));
    acc = add(acc, O::mul(c, u(0, 0, -1)));
    acc = add(acc, O::mul(c, u(0, 0, -2)));
    acc = add(acc, O::mul(c, u(0, 1, 0)));
    acc = add(acc, O::mul(c, u(0, 2, 0)));
    acc = add(acc, O::mul(c, u(0, -1, 0)));
    acc = add(acc, O::mul(c, u(0, -2, 0)));
    acc = add(acc, O::mul(c, u(1, 0, 0)));
    acc = add(acc, O::mul(c, u(2, 0, 0)));
    acc = add(acc, O::mul(c, u(-1, 0, 0)));
    acc = add(acc, O::mul(c, u(-2, 0, 0)));
    return sub(acc, O::mul(T(0.996f), u(0, 0, 0)));
  }
}

template <class T, int SHAPE, int FIN = 0, class U>
__device__ __forceinline__ T point_ref(const U& u) {
  using O = RN<T>;
  constexpr int H = ShapeInfo<SHAPE>::H;
  if constexpr (SHAPE <= PERKS_2DS25PT) {
    return star2d_ref<T, SHAPE, FIN>(u, [](T a, T b) { return O::add(a, b); });
  } else if constexpr (SHAPE == PERKS_2D9PT || SHAPE == PERKS_2D25PT) {
    // Terms before the centre sum in T; the centre's double literal promotes
    // the rest of the sum to double; later products are still T products.
    using D = RN<double>;
    T accr = T(0);
    double accd = 0.0;
#pragma unroll
    for (int r = 0; r < 2 * H + 1; r++) {
#pragma unroll
      for (int c = 0; c < 2 * H + 1; c++) {
        const int w = (SHAPE == PERKS_2D9PT) ? box9_w(r, c) : box25_w(r, c);
        const T v = u(0, r - H, c - H);
        if (r == H && c == H) {
          accd = D::add(double(accr), D::mul(15.0, double(v)));
        } else if (r < H || (r == H && c < H)) {
          const T p = O::mul(T(w), v);
          accr = (r == 0 && c == 0) ? p : O::add(accr, p);
        } else {
          accd = D::add(accd, double(O::mul(T(w), v)));
        }
      }
    }
    return T(div_const<118, FIN>(accd));
  } else if constexpr (SHAPE == PERKS_3D7PT || SHAPE == PERKS_3D13PT) {
    return star3d_ref<T, SHAPE>(u, [](T a, T b) { return O::add(a, b); }, [](T a, T b) { return O::sub(a, b); });
  } else if constexpr (SHAPE == PERKS_3D17PT) {
    using D = RN<double>;
    T cb = O::add(u(-1, -1, -1), u(-1, -1, 1));
    cb = O::add(cb, u(-1, 1, -1));
    cb = O::add(cb, u(-1, 1, 1));
    double acc = D::mul(0.50, double(cb));
    acc = D::add(acc, D::mul(0.51, double(u(0, -1, -1))));
    acc = D::add(acc, D::mul(0.71, double(u(0, -1, 0))));
    acc = D::add(acc, D::mul(0.91, double(u(0, -1, 1))));
    acc = D::add(acc, D::mul(1.21, double(u(0, 0, -1))));
    acc = D::add(acc, D::mul(1.51, double(u(0, 0, 0))));
    acc = D::add(acc, D::mul(1.21, double(u(0, 0, 1))));
    acc = D::add(acc, D::mul(0.91, double(u(0, 1, -1))));
    acc = D::add(acc, D::mul(0.71, double(u(0, 1, 0))));
    acc = D::add(acc, D::mul(0.51, double(u(0, 1, 1))));
    T ct = O::add(u(1, -1, -1), u(1, -1, 1));
    ct = O::add(ct, u(1, 1, -1));
    ct = O::add(ct, u(1, 1, 1));
    acc = D::add(acc, D::mul(0.52, double(ct)));
    return T(div_const<159, FIN>(acc));
  } else if constexpr (SHAPE == PERKS_3D27PT) {
    using D = RN<double>;
    double acc = 0.0;
#pragma unroll
    for (int z = 0; z < 3; z++)
#pragma unroll
      for (int y = 0; y < 3; y++)
#pragma unroll
        for (int x = 0; x < 3; x++) {
          const double t = D::mul(c27(z, y, x), double(u(z - 1, y - 1, x - 1)));
          acc = (z == 0 && y == 0 && x == 0) ? t : D::add(acc, t);
        }
    return T(div_const<159, FIN>(acc));
  } else {  // PERKS_POISSON
    T f = O::add(u(-1, 0, 0), u(1, 0, 0));
    f = O::add(f, u(0, -1, 0));
    f = O::add(f, u(0, 1, 0));
    f = O::add(f, u(0, 0, 1));
    f = O::add(f, u(0, 0, -1));
    T e = O::add(u(-1, -1, 0), u(-1, 1, 0));
    e = O::add(e, u(1, -1, 0));
    e = O::add(e, u(1, 1, 0));
    e = O::add(e, u(-1, 0, -1));
    e = O::add(e, u(-1, 0, 1));
    e = O::add(e, u(1, 0, -1));
    e = O::add(e, u(1, 0, 1));
    e = O::add(e, u(0, -1, -1));
    e = O::add(e, u(0, -1, 1));
    e = O::add(e, u(0, 1, -1));
    e = O::add(e, u(0, 1, 1));
    T acc = O::sub(O::mul(T(2.666f), u(0, 0, 0)), O::mul(T(0.166f), f));
    return O::sub(acc, O::mul(T(0.0833f), e));
  }
}

// ----------------------------------------------------------- Fast order ----
template <class T, int SHAPE, class U>
__device__ __forceinline__ T point_fast(const U& u) {
  constexpr int H = ShapeInfo<SHAPE>::H;
  if constexpr (SHAPE <= PERKS_2DS25PT) {
    constexpr double k = 1.0 / 118.0;
    T acc = T(15 * k) * u(0, 0, 0);
#pragma unroll
    for (int h = 0; h < H; h++) {
      acc = fma(T(star_s(h) * k), u(0, -1 - h, 0), acc);
      acc = fma(T(star_w(h) * k), u(0, 0, -1 - h), acc);
      acc = fma(T(star_e(h) * k), u(0, 0, 1 + h), acc);
      acc = fma(T(star_n(h) * k), u(0, 1 + h, 0), acc);
    }
    return acc;
  } else if constexpr (SHAPE == PERKS_2D9PT || SHAPE == PERKS_2D25PT) {
    constexpr double k = 1.0 / 118.0;
    T acc = T(0);
#pragma unroll
    for (int r = 0; r < 2 * H + 1; r++)
#pragma unroll
      for (int c = 0; c < 2 * H + 1; c++) {
        const int w = (SHAPE == PERKS_2D9PT) ? box9_w(r, c) : box25_w(r, c);
        acc = fma(T(w * k), u(0, r - H, c - H), acc);
      }
    return acc;
  } else if constexpr (SHAPE == PERKS_3D7PT) {
    T acc = T(-1.67f) * u(0, 0, 0);
    acc = fma(T(0.161f), u(0, 0, 1), acc);
    acc = fma(T(0.162f), u(0, 0, -1), acc);
    acc = fma(T(0.163f), u(0, 1, 0), acc);
    acc = fma(T(0.164f), u(0, -1, 0), acc);
    acc = fma(T(0.165f), u(1, 0, 0), acc);
    acc = fma(T(0.166f), u(-1, 0, 0), acc);
    return acc;
  } else if constexpr (SHAPE == PERKS_3D13PT) {
    T s = u(0, 0, 1) + u(0, 0, 2) + u(0, 0, -1) + u(0, 0, -2) + u(0, 1, 0) + u(0, 2, 0) + u(0, -1, 0) +
          u(0, -2, 0) + u(1, 0, 0) + u(2, 0, 0) + u(-1, 0, 0) + u(-2, 0, 0);
    return fma(T(0.083f), s, T(-0.996f) * u(0, 0, 0));
  } else if constexpr (SHAPE == PERKS_3D17PT) {
    constexpr double k = 1.0 / 159.0;
    T cb = u(-1, -1, -1) + u(-1, -1, 1) + u(-1, 1, -1) + u(-1, 1, 1);
    T ct = u(1, -1, -1) + u(1, -1, 1) + u(1, 1, -1) + u(1, 1, 1);
    T acc = T(0.50 * k) * cb;
    acc = fma(T(0.52 * k), ct, acc);
#pragma unroll
    for (int y = 0; y < 3; y++)
#pragma unroll
      for (int x = 0; x < 3; x++) acc = fma(T(c27(1, y, x) * k), u(0, y - 1, x - 1), acc);
    return acc;
  } else if constexpr (SHAPE == PERKS_3D27PT) {
    constexpr double k = 1.0 / 159.0;
    T acc = T(0);
#pragma unroll
    for (int z = 0; z < 3; z++)
#pragma unroll
      for (int y = 0; y < 3; y++)
#pragma unroll
        for (int x = 0; x < 3; x++) acc = fma(T(c27(z, y, x) * k), u(z - 1, y - 1, x - 1), acc);
    return acc;
  } else {  // PERKS_POISSON
    T f = u(-1, 0, 0) + u(1, 0, 0) + u(0, -1, 0) + u(0, 1, 0) + u(0, 0, 1) + u(0, 0, -1);
    T e = u(-1, -1, 0) + u(-1, 1, 0) + u(1, -1, 0) + u(1, 1, 0) + u(-1, 0, -1) + u(-1, 0, 1) + u(1, 0, -1) +
          u(1, 0, 1) + u(0, -1, -1) + u(0, -1, 1) + u(0, 1, -1) + u(0, 1, 1);
    T acc = fma(T(-0.166f), f, T(2.666f) * u(0, 0, 0));
    return fma(T(-0.0833f), e, acc);
  }
}

template <class T, int SHAPE, bool FAST, int FIN = 0, class U>
__device__ __forceinline__ T stencil_point(const U& u) {
  if constexpr (FAST)
    return point_fast<T, SHAPE>(u);
  else
    return point_ref<T, SHAPE, FIN>(u);
}

}  // namespace perks
