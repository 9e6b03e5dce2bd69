/*
 * ORACLE — test infrastructure only.
 *
 * CPU restatement of the PERKS reference's CPU "gold" stencil code, used by
 * tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg to check
 * or time against. Nothing in the product library links or calls this file.
 *
 * Parity pin: tests/test_oracle.py checks every shape and both precisions of
 * this file bit-for-bit against the reference's own gold functions compiled
 * from the reference sources (oracle/_ref, built by oracle/Makefile) and
 * against the committed fixtures in tests/golden/ that were produced by them.
 *
 * Semantics restated (all citations are paths inside the reference project):
 *  - Every cell of the width_y x width_x (x height) array is updated each
 *    step; out-of-range neighbours are clamped to the nearest edge cell
 *    (stencil/2dstencil/2d5pt/jacobi_gold_gen.cpp:27-31,
 *     stencil/3dstencil/3d7pt/3d7pt_gold_gen.cpp:21-26).
 *  - Evaluation order is left to right exactly as the reference writes each
 *    expression; integer weights are converted to REAL, float literals keep
 *    their float value, double literals (15.0 in the 2D box shapes, the /159
 *    shapes in 3D) promote the running sum to double mid-expression.
 *  - Ping-pong iteration (jacobi_gold_iterative, 2d5pt/jacobi_gold_gen.cpp:49-74):
 *    after `iteration` steps the newest field is the output. iteration==0 is
 *    defined here as a plain copy (the reference would run one step).
 *  - PERKS_BOUNDARY_DIRICHLET is an extra mode the reference does not have:
 *    the outer `halo` cells on every face are held fixed and only the
 *    interior is updated.
 *
 * Build with -ffp-contract=off: the reference is compiled by g++ on x86-64
 * without FMA, so no multiply-add may be fused here either.
 */
#include <stdlib.h>
#include <string.h>
#include "stencil_oracle.h"
#ifdef _OPENMP
#include <omp.h>
#endif

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* Star-shape weights by distance (index 0 = nearest neighbour), from the
 * 2D gold files: 2ds25pt/jacobi_gold_gen.cpp:55-86 holds the full set, the
 * lower orders use prefixes of the same tables. Centre weight 15, divisor 118. */
static const int STAR_S[6] = {5, 7, 5, 1, 6, 2};
static const int STAR_W[6] = {12, 9, 3, 2, 5, 6};
static const int STAR_E[6] = {12, 9, 3, 3, 4, 6};
static const int STAR_N[6] = {5, 7, 5, 4, 3, 2};

/* Box weights, row-major from the south-most row, west-most column
 * (2d9pt/jacobi_gold_gen.cpp:33-36, 2d25pt/jacobi_gold_gen.cpp:35-40).
 * The centre (15.0) is a double literal in the reference. */
static const int BOX9[3][3] = {{7, 5, 9}, {12, 15, 12}, {9, 5, 7}};
static const int BOX25[5][5] = {{1, 2, 3, 4, 5},
                                {7, 7, 5, 7, 6},
                                {8, 12, 15, 12, 12},
                                {9, 9, 5, 7, 15},
                                {10, 11, 12, 13, 14}};

int oracle_shape_halo(int shape) {
  switch (shape) {
    case PERKS_2D5PT: return 1;
    case PERKS_2DS9PT: return 2;
    case PERKS_2D13PT: return 3;
    case PERKS_2D17PT: return 4;
    case PERKS_2D21PT: return 5;
    case PERKS_2DS25PT: return 6;
    case PERKS_2D9PT: return 1;
    case PERKS_2D25PT: return 2;
    case PERKS_3D7PT: return 1;
    case PERKS_3D13PT: return 2;
    case PERKS_3D17PT: return 1;
    case PERKS_3D27PT: return 1;
    case PERKS_POISSON: return 1;
    default: return -1;
  }
}

/* ------------------------------------------------------------------ 2D --- */
#define U2(yy, xx) in[(size_t)(yy) * wx + (xx)]

#define DEF_STAR2D(REAL, SUF)                                                     \
  static REAL star2d_##SUF(const REAL* in, int wy, int wx, int y, int x, int H) { \
    REAL acc = 0;                                                                 \
    int first = 1;                                                                \
    for (int h = H - 1; h >= 0; h--) {                                            \
      REAL t = (REAL)STAR_S[h] * U2(clampi(y - 1 - h, 0, wy - 1), x);            \
      if (first) { acc = t; first = 0; } else acc = acc + t;                      \
    }                                                                             \
    for (int h = H - 1; h >= 0; h--)                                              \
      acc = acc + (REAL)STAR_W[h] * U2(y, clampi(x - 1 - h, 0, wx - 1));         \
    acc = acc + (REAL)15 * U2(y, x);                                              \
    for (int h = 0; h < H; h++)                                                   \
      acc = acc + (REAL)STAR_E[h] * U2(y, clampi(x + 1 + h, 0, wx - 1));         \
    for (int h = 0; h < H; h++)                                                   \
      acc = acc + (REAL)STAR_N[h] * U2(clampi(y + 1 + h, 0, wy - 1), x);         \
    return acc / (REAL)118;                                                       \
  }

/* Box shapes: the sum runs in REAL up to the centre term, whose double
 * literal promotes the rest of the expression to double; the terms after the
 * centre are still REAL products added to a double. */
#define DEF_BOX2D(REAL, SUF)                                                      \
  static REAL box2d_##SUF(const REAL* in, int wy, int wx, int y, int x, int H,    \
                          const int* wts) {                                       \
    int n = 2 * H + 1;                                                            \
    REAL accr = 0;                                                                \
    double accd = 0;                                                              \
    int first = 1, promoted = 0;                                                  \
    for (int dy = -H; dy <= H; dy++) {                                            \
      int yy = clampi(y + dy, 0, wy - 1);                                         \
      for (int dx = -H; dx <= H; dx++) {                                          \
        int xx = clampi(x + dx, 0, wx - 1);                                       \
        int w = wts[(dy + H) * n + (dx + H)];                                     \
        if (dy == 0 && dx == 0) {                                                 \
          accd = (double)accr + 15.0 * (double)U2(yy, xx);                        \
          promoted = 1;                                                           \
        } else if (!promoted) {                                                   \
          REAL t = (REAL)w * U2(yy, xx);                                          \
          if (first) { accr = t; first = 0; } else accr = accr + t;               \
        } else {                                                                  \
          REAL t = (REAL)w * U2(yy, xx);                                          \
          accd = accd + (double)t;                                                \
        }                                                                         \
      }                                                                           \
    }                                                                             \
    return (REAL)(accd / 118.0);                                                  \
  }

DEF_STAR2D(float, f32)
DEF_STAR2D(double, f64)
DEF_BOX2D(float, f32)
DEF_BOX2D(double, f64)

#define DEF_STEP2D(REAL, SUF)                                                      \
  static int step2d_##SUF(int shape, const REAL* in, int wy, int wx, REAL* out,    \
                          int boundary) {                                          \
    int H = oracle_shape_halo(shape);                                              \
    int isbox = (shape == PERKS_2D9PT || shape == PERKS_2D25PT);                   \
    const int* wts = shape == PERKS_2D9PT ? &BOX9[0][0] : &BOX25[0][0];            \
    if (H < 0 || shape > PERKS_2D25PT) return -1;                                  \
    _Pragma("omp parallel for schedule(static)")                                   \
    for (int y = 0; y < wy; y++) {                                                 \
      for (int x = 0; x < wx; x++) {                                               \
        REAL v;                                                                    \
        if (boundary == PERKS_BOUNDARY_DIRICHLET &&                                \
            (y < H || y >= wy - H || x < H || x >= wx - H))                        \
          v = U2(y, x);                                                            \
        else if (isbox)                                                            \
          v = box2d_##SUF(in, wy, wx, y, x, H, wts);                               \
        else                                                                       \
          v = star2d_##SUF(in, wy, wx, y, x, H);                                   \
        out[(size_t)y * wx + x] = v;                                               \
      }                                                                            \
    }                                                                              \
    return 0;                                                                      \
  }

DEF_STEP2D(float, f32)
DEF_STEP2D(double, f64)

/* ------------------------------------------------------------------ 3D --- */
#define U3(zz, yy, xx) in[((size_t)(zz) * wy + (yy)) * wx + (xx)]

/* One neighbour of a 3D point with clamped coordinates. */
#define NB(dz, dy, dx) \
  U3(clampi(z + (dz), 0, h - 1), clampi(y + (dy), 0, wy - 1), clampi(x + (dx), 0, wx - 1))

/* 3d7pt (3d7pt/3d7pt_gold_gen.cpp:28-33): float-literal coefficients over
 * e,w,n,s,t,b then minus the centre term. */
static const float C7[6] = {0.161f, 0.162f, 0.163f, 0.164f, 0.165f, 0.166f};
static const int D7[6][3] = {{0, 0, 1}, {0, 0, -1}, {0, 1, 0}, {0, -1, 0}, {1, 0, 0}, {-1, 0, 0}};
/* 3d13pt (3d13pt/3d13pt_gold_gen.cpp:34-40): e0,e1,w0,w1,n0,n1,s0,s1,t0,t1,b0,b1. */
static const int D13[12][3] = {{0, 0, 1}, {0, 0, 2}, {0, 0, -1}, {0, 0, -2}, {0, 1, 0}, {0, 2, 0},
                               {0, -1, 0}, {0, -2, 0}, {1, 0, 0}, {2, 0, 0}, {-1, 0, 0}, {-2, 0, 0}};
/* 3d27pt (3d27pt/3d27pt_gold_gen.cpp:30-45): double coefficients, planes
 * b,c,t; rows s,c,n; columns w,c,e; divisor 159. */
static const double C27[3][3][3] = {{{0.5, 0.7, 0.9}, {1.2, 1.5, 1.2}, {0.9, 0.7, 0.5}},
                                    {{0.51, 0.71, 0.91}, {1.21, 1.51, 1.21}, {0.91, 0.71, 0.51}},
                                    {{0.52, 0.72, 0.92}, {1.22, 1.52, 1.22}, {0.92, 0.72, 0.52}}};

#define DEF_POINT3D(REAL, SUF)                                                         \
  static REAL point3d_##SUF(int shape, const REAL* in, int h, int wy, int wx, int z,   \
                            int y, int x) {                                            \
    switch (shape) {                                                                   \
      case PERKS_3D7PT: {                                                              \
        REAL acc = (REAL)C7[0] * NB(D7[0][0], D7[0][1], D7[0][2]);                     \
        for (int i = 1; i < 6; i++) acc = acc + (REAL)C7[i] * NB(D7[i][0], D7[i][1], D7[i][2]); \
        return acc - (REAL)1.67f * NB(0, 0, 0);                                        \
      }                                                                                \
      case PERKS_3D13PT: {                                                             \
        REAL acc = (REAL)0.083f * NB(D13[0][0], D13[0][1], D13[0][2]);                 \
        for (int i = 1; i < 12; i++)                                                   \
          acc = acc + (REAL)0.083f * NB(D13[i][0], D13[i][1], D13[i][2]);              \
        return acc - (REAL)0.996f * NB(0, 0, 0);                                       \
      }                                                                                \
      case PERKS_3D17PT: {                                                             \
        /* 3d17pt/3d17pt_gold_gen.cpp:28-33: corner sums in REAL, the rest double */   \
        REAL cb = NB(-1, -1, -1) + NB(-1, -1, 1);                                      \
        cb = cb + NB(-1, 1, -1);                                                       \
        cb = cb + NB(-1, 1, 1);                                                        \
        double acc = 0.50 * (double)cb;                                                \
        acc = acc + 0.51 * (double)NB(0, -1, -1);                                      \
        acc = acc + 0.71 * (double)NB(0, -1, 0);                                       \
        acc = acc + 0.91 * (double)NB(0, -1, 1);                                       \
        acc = acc + 1.21 * (double)NB(0, 0, -1);                                       \
        acc = acc + 1.51 * (double)NB(0, 0, 0);                                        \
        acc = acc + 1.21 * (double)NB(0, 0, 1);                                        \
        acc = acc + 0.91 * (double)NB(0, 1, -1);                                       \
        acc = acc + 0.71 * (double)NB(0, 1, 0);                                        \
        acc = acc + 0.51 * (double)NB(0, 1, 1);                                        \
        REAL ct = NB(1, -1, -1) + NB(1, -1, 1);                                        \
        ct = ct + NB(1, 1, -1);                                                        \
        ct = ct + NB(1, 1, 1);                                                         \
        acc = acc + 0.52 * (double)ct;                                                 \
        return (REAL)(acc / 159.0);                                                    \
      }                                                                                \
      case PERKS_3D27PT: {                                                             \
        double acc = 0;                                                                \
        int first = 1;                                                                 \
        for (int dz = -1; dz <= 1; dz++)                                               \
          for (int dy = -1; dy <= 1; dy++)                                             \
            for (int dx = -1; dx <= 1; dx++) {                                         \
              double t = C27[dz + 1][dy + 1][dx + 1] * (double)NB(dz, dy, dx);         \
              if (first) { acc = t; first = 0; } else acc = acc + t;                   \
            }                                                                          \
        return (REAL)(acc / 159.0);                                                    \
      }                                                                                \
      case PERKS_POISSON: {                                                            \
        /* poisson/poisson_gold_gen.cpp:26-34 */                                       \
        REAL f = NB(-1, 0, 0) + NB(1, 0, 0);                                           \
        f = f + NB(0, -1, 0);                                                          \
        f = f + NB(0, 1, 0);                                                           \
        f = f + NB(0, 0, 1);                                                           \
        f = f + NB(0, 0, -1);                                                          \
        REAL e = NB(-1, -1, 0) + NB(-1, 1, 0);                                         \
        e = e + NB(1, -1, 0);                                                          \
        e = e + NB(1, 1, 0);                                                           \
        e = e + NB(-1, 0, -1);                                                         \
        e = e + NB(-1, 0, 1);                                                          \
        e = e + NB(1, 0, -1);                                                          \
        e = e + NB(1, 0, 1);                                                           \
        e = e + NB(0, -1, -1);                                                         \
        e = e + NB(0, -1, 1);                                                          \
        e = e + NB(0, 1, -1);                                                          \
        e = e + NB(0, 1, 1);                                                           \
        REAL acc = (REAL)2.666f * NB(0, 0, 0) - (REAL)0.166f * f;                      \
        return acc - (REAL)0.0833f * e;                                                \
      }                                                                                \
      default: return 0;                                                               \
    }                                                                                  \
  }

DEF_POINT3D(float, f32)
DEF_POINT3D(double, f64)

#define DEF_STEP3D(REAL, SUF)                                                          \
  static int step3d_##SUF(int shape, const REAL* in, int h, int wy, int wx, REAL* out, \
                          int boundary) {                                              \
    int H = oracle_shape_halo(shape);                                                  \
    if (H < 0 || shape < PERKS_3D7PT) return -1;                                       \
    _Pragma("omp parallel for schedule(static)")                                       \
    for (int z = 0; z < h; z++)                                                        \
      for (int y = 0; y < wy; y++)                                                     \
        for (int x = 0; x < wx; x++) {                                                 \
          REAL v;                                                                      \
          if (boundary == PERKS_BOUNDARY_DIRICHLET &&                                  \
              (z < H || z >= h - H || y < H || y >= wy - H || x < H || x >= wx - H))   \
            v = U3(z, y, x);                                                           \
          else                                                                         \
            v = point3d_##SUF(shape, in, h, wy, wx, z, y, x);                          \
          out[((size_t)z * wy + y) * wx + x] = v;                                      \
        }                                                                              \
    return 0;                                                                          \
  }

DEF_STEP3D(float, f32)
DEF_STEP3D(double, f64)

/* ------------------------------------------------------- iteration driver --- */
/* Ping-pong driver. The reference alternates between the output buffer and
 * one temporary so that the newest field lands in the output
 * (2d5pt/jacobi_gold_gen.cpp:49-74); the same final placement is reached here
 * by choosing the first destination from the parity of `steps`. */
#define DEF_ITER(REAL, SUF)                                                             \
  int oracle_stencil2d_##SUF(int shape, const REAL* in, int wy, int wx, REAL* out,      \
                             int steps, int boundary) {                                 \
    size_t n = (size_t)wy * wx;                                                         \
    if (wy <= 0 || wx <= 0 || steps < 0 || shape < 0 || shape > PERKS_2D25PT) return -1; \
    if (steps == 0) { memmove(out, in, n * sizeof(REAL)); return 0; }                   \
    REAL* tmp = (REAL*)malloc(n * sizeof(REAL));                                        \
    if (!tmp) return -2;                                                                \
    REAL* a = (steps % 2 == 1) ? out : tmp;                                             \
    REAL* b = (steps % 2 == 1) ? tmp : out;                                             \
    step2d_##SUF(shape, in, wy, wx, a, boundary);                                       \
    for (int t = 1; t < steps; t++) {                                                   \
      step2d_##SUF(shape, a, wy, wx, b, boundary);                                      \
      REAL* s = a; a = b; b = s;                                                        \
    }                                                                                   \
    free(tmp);                                                                          \
    return 0;                                                                           \
  }                                                                                     \
  int oracle_stencil3d_##SUF(int shape, const REAL* in, int h, int wy, int wx, REAL* out, \
                             int steps, int boundary) {                                 \
    size_t n = (size_t)h * wy * wx;                                                     \
    if (h <= 0 || wy <= 0 || wx <= 0 || steps < 0 || shape < PERKS_3D7PT ||             \
        shape > PERKS_POISSON) return -1;                                               \
    if (steps == 0) { memmove(out, in, n * sizeof(REAL)); return 0; }                   \
    REAL* tmp = (REAL*)malloc(n * sizeof(REAL));                                        \
    if (!tmp) return -2;                                                                \
    REAL* a = (steps % 2 == 1) ? out : tmp;                                             \
    REAL* b = (steps % 2 == 1) ? tmp : out;                                             \
    step3d_##SUF(shape, in, h, wy, wx, a, boundary);                                    \
    for (int t = 1; t < steps; t++) {                                                   \
      step3d_##SUF(shape, a, h, wy, wx, b, boundary);                                   \
      REAL* s = a; a = b; b = s;                                                        \
    }                                                                                   \
    free(tmp);                                                                          \
    return 0;                                                                           \
  }

DEF_ITER(float, f32)
DEF_ITER(double, f64)

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* Threads of the parallel loops from now on (n <= 0: all cores); returns the
 * previous count. For timing the port on one core as well as on all. */
int oracle_set_num_threads(int n) {
#ifdef _OPENMP
  static int all = 0;
  if (!all) all = omp_get_num_procs();
  const int prev = omp_get_max_threads();
  omp_set_num_threads(n > 0 ? n : all);
  return prev;
#else
  (void)n;
  return 1;
#endif
}
