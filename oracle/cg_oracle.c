/*
 * ORACLE — test infrastructure only.
 *
 * CPU restatement of the PERKS reference's conjugate-gradient iteration and
 * its SpMV, used by tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline leg to check or time against, never as the thing measured.
 * The product library never links it.
 *
 * The iteration follows cpuConjugateGrad (conjugateGradient/cg_cpu.cpp:40-81)
 * step for step:
 *   Ax = A x; r = -1*Ax + r; r1 = r.r;  k = 1
 *   loop: p = r (k == 1) or p = 1*r + (r1/r0)*p;  Ax = A p;
 *         a = r1 / p.Ax;  x = a*p + x;  r = (-a)*Ax + r;  r0 = r1;  r1 = r.r
 * with the stop test the reference's GPU kernel applies at the top of each
 * iteration (conjugateGradient/cg_kernels.cuh:834): stop when r1 < tol^2
 * (PERKS_STOP_ABS_RR) unless static_iter, or when k > max_iter. The relative
 * stop PERKS_STOP_REL (r1 < tol^2 * b.b) is an addition of this project.
 *
 * oracle_cg_f32 reproduces the reference's float build bit for bit: float
 * vectors, dot products accumulated in double from float products
 * (cg_cpu.cpp:18-26) and rounded back to float for r1 and p.Ap, a = r1/dot in
 * float (cg_cpu.cpp:70-71). Pinned against the reference's own cg_cpu.cpp
 * functions in tests/test_oracle.py.
 *
 * oracle_cg_f64 is the same algorithm in double; the reference ships no
 * double CPU CG (its cg_cpu.cpp is float only), so this is the FP64 oracle.
 *
 * Returns the number of iterations executed, or -1 on a breakdown
 * (p.Ap <= 0 or non-finite) when breakdown checks are enabled (FP64 only;
 * the float variant mirrors the reference, which has no such check).
 * Build with -ffp-contract=off.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "stencil_oracle.h"

/* cpuSpMV (cg_cpu.cpp:3-16) with alpha = 1: output += (1*val)*x in float. */
void oracle_spmv_csr_f32(int n, const int* rp, const int* ci, const float* v, const float* x, float* y) {
  for (int i = 0; i < n; i++) {
    float acc = 0.0f;
    for (int j = rp[i]; j < rp[i + 1]; j++) acc = acc + (1.0f * v[j]) * x[ci[j]];
    y[i] = acc;
  }
}

void oracle_spmv_csr_f64(int n, const int* rp, const int* ci, const double* v, const double* x, double* y) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; i++) {
    double acc = 0.0;
    for (int j = rp[i]; j < rp[i + 1]; j++) acc = acc + v[j] * x[ci[j]];
    y[i] = acc;
  }
}

/* DIA, diagonal-major: data[k*n + i] = A[i][i + off[k]]. */
void oracle_spmv_dia_f64(int n, int ndiag, const int* off, const double* data, const double* x, double* y) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; i++) {
    double acc = 0.0;
    for (int k = 0; k < ndiag; k++) {
      long c = (long)i + off[k];
      if (c >= 0 && c < n) acc = acc + data[(size_t)k * n + i] * x[c];
    }
    y[i] = acc;
  }
}

static double dot_f32(const float* a, const float* b, int n) {
  double s = 0.0;
  for (int i = 0; i < n; i++) s = s + (double)(a[i] * b[i]);
  return s;
}

static double dot_f64(const double* a, const double* b, int n) {
  double s = 0.0;
  for (int i = 0; i < n; i++) s = s + a[i] * b[i];
  return s;
}

int oracle_cg_f32(int n, const int* rp, const int* ci, const float* v, const float* b, float* x,
                  int max_iter, int stop, double tol, int static_iter, double* rr_out, double* trace) {
  float* r = (float*)malloc(sizeof(float) * n);
  float* p = (float*)malloc(sizeof(float) * n);
  float* Ax = (float*)malloc(sizeof(float) * n);
  if (!r || !p || !Ax) { free(r); free(p); free(Ax); return -2; }
  const float ftol = (float)tol;
  const float tol2 = ftol * ftol;
  const double bb = dot_f32(b, b, n);
  memcpy(r, b, sizeof(float) * n);
  oracle_spmv_csr_f32(n, rp, ci, v, x, Ax);
  for (int i = 0; i < n; i++) r[i] = -1.0f * Ax[i] + r[i];
  float r1 = (float)dot_f32(r, r, n), r0 = 0.0f;
  int k = 1;
  if (trace) trace[0] = r1;
  while (k <= max_iter) {
    if (!static_iter) {
      if (stop == PERKS_STOP_ABS_RR && r1 < tol2) break;
      if (stop == PERKS_STOP_REL && (double)r1 < (double)tol2 * bb) break;
    }
    if (k > 1) {
      float beta = r1 / r0;
      for (int i = 0; i < n; i++) p[i] = beta * p[i];
      for (int i = 0; i < n; i++) p[i] = 1.0f * r[i] + p[i];
    } else {
      memcpy(p, r, sizeof(float) * n);
    }
    oracle_spmv_csr_f32(n, rp, ci, v, p, Ax);
    float dot = (float)dot_f32(p, Ax, n);
    float a = r1 / dot;
    for (int i = 0; i < n; i++) x[i] = a * p[i] + x[i];
    float na = -a;
    for (int i = 0; i < n; i++) r[i] = na * Ax[i] + r[i];
    r0 = r1;
    r1 = (float)dot_f32(r, r, n);
    if (trace) trace[k] = r1;
    k++;
  }
  if (rr_out) *rr_out = r1;
  free(r); free(p); free(Ax);
  return k - 1;
}

typedef void (*spmv64_fn)(const void* ctx, const double* x, double* y);

typedef struct { int n; const int* rp; const int* ci; const double* v; } csr_ctx;
typedef struct { int n; int nd; const int* off; const double* data; } dia_ctx;

static void csr_apply(const void* c, const double* x, double* y) {
  const csr_ctx* m = (const csr_ctx*)c;
  oracle_spmv_csr_f64(m->n, m->rp, m->ci, m->v, x, y);
}
static void dia_apply(const void* c, const double* x, double* y) {
  const dia_ctx* m = (const dia_ctx*)c;
  oracle_spmv_dia_f64(m->n, m->nd, m->off, m->data, x, y);
}

static int cg64(int n, spmv64_fn A, const void* ctx, const double* b, double* x, int max_iter, int stop,
                double tol, int static_iter, double* rr_out, double* trace) {
  double* r = (double*)malloc(sizeof(double) * n);
  double* p = (double*)malloc(sizeof(double) * n);
  double* Ax = (double*)malloc(sizeof(double) * n);
  if (!r || !p || !Ax) { free(r); free(p); free(Ax); return -2; }
  const double tol2 = tol * tol;
  const double bb = dot_f64(b, b, n);
  int status = 0;
  memcpy(r, b, sizeof(double) * n);
  A(ctx, x, Ax);
  /* element-wise loops run in parallel (each element's arithmetic is the
   * same whatever the thread); the dot products stay sequential */
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; i++) r[i] = -1.0 * Ax[i] + r[i];
  double r1 = dot_f64(r, r, n), r0 = 0.0;
  int k = 1;
  if (trace) trace[0] = r1;
  while (k <= max_iter) {
    if (!static_iter) {
      if (stop == PERKS_STOP_ABS_RR && r1 < tol2) break;
      if (stop == PERKS_STOP_REL && r1 < tol2 * bb) break;
    }
    if (k > 1) {
      double beta = r1 / r0;
#pragma omp parallel for schedule(static)
      for (int i = 0; i < n; i++) p[i] = r[i] + beta * p[i];
    } else {
      memcpy(p, r, sizeof(double) * n);
    }
    A(ctx, p, Ax);
    double dot = dot_f64(p, Ax, n);
    if (!(dot > 0.0) || !isfinite(dot)) { status = -1; break; }
    double a = r1 / dot;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; i++) {
      x[i] = a * p[i] + x[i];
      r[i] = -a * Ax[i] + r[i];
    }
    r0 = r1;
    r1 = dot_f64(r, r, n);
    if (trace) trace[k] = r1;
    k++;
  }
  if (rr_out) *rr_out = r1;
  free(r); free(p); free(Ax);
  return status < 0 ? -1 : k - 1;
}

int oracle_cg_f64(int n, const int* rp, const int* ci, const double* v, const double* b, double* x,
                  int max_iter, int stop, double tol, int static_iter, double* rr_out, double* trace) {
  csr_ctx c = {n, rp, ci, v};
  return cg64(n, csr_apply, &c, b, x, max_iter, stop, tol, static_iter, rr_out, trace);
}

int oracle_cg_dia_f64(int n, int ndiag, const int* off, const double* data, const double* b, double* x,
                      int max_iter, int stop, double tol, int static_iter, double* rr_out, double* trace) {
  dia_ctx c = {n, ndiag, off, data};
  return cg64(n, dia_apply, &c, b, x, max_iter, stop, tol, static_iter, rr_out, trace);
}

/* Random symmetric tridiagonal matrix as genTridiag makes it
 * (conjugateGradient/matrix/tridiag.cpp:11-41): diagonal rand()/RAND_MAX + 10,
 * off-diagonal rand()/RAND_MAX, drawn in the order d0, o01, d1, o12, ... from
 * the C library rand() after srand(seed). nnz = 3n - 2. */
#define DEF_TRIDIAG(REAL, SUF)                                                   \
  void oracle_gen_tridiag_##SUF(int n, unsigned seed, int* rp, int* ci, REAL* v) { \
    srand(seed);                                                                 \
    rp[0] = 0;                                                                   \
    ci[0] = 0;                                                                   \
    ci[1] = 1;                                                                   \
    v[0] = (REAL)rand() / RAND_MAX + 10.0f;                                      \
    v[1] = (REAL)rand() / RAND_MAX;                                              \
    for (int i = 1; i < n; i++) {                                                \
      rp[i] = (i > 1) ? rp[i - 1] + 3 : 2;                                       \
      int s = (i - 1) * 3 + 2;                                                   \
      ci[s] = i - 1;                                                             \
      ci[s + 1] = i;                                                             \
      if (i < n - 1) ci[s + 2] = i + 1;                                          \
      v[s] = v[s - 1];                                                           \
      v[s + 1] = (REAL)rand() / RAND_MAX + 10.0f;                                \
      if (i < n - 1) v[s + 2] = (REAL)rand() / RAND_MAX;                         \
    }                                                                            \
    rp[n] = 3 * n - 2;                                                           \
  }
DEF_TRIDIAG(float, f32)
DEF_TRIDIAG(double, f64)
