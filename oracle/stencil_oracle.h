/* ORACLE — test infrastructure only (see stencil_oracle.c, cg_oracle.c). */
#ifndef PERKS_ORACLE_H
#define PERKS_ORACLE_H
#include <stddef.h>
#include "../include/perks.h"
#ifdef __cplusplus
extern "C" {
#endif
int oracle_shape_halo(int shape);
int oracle_stencil2d_f32(int shape, const float* in, int wy, int wx, float* out, int steps, int boundary);
int oracle_stencil2d_f64(int shape, const double* in, int wy, int wx, double* out, int steps, int boundary);
int oracle_stencil3d_f32(int shape, const float* in, int h, int wy, int wx, float* out, int steps, int boundary);
int oracle_stencil3d_f64(int shape, const double* in, int h, int wy, int wx, double* out, int steps, int boundary);
int oracle_num_threads(void);
int oracle_set_num_threads(int n);

void oracle_spmv_csr_f64(int n, const int* rp, const int* ci, const double* v, const double* x, double* y);
void oracle_spmv_csr_f32(int n, const int* rp, const int* ci, const float* v, const float* x, float* y);
void oracle_spmv_dia_f64(int n, int ndiag, const int* off, const double* data, const double* x, double* y);
int oracle_cg_f64(int n, const int* rp, const int* ci, const double* v, const double* b, double* x,
                  int max_iter, int stop, double tol, int static_iter, double* rr_out, double* trace);
int oracle_cg_f32(int n, const int* rp, const int* ci, const float* v, const float* b, float* x,
                  int max_iter, int stop, double tol, int static_iter, double* rr_out, double* trace);
int oracle_cg_dia_f64(int n, int ndiag, const int* off, const double* data, const double* b, double* x,
                      int max_iter, int stop, double tol, int static_iter, double* rr_out, double* trace);
void oracle_gen_tridiag_f32(int n, unsigned seed, int* rp, int* ci, float* v);
void oracle_gen_tridiag_f64(int n, unsigned seed, int* rp, int* ci, double* v);
#ifdef __cplusplus
}
#endif
#endif
