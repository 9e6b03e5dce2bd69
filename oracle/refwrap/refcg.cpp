// Reference-side shim (test infrastructure): compiles the reference's
// unmodified conjugateGradient/cg_cpu.cpp and matrix/tridiag.cpp and exports
//  - ref_cpu_cg: cpuConjugateGrad exactly as shipped (MAXITER iterations);
//  - ref_cg_steps: the same loop body for a chosen iteration count, built
//    from the reference's own cpuSpMV/dotProduct/scaleVector/saxpy, so that
//    iterates can be compared before the shipped loop runs into 0/0;
//  - ref_gen_tridiag_f32/f64: genTridiag after srand(seed).
#include <cstdlib>
#include <cstring>
#include CG_SRC
#include TRIDIAG_SRC

extern "C" void ref_cpu_cg(int* I, int* J, float* val, float* x, float* Ax, float* p, float* r, int nnz,
                           int N, float tol) {
  cpuConjugateGrad(I, J, val, x, Ax, p, r, nnz, N, tol);
}
extern "C" int ref_max_iter(void) { return MAXITER; }

extern "C" void ref_cg_steps(int* I, int* J, float* val, float* x, float* Ax, float* p, float* r, int nnz,
                             int N, int iters, double* trace) {
  float alpha = 1.0f, alpham1 = -1.0f, r0 = 0.0f, b, a, na;
  cpuSpMV(I, J, val, nnz, N, alpha, x, Ax);
  saxpy(Ax, r, alpham1, N);
  float r1 = dotProduct(r, r, N);
  if (trace) trace[0] = r1;
  for (int k = 1; k <= iters; k++) {
    if (k > 1) {
      b = r1 / r0;
      scaleVector(p, b, N);
      saxpy(r, p, alpha, N);
    } else {
      for (int i = 0; i < N; i++) p[i] = r[i];
    }
    cpuSpMV(I, J, val, nnz, N, alpha, p, Ax);
    float dot = dotProduct(p, Ax, N);
    a = r1 / dot;
    saxpy(p, x, a, N);
    na = -a;
    saxpy(Ax, r, na, N);
    r0 = r1;
    r1 = dotProduct(r, r, N);
    if (trace) trace[k] = r1;
  }
}

extern "C" void ref_gen_tridiag_f32(int N, unsigned seed, int* I, int* J, float* val) {
  srand(seed);
  genTridiag<float, int>(I, J, val, N, 3 * N - 2);
}
extern "C" void ref_gen_tridiag_f64(int N, unsigned seed, int* I, int* J, double* val) {
  srand(seed);
  genTridiag<double, int>(I, J, val, N, 3 * N - 2);
}
