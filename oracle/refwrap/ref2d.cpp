// Reference-side shim (test infrastructure): compiles one of the reference's
// unmodified 2D CPU gold files (passed in as REF_SRC by oracle/Makefile) and
// exports its jacobi_gold_iterative<float/double> under C names for ctypes.
#include REF_SRC
extern "C" void ref_stencil2d_f32(float* in, int wy, int wx, float* out, int it) {
  jacobi_gold_iterative<float>(in, wy, wx, out, it);
}
extern "C" void ref_stencil2d_f64(double* in, int wy, int wx, double* out, int it) {
  jacobi_gold_iterative<double>(in, wy, wx, out, it);
}
