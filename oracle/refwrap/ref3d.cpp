// Reference-side shim (test infrastructure): compiles one of the reference's
// unmodified 3D CPU gold files (REF_SRC) and exports j3d_gold_iterative.
#include REF_SRC
extern "C" void ref_stencil3d_f32(float* in, int h, int wy, int wx, float* out, int it) {
  j3d_gold_iterative<float>(in, h, wy, wx, out, it);
}
extern "C" void ref_stencil3d_f64(double* in, int h, int wy, int wx, double* out, int it) {
  j3d_gold_iterative<double>(in, h, wy, wx, out, it);
}
