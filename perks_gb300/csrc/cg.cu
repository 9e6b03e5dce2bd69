// Conjugate gradient (CSR / DIA): persistent cooperative solver.
#include "runtime.cuh"

using namespace perks;

extern "C" {
void perks_cg_default_opts(perks_cg_opts* o) {
  if (!o) return;
  *o = perks_cg_opts{};
  o->dtype = PERKS_FP64;
  o->stop = PERKS_STOP_REL;
  o->tol = 1e-10;
  o->max_iter = 10000;
  o->kernel = PERKS_KERNEL_PERSISTENT;
}
int perks_cg_csr(int, int, const int*, const int*, const void*, const void*, void*, const perks_cg_opts*,
                 perks_cg_result*) {
  return fail(PERKS_ERR_UNSUPPORTED, "CG not built yet");
}
int perks_cg_dia(int, int, const int*, const void*, const void*, void*, const perks_cg_opts*, perks_cg_result*) {
  return fail(PERKS_ERR_UNSUPPORTED, "CG not built yet");
}
int perks_spmv_csr(int, int, int, const int*, const int*, const void*, const void*, void*, void*) {
  return fail(PERKS_ERR_UNSUPPORTED, "SpMV not built yet");
}
int perks_spmv_dia(int, int, int, const int*, const void*, const void*, void*, void*) {
  return fail(PERKS_ERR_UNSUPPORTED, "SpMV not built yet");
}
}
