// C ABI entry points (include/perks.h): argument checks, dtype/order
// dispatch, and the host-buffer drop-ins for the reference's
// jacobi_iterative / j3d_iterative.
#include <cuda_runtime.h>
#include <string>
#include "runtime.cuh"

namespace perks {
#define PERKS_DECL_2D(sfx)                                                                            \
  int stencil2d_##sfx(int shape, const perks_stencil_opts& o, const void* in, void* out, int wy, int wx, \
                      int steps, perks_stencil_stats* st, bool host_io);
PERKS_DECL_2D(f32_ref)
PERKS_DECL_2D(f32_fast)
PERKS_DECL_2D(f64_ref)
PERKS_DECL_2D(f64_fast)
PERKS_DECL_2D(f32_ref_tma)
PERKS_DECL_2D(f32_fast_tma)
PERKS_DECL_2D(f64_ref_tma)
PERKS_DECL_2D(f64_fast_tma)
#define PERKS_DECL_3D(sfx)                                                                              \
  int stencil3d_##sfx(int shape, const perks_stencil_opts& o, const void* in, void* out, int h, int wy, \
                      int wx, int steps, perks_stencil_stats* st, bool host_io);
PERKS_DECL_3D(f32_ref)
PERKS_DECL_3D(f32_fast)
PERKS_DECL_3D(f64_ref)
PERKS_DECL_3D(f64_fast)

static bool is2d(int s) { return s >= PERKS_2D5PT && s <= PERKS_2D25PT; }
static bool is3d(int s) { return s >= PERKS_3D7PT && s <= PERKS_POISSON; }

static int check_opts(const perks_stencil_opts* o, bool want3d) {
  if (!o) return fail(PERKS_ERR_INVALID_ARG, "opts is NULL");
  if (want3d ? !is3d(o->shape) : !is2d(o->shape))
    return fail(PERKS_ERR_INVALID_ARG, std::string("shape ") + std::to_string(o->shape) +
                                           (want3d ? " is not a 3D shape" : " is not a 2D shape"));
  if (o->dtype != PERKS_FP32 && o->dtype != PERKS_FP64)
    return fail(PERKS_ERR_INVALID_ARG, "stencil dtype must be PERKS_FP32 or PERKS_FP64");
  if (o->boundary != PERKS_BOUNDARY_CLAMP && o->boundary != PERKS_BOUNDARY_DIRICHLET)
    return fail(PERKS_ERR_INVALID_ARG, "unknown boundary mode");
  if (o->order != PERKS_ORDER_REFERENCE && o->order != PERKS_ORDER_FAST)
    return fail(PERKS_ERR_INVALID_ARG, "unknown evaluation order");
  if (o->kernel != PERKS_KERNEL_PERSISTENT && o->kernel != PERKS_KERNEL_PER_STEP &&
      !(o->kernel == PERKS_KERNEL_NAIVE && !want3d))
    return fail(PERKS_ERR_INVALID_ARG, "unknown kernel kind");
  if (o->tma != 0 && o->tma != 1) return fail(PERKS_ERR_INVALID_ARG, "tma must be 0 or 1");
  return PERKS_OK;
}

static int run2d(const perks_stencil_opts& o, const void* in, void* out, int wy, int wx, int steps,
                 perks_stencil_stats* st, bool host_io) {
  const bool fast = o.order == PERKS_ORDER_FAST;
  if (o.tma && o.kernel != PERKS_KERNEL_NAIVE) {
    if (o.dtype == PERKS_FP32)
      return fast ? stencil2d_f32_fast_tma(o.shape, o, in, out, wy, wx, steps, st, host_io)
                  : stencil2d_f32_ref_tma(o.shape, o, in, out, wy, wx, steps, st, host_io);
    return fast ? stencil2d_f64_fast_tma(o.shape, o, in, out, wy, wx, steps, st, host_io)
                : stencil2d_f64_ref_tma(o.shape, o, in, out, wy, wx, steps, st, host_io);
  }
  if (o.dtype == PERKS_FP32)
    return fast ? stencil2d_f32_fast(o.shape, o, in, out, wy, wx, steps, st, host_io)
                : stencil2d_f32_ref(o.shape, o, in, out, wy, wx, steps, st, host_io);
  return fast ? stencil2d_f64_fast(o.shape, o, in, out, wy, wx, steps, st, host_io)
              : stencil2d_f64_ref(o.shape, o, in, out, wy, wx, steps, st, host_io);
}

static int run3d(const perks_stencil_opts& o, const void* in, void* out, int h, int wy, int wx, int steps,
                 perks_stencil_stats* st, bool host_io) {
  const bool fast = o.order == PERKS_ORDER_FAST;
  if (o.dtype == PERKS_FP32)
    return fast ? stencil3d_f32_fast(o.shape, o, in, out, h, wy, wx, steps, st, host_io)
                : stencil3d_f32_ref(o.shape, o, in, out, h, wy, wx, steps, st, host_io);
  return fast ? stencil3d_f64_fast(o.shape, o, in, out, h, wy, wx, steps, st, host_io)
              : stencil3d_f64_ref(o.shape, o, in, out, h, wy, wx, steps, st, host_io);
}

// Host-buffer round trip used by the reference-signature drop-ins: the field
// is copied from h_in straight into the library's internal field and the
// result straight back into h_out (no staging buffers, nothing allocated per
// call once the workspace has grown to the field size).
template <class T>
static int host_roundtrip(const perks_stencil_opts& o, const T* h_in, T* h_out, int h, int wy, int wx,
                          int iteration, int usewarmup, int warmupiteration) {
  if ((long long)h * wy * wx > (1ll << 40)) return fail(PERKS_ERR_INVALID_ARG, "domain too large");
  int rc = PERKS_OK;
  const bool two = h == 1 && !is3d(o.shape);
  if (usewarmup) {
    const int wi = warmupiteration > 0 ? warmupiteration : iteration;
    rc = two ? run2d(o, h_in, h_out, wy, wx, wi, nullptr, true) : run3d(o, h_in, h_out, h, wy, wx, wi, nullptr, true);
  }
  if (rc == PERKS_OK)
    rc = two ? run2d(o, h_in, h_out, wy, wx, iteration, nullptr, true)
             : run3d(o, h_in, h_out, h, wy, wx, iteration, nullptr, true);
  return rc;
}

}  // namespace perks

using namespace perks;

extern "C" {

void perks_stencil_default_opts(perks_stencil_opts* o, int shape, int dtype) {
  if (!o) return;
  *o = perks_stencil_opts{};
  o->shape = shape;
  o->dtype = dtype;
  o->boundary = PERKS_BOUNDARY_CLAMP;
  o->order = PERKS_ORDER_REFERENCE;
  o->kernel = PERKS_KERNEL_PERSISTENT;
  // 2D: as many resident rows as fit. 3D: no resident planes -- measured
  // slower on GB300 in every regime (the plane copies stall the kernel's copy
  // ring more than the saved reads gain); cache_rows > 0 or -1 asks for them.
  o->cache_rows = is3d(shape) ? 0 : -1;
  o->l2_sweep = 0;
  o->tile_x = 0;
  o->tile_y = 0;
  o->ctas = 0;
  o->stream = nullptr;
}

int perks_stencil2d(const perks_stencil_opts* o, const void* d_in, void* d_out, int wy, int wx, int steps,
                    perks_stencil_stats* st) {
  int rc = check_opts(o, false);
  if (rc != PERKS_OK) return rc;
  if (!d_in || !d_out) return fail(PERKS_ERR_INVALID_ARG, "null device pointer");
  if (wy <= 0 || wx <= 0 || steps < 0) return fail(PERKS_ERR_INVALID_ARG, "sizes must be positive, steps >= 0");
  if ((long long)wy * wx > (1ll << 40)) return fail(PERKS_ERR_INVALID_ARG, "domain too large");
  return run2d(*o, d_in, d_out, wy, wx, steps, st, false);
}

int perks_stencil3d(const perks_stencil_opts* o, const void* d_in, void* d_out, int h, int wy, int wx, int steps,
                    perks_stencil_stats* st) {
  int rc = check_opts(o, true);
  if (rc != PERKS_OK) return rc;
  if (!d_in || !d_out) return fail(PERKS_ERR_INVALID_ARG, "null device pointer");
  if (h <= 0 || wy <= 0 || wx <= 0 || steps < 0)
    return fail(PERKS_ERR_INVALID_ARG, "sizes must be positive, steps >= 0");
  return run3d(*o, d_in, d_out, h, wy, wx, steps, st, false);
}

static int jacobi_common(int shape, int dtype, const void* h_in, int wy, int wx, void* h_out, int iteration,
                         int useSM, int usewarmup, int warmupiteration) {
  if (!is2d(shape)) return fail(PERKS_ERR_INVALID_ARG, "not a 2D shape");
  if (!h_in || !h_out) return fail(PERKS_ERR_INVALID_ARG, "null host pointer");
  if (wy <= 0 || wx <= 0 || iteration < 0) return fail(PERKS_ERR_INVALID_ARG, "bad sizes");
  perks_stencil_opts o;
  perks_stencil_default_opts(&o, shape, dtype);
  o.cache_rows = useSM ? -1 : 0;
  if (dtype == PERKS_FP32)
    return host_roundtrip<float>(o, static_cast<const float*>(h_in), static_cast<float*>(h_out), 1, wy, wx,
                                 iteration, usewarmup, warmupiteration);
  return host_roundtrip<double>(o, static_cast<const double*>(h_in), static_cast<double*>(h_out), 1, wy, wx,
                                iteration, usewarmup, warmupiteration);
}

int perks_jacobi_iterative_f32(int shape, const float* h_in, int wy, int wx, float* h_out, int, int, int iteration,
                               int, int useSM, int usewarmup, int warmupiteration, int) {
  return jacobi_common(shape, PERKS_FP32, h_in, wy, wx, h_out, iteration, useSM, usewarmup, warmupiteration);
}
int perks_jacobi_iterative_f64(int shape, const double* h_in, int wy, int wx, double* h_out, int, int,
                               int iteration, int, int useSM, int usewarmup, int warmupiteration, int) {
  return jacobi_common(shape, PERKS_FP64, h_in, wy, wx, h_out, iteration, useSM, usewarmup, warmupiteration);
}

static int j3d_common(int shape, int dtype, const void* h_in, int h, int wy, int wx, void* h_out, int iteration,
                      int useSM, int usewarmup, int warmupiteration, int getminHeight) {
  if (!is3d(shape)) return fail(PERKS_ERR_INVALID_ARG, "not a 3D shape");
  if (getminHeight) {  // the largest height whose every run-interior plane stays on chip (0: none fits)
    perks_stencil_opts o;
    perks_stencil_default_opts(&o, shape, dtype);
    o.cache_rows = useSM ? -1 : 0;
    int hm = 0;
    const int rc = perks_stencil3d_min_domain(&o, wy, wx, &hm);
    return rc == PERKS_OK ? hm : rc;
  }
  if (!h_in || !h_out) return fail(PERKS_ERR_INVALID_ARG, "null host pointer");
  if (wy <= 0 || wx <= 0) return -2;  // reference: unsupported widths
  if (h <= 0) return -4;              // reference: height too small
  if (iteration < 0) return fail(PERKS_ERR_INVALID_ARG, "bad iteration count");
  perks_stencil_opts o;
  perks_stencil_default_opts(&o, shape, dtype);
  o.cache_rows = useSM ? -1 : 0;
  if (dtype == PERKS_FP32)
    return host_roundtrip<float>(o, static_cast<const float*>(h_in), static_cast<float*>(h_out), h, wy, wx,
                                 iteration, usewarmup, warmupiteration);
  return host_roundtrip<double>(o, static_cast<const double*>(h_in), static_cast<double*>(h_out), h, wy, wx,
                                iteration, usewarmup, warmupiteration);
}

int perks_j3d_iterative_f32(int shape, const float* h_in, int h, int wy, int wx, float* h_out, int, int,
                            int iteration, int useSM, int usewarmup, int warmupiteration, int, int getminHeight) {
  return j3d_common(shape, PERKS_FP32, h_in, h, wy, wx, h_out, iteration, useSM, usewarmup, warmupiteration,
                    getminHeight);
}
int perks_j3d_iterative_f64(int shape, const double* h_in, int h, int wy, int wx, double* h_out, int, int,
                            int iteration, int useSM, int usewarmup, int warmupiteration, int, int getminHeight) {
  return j3d_common(shape, PERKS_FP64, h_in, h, wy, wx, h_out, iteration, useSM, usewarmup, warmupiteration,
                    getminHeight);
}

}  // extern "C"
