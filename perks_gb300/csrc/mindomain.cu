// Minimum-domain queries: the reference's --small mode
// (stencil/2dstencil/jacobi.driver.cpp:84-109 calls getMinWidthY,
// stencil/2dstencil/jacobi-2d.cu:79-136, and runs the stencil at the width_y
// it returns). The answer is the largest domain that the persistent kernel
// keeps on chip between time steps, used to report all-on-chip throughput.
// Host arithmetic only; it reads the device's SM count and shared memory.
#include <string>
#include "stencil2d_host.cuh"
#include "stencil3d_host.cuh"

namespace perks {

template <class T, int SHAPE>
static int min_rows(const perks_stencil_opts& o, int wx, int* wy) {
  return o.order == PERKS_ORDER_FAST ? min_domain_rows<Cfg2D<T, SHAPE, true>>(o, wx, wy)
                                     : min_domain_rows<Cfg2D<T, SHAPE, false>>(o, wx, wy);
}

template <class T>
static int min_domain_2d(int shape, const perks_stencil_opts& o, int wx, int* wy) {
  switch (shape) {
    case PERKS_2D5PT: return min_rows<T, PERKS_2D5PT>(o, wx, wy);
    case PERKS_2DS9PT: return min_rows<T, PERKS_2DS9PT>(o, wx, wy);
    case PERKS_2D13PT: return min_rows<T, PERKS_2D13PT>(o, wx, wy);
    case PERKS_2D17PT: return min_rows<T, PERKS_2D17PT>(o, wx, wy);
    case PERKS_2D21PT: return min_rows<T, PERKS_2D21PT>(o, wx, wy);
    case PERKS_2DS25PT: return min_rows<T, PERKS_2DS25PT>(o, wx, wy);
    case PERKS_2D9PT: return min_rows<T, PERKS_2D9PT>(o, wx, wy);
    case PERKS_2D25PT: return min_rows<T, PERKS_2D25PT>(o, wx, wy);
    default: return fail(PERKS_ERR_INVALID_ARG, "not a 2D shape: " + std::to_string(shape));
  }
}

template <class T, int SHAPE>
static int min_planes(const perks_stencil_opts& o, int wy, int wx, int* h) {
  return o.order == PERKS_ORDER_FAST ? min_domain_planes<Cfg3D<T, SHAPE, true>>(o, wy, wx, h)
                                     : min_domain_planes<Cfg3D<T, SHAPE, false>>(o, wy, wx, h);
}

template <class T>
static int min_domain_3d(int shape, const perks_stencil_opts& o, int wy, int wx, int* h) {
  switch (shape) {
    case PERKS_3D7PT: return min_planes<T, PERKS_3D7PT>(o, wy, wx, h);
    case PERKS_3D13PT: return min_planes<T, PERKS_3D13PT>(o, wy, wx, h);
    case PERKS_3D17PT: return min_planes<T, PERKS_3D17PT>(o, wy, wx, h);
    case PERKS_3D27PT: return min_planes<T, PERKS_3D27PT>(o, wy, wx, h);
    case PERKS_POISSON: return min_planes<T, PERKS_POISSON>(o, wy, wx, h);
    default: return fail(PERKS_ERR_INVALID_ARG, "not a 3D shape: " + std::to_string(shape));
  }
}

}  // namespace perks

using namespace perks;

extern "C" {

int perks_stencil2d_min_domain(const perks_stencil_opts* o, int wx, int* wy) {
  if (!o || !wy) return fail(PERKS_ERR_INVALID_ARG, "NULL argument");
  if (o->dtype != PERKS_FP32 && o->dtype != PERKS_FP64)
    return fail(PERKS_ERR_INVALID_ARG, "stencil dtype must be PERKS_FP32 or PERKS_FP64");
  if (o->kernel != PERKS_KERNEL_PERSISTENT && o->kernel != PERKS_KERNEL_PER_STEP)
    return fail(PERKS_ERR_INVALID_ARG, "unknown kernel kind");
  if (o->order != PERKS_ORDER_REFERENCE && o->order != PERKS_ORDER_FAST)
    return fail(PERKS_ERR_INVALID_ARG, "unknown evaluation order");
  if (wx <= 0) return fail(PERKS_ERR_INVALID_ARG, "width_x must be positive");
  *wy = 0;
  return o->dtype == PERKS_FP32 ? min_domain_2d<float>(o->shape, *o, wx, wy)
                                : min_domain_2d<double>(o->shape, *o, wx, wy);
}

int perks_get_min_width_y(int shape, int dtype, int wx, int, int, int useSM, int, int) {
  perks_stencil_opts o;
  perks_stencil_default_opts(&o, shape, dtype);
  o.cache_rows = useSM ? -1 : 0;
  int wy = 0;
  const int rc = perks_stencil2d_min_domain(&o, wx, &wy);
  return rc == PERKS_OK ? wy : rc;
}

int perks_stencil3d_min_domain(const perks_stencil_opts* o, int wy, int wx, int* h) {
  if (!o || !h) return fail(PERKS_ERR_INVALID_ARG, "NULL argument");
  if (o->dtype != PERKS_FP32 && o->dtype != PERKS_FP64)
    return fail(PERKS_ERR_INVALID_ARG, "stencil dtype must be PERKS_FP32 or PERKS_FP64");
  if (o->order != PERKS_ORDER_REFERENCE && o->order != PERKS_ORDER_FAST)
    return fail(PERKS_ERR_INVALID_ARG, "unknown evaluation order");
  if (wy <= 0 || wx <= 0) return fail(PERKS_ERR_INVALID_ARG, "width_y and width_x must be positive");
  *h = 0;
  return o->dtype == PERKS_FP32 ? min_domain_3d<float>(o->shape, *o, wy, wx, h)
                                : min_domain_3d<double>(o->shape, *o, wy, wx, h);
}

}  // extern "C"
