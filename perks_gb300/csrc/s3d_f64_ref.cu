// 3D stencil kernels instantiated for double storage, reference evaluation order.
#include "stencil3d_host.cuh"

namespace perks {
int stencil3d_f64_ref(int shape, const perks_stencil_opts& o, const void* in, void* out, int h, int wy,
                          int wx, int steps, perks_stencil_stats* st, bool host_io) {
  const double* i = static_cast<const double*>(in);
  double* q = static_cast<double*>(out);
  switch (shape) {
    case PERKS_3D7PT: return launch_stencil3d<double, PERKS_3D7PT, false>(o, i, q, h, wy, wx, steps, st, host_io);
    case PERKS_3D13PT: return launch_stencil3d<double, PERKS_3D13PT, false>(o, i, q, h, wy, wx, steps, st, host_io);
    case PERKS_3D17PT: return launch_stencil3d<double, PERKS_3D17PT, false>(o, i, q, h, wy, wx, steps, st, host_io);
    case PERKS_3D27PT: return launch_stencil3d<double, PERKS_3D27PT, false>(o, i, q, h, wy, wx, steps, st, host_io);
    case PERKS_POISSON: return launch_stencil3d<double, PERKS_POISSON, false>(o, i, q, h, wy, wx, steps, st, host_io);
    default: return fail(PERKS_ERR_INVALID_ARG, "not a 3D shape: " + std::to_string(shape));
  }
}
}  // namespace perks
