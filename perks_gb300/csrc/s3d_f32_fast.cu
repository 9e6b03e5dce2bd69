// 3D stencil kernels instantiated for float storage, fast (FMA) evaluation order.
#include "stencil3d_host.cuh"

namespace perks {
int stencil3d_f32_fast(int shape, const perks_stencil_opts& o, const void* in, void* out, int h, int wy,
                          int wx, int steps, perks_stencil_stats* st, bool host_io) {
  const float* i = static_cast<const float*>(in);
  float* q = static_cast<float*>(out);
  switch (shape) {
    case PERKS_3D7PT: return launch_stencil3d<float, PERKS_3D7PT, true>(o, i, q, h, wy, wx, steps, st, host_io);
    case PERKS_3D13PT: return launch_stencil3d<float, PERKS_3D13PT, true>(o, i, q, h, wy, wx, steps, st, host_io);
    case PERKS_3D17PT: return launch_stencil3d<float, PERKS_3D17PT, true>(o, i, q, h, wy, wx, steps, st, host_io);
    case PERKS_3D27PT: return launch_stencil3d<float, PERKS_3D27PT, true>(o, i, q, h, wy, wx, steps, st, host_io);
    case PERKS_POISSON: return launch_stencil3d<float, PERKS_POISSON, true>(o, i, q, h, wy, wx, steps, st, host_io);
    default: return fail(PERKS_ERR_INVALID_ARG, "not a 3D shape: " + std::to_string(shape));
  }
}
}  // namespace perks
