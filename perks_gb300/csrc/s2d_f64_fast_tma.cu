// 2D stencil kernels fed by TMA tensor copies, instantiated for double storage,
// fast (FMA) evaluation order.
#include "stencil2d_host.cuh"

namespace perks {
int stencil2d_f64_fast_tma(int shape, const perks_stencil_opts& o, const void* in, void* out, int wy, int wx,
                          int steps, perks_stencil_stats* st, bool host_io) {
  const double* i = static_cast<const double*>(in);
  double* q = static_cast<double*>(out);
  switch (shape) {
    case PERKS_2D5PT: return launch_stencil2d<double, PERKS_2D5PT, true, true>(o, i, q, wy, wx, steps, st, host_io);
    case PERKS_2DS9PT: return launch_stencil2d<double, PERKS_2DS9PT, true, true>(o, i, q, wy, wx, steps, st, host_io);
    case PERKS_2D13PT: return launch_stencil2d<double, PERKS_2D13PT, true, true>(o, i, q, wy, wx, steps, st, host_io);
    case PERKS_2D17PT: return launch_stencil2d<double, PERKS_2D17PT, true, true>(o, i, q, wy, wx, steps, st, host_io);
    case PERKS_2D21PT: return launch_stencil2d<double, PERKS_2D21PT, true, true>(o, i, q, wy, wx, steps, st, host_io);
    case PERKS_2DS25PT: return launch_stencil2d<double, PERKS_2DS25PT, true, true>(o, i, q, wy, wx, steps, st, host_io);
    case PERKS_2D9PT: return launch_stencil2d<double, PERKS_2D9PT, true, true>(o, i, q, wy, wx, steps, st, host_io);
    case PERKS_2D25PT: return launch_stencil2d<double, PERKS_2D25PT, true, true>(o, i, q, wy, wx, steps, st, host_io);
    default: return fail(PERKS_ERR_INVALID_ARG, "not a 2D shape: " + std::to_string(shape));
  }
}
}  // namespace perks
