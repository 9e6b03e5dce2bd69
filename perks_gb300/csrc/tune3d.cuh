// Measured launch parameters of the 3D stencil kernels on GB300, per dtype
// (0 FP32, 1 FP64), evaluation order (0 reference, 1 fast) and 3D shape
// (PERKS_3D7PT .. PERKS_POISSON): compute warps per CTA, rows per compute
// warp and KB of planes in flight. 0 keeps the built-in choice of
// stencil3d.cuh. `python -m perks_gb300.autotune --kind 3d` measures the
// candidates and rewrites the table below.
#pragma once

namespace perks {

struct Tune3D {
  int nwc, ry, dkb;
};

// clang-format off
// BEGIN TABLE
constexpr Tune3D kTune3D[2][2][5] = {
  {{{0, 0, 0}, {15, 4, 72}, {0, 0, 0}, {8, 4, 72}, {15, 4, 1}},
   {{11, 4, 72}, {15, 4, 72}, {15, 4, 72}, {15, 4, 72}, {15, 4, 1}}},
  {{{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}},
   {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}}}};
// END TABLE
// clang-format on

}  // namespace perks
