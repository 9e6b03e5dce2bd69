// Measured launch parameters of the 2D stencil kernels on GB300, per dtype
// (0 FP32, 1 FP64), evaluation order (0 reference, 1 fast) and 2D shape
// (PERKS_2D5PT .. PERKS_2D25PT): warps per CTA, rows in flight per warp, the
// division form of divconst.cuh, rows per copy wait and 16-byte vectors per
// lane. 0 in nw, d, rp or nv keeps the built-in choice of stencil2d.cuh. `python -m perks_gb300.autotune` measures the candidates
// and rewrites the table below.
#pragma once

namespace perks {

struct Tune2D {
  int nw, d, fin, rp, nv;  // rp 0 = one row per copy wait; nv 0 = built-in vectors per lane
};

// clang-format off
// BEGIN TABLE
constexpr Tune2D kTune2D[2][2][8] = {
  {{{16, 4, 1, 0, 0}, {0, 0, 3, 0, 0}, {0, 0, 3, 0, 0}, {0, 0, 3, 0, 0}, {0, 0, 2, 0, 0}, {8, 6, 3, 1, 1}, {0, 0, 0, 0, 0}, {0, 0, 0, 0, 0}},
   {{8, 4, 0, 0, 0}, {8, 6, 0, 0, 0}, {12, 6, 0, 2, 0}, {12, 6, 0, 0, 0}, {12, 4, 0, 0, 0}, {16, 6, 0, 1, 1}, {8, 4, 0, 0, 0}, {12, 4, 0, 0, 0}}},
  {{{0, 0, 0, 0, 0}, {0, 0, 0, 0, 0}, {0, 0, 0, 0, 0}, {8, 4, 1, 0, 0}, {12, 6, 0, 0, 0}, {12, 4, 0, 1, 0}, {0, 0, 0, 0, 0}, {0, 0, 0, 0, 0}},
   {{0, 0, 0, 0, 0}, {0, 0, 0, 0, 0}, {0, 0, 0, 0, 0}, {0, 0, 0, 0, 0}, {12, 4, 0, 1, 0}, {0, 0, 0, 0, 0}, {0, 0, 0, 0, 0}, {0, 0, 0, 0, 0}}}};
// END TABLE
// clang-format on

}  // namespace perks
