"""Generate the golden fixtures in this directory from the reference's own
CPU code (compiled unmodified from the reference sources into oracle/_ref by
oracle/Makefile). Run here, where the reference sources exist:

    python tests/golden/make_golden.py

Fixtures:
  stencil_golden.npz — for every shape and both precisions: a seeded input
      (numpy default_rng, uniform [0,1)) and the reference gold output after
      1, 2 and 7 steps; 2D fields 17x29, 3D fields 7x9x11 (clamped edges on
      every side, halo up to 6).
  cg_golden.npz — genTridiag(n=64, srand(3)) in float, rhs = 1, x0 = 0: the
      reference's float CG iterate x and r.r trace after 12 iterations (its
      own cpuSpMV/dotProduct/saxpy/scaleVector), the NaN pattern of the shipped
      cpuConjugateGrad after its fixed 10000 iterations, and the double
      genTridiag values for srand(7), n=32.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

STEPS = (1, 2, 7)
SEED = 20260101


def main():
    O.build()
    if not O.ref_available("2d5pt"):
        raise SystemExit("reference sources not available: oracle/_ref was not built")
    out = {}
    for i, shape in enumerate(O.SHAPES):
        for dt in (np.float32, np.float64):
            rng = np.random.default_rng(SEED + i)
            dims = (17, 29) if shape in O.SHAPES_2D else (7, 9, 11)
            f = rng.random(dims).astype(dt)
            tag = f"{shape}_{np.dtype(dt).name}"
            out[tag + "_in"] = f
            for s in STEPS:
                out[f"{tag}_s{s}"] = O.ref_stencil(shape, f, s)
    np.savez_compressed(os.path.join(HERE, "stencil_golden.npz"), **out)

    rp, ci, v = O.ref_gen_tridiag(64, 3, np.float32)
    b = np.ones(64, np.float32)
    x12, tr12 = O.ref_cg_steps(rp, ci, v, b, 12)
    xfull, maxiter = O.ref_cpu_cg(rp, ci, v, b)
    rp7, ci7, v7 = O.ref_gen_tridiag(32, 7, np.float64)
    np.savez_compressed(os.path.join(HERE, "cg_golden.npz"), row_ptr=rp, col=ci, val=v, rhs=b, x12=x12,
                        rr12=tr12, full_nan=np.isnan(xfull), full_iters=np.int64(maxiter), tri64_row_ptr=rp7,
                        tri64_col=ci7, tri64_val=v7)
    print("wrote", sorted(os.listdir(HERE)))


if __name__ == "__main__":
    main()
