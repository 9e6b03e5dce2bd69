"""Generate cg_lap2d_2048.npz: the FP64 CG oracle on the 2D 5-point
Laplacian of a 2048 x 2048 grid (N = 4,194,304 rows, 20,963,328 nonzeros,
perks_gb300.matrices.laplacian_2d), right-hand side uniform [-1, 1) from
numpy default_rng(1), x0 = 0, stopped at ||r|| / ||b|| < 1e-10.

That solve takes 6.7k iterations, minutes on a CPU, so the GPU tests compare
against this fixture instead of running the oracle:

    python tests/golden/make_cg_fixture.py

Stored: the oracle's iteration count, its final recursive r.r and b.b, the
true relative residual ||b - A x|| / ||b|| of its solution recomputed in
FP64, and every 4096th entry of that solution.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from perks_gb300 import matrices as M  # noqa: E402

GRID = 2048
SEED = 1
TOL = 1e-10
SAMPLE = 4096


def problem():
    rp, ci, v = M.laplacian_2d(GRID)
    b = np.random.default_rng(SEED).uniform(-1, 1, len(rp) - 1)
    return rp, ci, v, b


def main():
    O.build()
    rp, ci, v, b = problem()
    t0 = time.time()
    x, it, rr, _ = O.cg(rp, ci, v, b, max_iter=50000, stop=1, tol=TOL)
    dt = time.time() - t0
    r = b - O.spmv_csr(rp, ci, v, x)
    rel = float(np.linalg.norm(r) / np.linalg.norm(b))
    out = os.path.join(HERE, "cg_lap2d_2048.npz")
    np.savez_compressed(out, iterations=np.int64(it), rr=np.float64(rr), bb=np.float64(b @ b),
                        true_rel_res=np.float64(rel), x_sample=x[::SAMPLE], sample=np.int64(SAMPLE),
                        grid=np.int64(GRID), seed=np.int64(SEED), tol=np.float64(TOL))
    print(f"{out}: {it} iterations, true relative residual {rel:.3e}, {dt:.0f} s")


if __name__ == "__main__":
    main()
