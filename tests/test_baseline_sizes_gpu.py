"""Parity at the benchmark configurations' own sizes.

* Plain 2D 5-point Jacobi in FP64 on 1024 x 1024 cells with the reference's
  clamp boundary (its driver's own check, stencil/2dstencil/jacobi.driver.cpp:
  164-184) and on 1026 x 1026 cells whose outer ring is a fixed Dirichlet
  border, at 785 and 1000 time steps: bit-identical to the oracle through the
  device entry point (persistent and one launch per step) and through the
  reference-signature host drop-in. At 1000 steps the clamp field is zero
  everywhere: it decays through the subnormal range near step 790.
* The headline field: 2ds9pt FP32 on 8192 x 8192 cells, 20 steps, the
  persistent kernel as benchmarked (and one launch per step): bit-identical
  to the oracle over the whole field.
* CG at the configuration sizes, FP64 and mixed precision, right-hand side
  uniform [-1, 1) from seed 1, x0 = 0, stop at ||r|| / ||b|| < 1e-10: the
  iteration count of the FP64 solve against the FP64 oracle (within 1, or 1%
  for solves of hundreds of iterations and more: the GPU sums dot products in
  another order), and the true relative residual of every solution
  recomputed on the host in FP64 with the oracle's SpMV, not with the
  library. The 3D 7-point Laplacian on 160^3 cells and the random SPD matrix
  with n = 1e6 run the oracle here; the 2048^2 Laplacian (6.7k iterations)
  compares against tests/golden/cg_lap2d_2048.npz, made by
  tests/golden/make_cg_fixture.py.
"""
import os

import numpy as np
import pytest

from test_stencil_gpu import bits_equal, run

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
TOL = 1e-10


def it_close(a, b):
    return abs(a - b) <= max(1, int(0.01 * max(a, b)))


@pytest.fixture(scope="module")
def config1_field():
    return np.random.default_rng(1).random((1026, 1026))


@pytest.mark.parametrize("steps", [785, 1000])
@pytest.mark.parametrize("boundary", ["clamp", "dirichlet"])
def test_config1_2d5pt_fp64(native, cuda, oracle, config1_field, steps, boundary):
    f = config1_field[1:-1, 1:-1].copy() if boundary == "clamp" else config1_field
    ref = oracle.stencil("2d5pt", f, steps, boundary=0 if boundary == "clamp" else 1)
    if boundary == "clamp":
        # all zero at 1000 steps, as the reference's own run ends; not yet at 785
        assert ref.any() == (steps == 785)
    else:
        assert np.array_equal(ref[0], f[0]) and np.array_equal(ref[:, -1], f[:, -1])  # the fixed border
    for kernel in ("persistent", "per_step"):
        g, st = run(native, cuda, f, "2d5pt", steps, kernel=kernel, boundary=boundary)
        assert bits_equal(g, ref), (boundary, steps, kernel)
    if boundary == "clamp":
        out = np.full_like(f, np.nan)
        rc = native.jacobi_iterative(f, f.shape[0], f.shape[1], out, iteration=steps, shape="2d5pt")
        assert rc == 0, native.last_error()
        assert bits_equal(out, ref)


def test_headline_field_full_8192(native, cuda, oracle):
    import torch
    steps = 20
    g = torch.Generator(device="cpu").manual_seed(1234)
    f = torch.rand((8192, 8192), generator=g, dtype=torch.float32)
    ref = oracle.stencil("2ds9pt", f.numpy(), steps)
    d = f.to(cuda)
    for kw in ({"kernel": "persistent", "l2_sweep": False}, {"kernel": "per_step"}):
        out, st = native.stencil2d(d, "2ds9pt", steps, order="reference", **kw)
        torch.cuda.synchronize()
        assert bits_equal(out.cpu().numpy(), ref), kw
        del out


def _host_true_rel(oracle, rp, ci, v, b, x):
    r = b - oracle.spmv_csr(rp, ci, np.asarray(v, np.float64), np.asarray(x.cpu().numpy(), np.float64))
    return float(np.linalg.norm(r) / np.linalg.norm(b))


def _cg_case(native, cuda, oracle, rp, ci, v, b, it_ref):
    its = {}
    for dt in ("fp64", "mixed"):
        x, res = native.cg_csr(rp, ci, v, b, dtype=dt, tol=TOL, device=cuda)
        rel = _host_true_rel(oracle, rp, ci, v, b, x)
        assert rel <= TOL * 1.05, (dt, rel, res)
        its[dt] = res["iterations"]
        del x
    assert it_close(its["fp64"], it_ref), (its, it_ref)
    return its


def test_cg_lap3d_160(native, cuda, oracle):
    from perks_gb300 import matrices as M
    rp, ci, v = M.laplacian_3d(160)
    b = np.random.default_rng(1).uniform(-1, 1, len(rp) - 1)
    xo, it, _, _ = oracle.cg(rp, ci, v, b, max_iter=20000, stop=1, tol=TOL)
    assert _host_true_rel(oracle, rp, ci, v, b, _Host(xo)) <= TOL
    _cg_case(native, cuda, oracle, rp, ci, v, b, it)


def test_cg_random_spd_1e6(native, cuda, oracle):
    from perks_gb300 import matrices as M
    rp, ci, v = M.random_spd(1_000_000, 7)
    b = np.random.default_rng(1).uniform(-1, 1, len(rp) - 1)
    xo, it, _, _ = oracle.cg(rp, ci, v, b, max_iter=20000, stop=1, tol=TOL)
    _cg_case(native, cuda, oracle, rp, ci, v, b, it)


def test_cg_lap2d_2048_vs_fixture(native, cuda, oracle):
    from perks_gb300 import matrices as M
    fx = np.load(os.path.join(HERE, "golden", "cg_lap2d_2048.npz"))
    rp, ci, v = M.laplacian_2d(int(fx["grid"]))
    b = np.random.default_rng(int(fx["seed"])).uniform(-1, 1, len(rp) - 1)
    # the same right-hand side as the fixture's (b.b to rounding: numpy's dot
    # sums in a machine-dependent order)
    assert abs(float(b @ b) - float(fx["bb"])) <= 1e-12 * float(fx["bb"])
    its = _cg_case(native, cuda, oracle, rp, ci, v, b, int(fx["iterations"]))
    # DIA input of the same matrix
    off, data = M.csr_to_dia(rp, ci, v)
    x, res = native.cg_dia(off, data, b, dtype="fp64", tol=TOL, device=cuda)
    assert it_close(res["iterations"], int(fx["iterations"]))
    assert _host_true_rel(oracle, rp, ci, v, b, x) <= TOL * 1.05
    assert its["mixed"] > 0


class _Host:
    """A numpy vector with the .cpu().numpy() of a tensor."""

    def __init__(self, a):
        self.a = a

    def cpu(self):
        return self

    def numpy(self):
        return self.a
