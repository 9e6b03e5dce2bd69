"""The oracle (CPU restatement of the reference) against the reference's own
CPU code: committed golden fixtures always, the compiled reference sources
(oracle/_ref) when they exist on this machine."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
SHAPES = ["2d5pt", "2ds9pt", "2d13pt", "2d17pt", "2d21pt", "2ds25pt", "2d9pt", "2d25pt",
          "3d7pt", "3d13pt", "3d17pt", "3d27pt", "poisson"]


def bits_equal(a, b):
    return a.shape == b.shape and a.dtype == b.dtype and np.array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.fixture(scope="module")
def golden():
    return np.load(os.path.join(GOLD, "stencil_golden.npz"))


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("dt", ["float32", "float64"])
def test_oracle_matches_golden(oracle, golden, shape, dt):
    f = golden[f"{shape}_{dt}_in"]
    for s in (1, 2, 7):
        assert bits_equal(oracle.stencil(shape, f, s), golden[f"{shape}_{dt}_s{s}"]), (shape, dt, s)


@pytest.mark.parametrize("shape", SHAPES)
def test_oracle_matches_reference_build(oracle, shape):
    if not oracle.ref_available(shape):
        pytest.skip("reference sources not present on this machine")
    rng = np.random.default_rng(5)
    dims2 = [(1, 1), (1, 9), (9, 1), (6, 6), (13, 40)]
    dims3 = [(1, 1, 1), (2, 3, 4), (5, 6, 13), (9, 4, 3)]
    for dims in (dims2 if shape.startswith("2d") else dims3):
        for dt in (np.float32, np.float64):
            f = rng.random(dims).astype(dt)
            for s in (1, 3, 10):
                assert bits_equal(oracle.stencil(shape, f, s), oracle.ref_stencil(shape, f, s)), (shape, dims, dt, s)


def test_zero_steps_is_copy(oracle):
    f = np.random.default_rng(1).random((5, 7))
    assert bits_equal(oracle.stencil("2d5pt", f, 0), f)


def test_dirichlet_border_fixed(oracle):
    f = np.random.default_rng(2).random((20, 25))
    for shape in ("2d5pt", "2ds25pt", "2d25pt"):
        H = oracle.HALO[shape]
        g = oracle.stencil(shape, f, 3, boundary=1)
        m = np.ones_like(f, bool)
        m[H:-H, H:-H] = False
        assert np.array_equal(g[m], f[m])
        assert not np.array_equal(g[~m], f[~m])


def test_cg_float_matches_reference_golden(oracle):
    g = np.load(os.path.join(GOLD, "cg_golden.npz"))
    rp, ci, v, b = g["row_ptr"], g["col"], g["val"], g["rhs"]
    gp, gc, gv = oracle.gen_tridiag(64, 3, np.float32)
    assert np.array_equal(gp, rp) and np.array_equal(gc, ci) and bits_equal(gv, v)
    x, it, rr, tr = oracle.cg(rp, ci, v, b, max_iter=12, static_iter=True, trace=True)
    assert it == 12
    assert bits_equal(x, g["x12"])
    assert np.array_equal(tr, g["rr12"])
    # the shipped loop runs a fixed 10000 iterations and ends in 0/0
    x, it, rr, _ = oracle.cg(rp, ci, v, b, max_iter=int(g["full_iters"]), static_iter=True)
    assert np.array_equal(np.isnan(x), g["full_nan"])
    p7, c7, v7 = oracle.gen_tridiag(32, 7, np.float64)
    assert bits_equal(v7, g["tri64_val"]) and np.array_equal(p7, g["tri64_row_ptr"])


def test_cg_float_matches_reference_build(oracle):
    if not oracle.ref_available():
        pytest.skip("reference sources not present on this machine")
    for n, seed in ((10, 1), (100, 2), (257, 3)):
        rp, ci, v = oracle.ref_gen_tridiag(n, seed, np.float32)
        b = np.ones(n, np.float32)
        for k in (1, 5, 17):
            xr, trr = oracle.ref_cg_steps(rp, ci, v, b, k)
            xo, it, rr, tro = oracle.cg(rp, ci, v, b, max_iter=k, static_iter=True, trace=True)
            assert bits_equal(xr, xo) and np.array_equal(trr, tro, equal_nan=True)


def test_cg64_converges_and_stops(oracle):
    from perks_gb300 import matrices as Mx
    rp, ci, v = Mx.laplacian_2d(24)
    n = len(rp) - 1
    b = np.random.default_rng(3).uniform(-1, 1, n)
    x, it, rr, _ = oracle.cg(rp, ci, v, b, max_iter=2000, stop=1, tol=1e-10)
    assert it > 0
    res = b - oracle.spmv_csr(rp, ci, v, x)
    assert np.linalg.norm(res) / np.linalg.norm(b) < 2e-10
    # DIA form of the same matrix gives the same answer
    off, data = Mx.csr_to_dia(rp, ci, v)
    xd, itd, _ = oracle.cg_dia(off, data, b, max_iter=2000, stop=1, tol=1e-10)
    assert abs(itd - it) <= 1
    assert np.allclose(xd, x, rtol=1e-8, atol=1e-12)


def test_cg64_breakdown_on_indefinite(oracle):
    from perks_gb300 import matrices as Mx
    rp, ci, v = Mx.laplacian_2d(6)
    v = -v  # negative definite
    b = np.ones(len(rp) - 1)
    _, it, _, _ = oracle.cg(rp, ci, v, b, max_iter=100, stop=1, tol=1e-10)
    assert it == -1
