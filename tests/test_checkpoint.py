"""Checkpoint / resume of the two iterative paths.

CG: a solve that stops (iteration cap) and resumes from its perks_cg_state
must give bit-identical x, r and p to one uninterrupted solve with the same
options, for both kernels, FP64 and FP32, CSR and DIA input. The stencil time
loop needs no extra state: its checkpoint is the field, and a run split into
two calls must match one call bit for bit."""
import numpy as np
import pytest

from test_stencil_gpu import bits_equal, run

pytestmark = pytest.mark.gpu


def _problem(fmt):
    from perks_gb300 import matrices as M
    rp, ci, v = M.shifted(*M.laplacian_2d(64), 0.05)
    b = np.random.default_rng(5).uniform(-1, 1, len(rp) - 1)
    return (rp, ci, v), b, fmt


def _solve(native, cuda, prob, dtype, x0=None, **kw):
    (rp, ci, v), b, fmt = prob
    if fmt == "csr":
        return native.cg_csr(rp, ci, v, b, x0, dtype=dtype, device=cuda, **kw)
    from perks_gb300 import matrices as M
    off, data = M.csr_to_dia(rp, ci, v)
    return native.cg_dia(off, data, b, x0, dtype=dtype, device=cuda, **kw)


@pytest.mark.parametrize("fmt", ["csr", "dia"])
@pytest.mark.parametrize("kernel", ["persistent", "per_step"])
@pytest.mark.parametrize("dtype", ["fp64", "fp32", "mixed"])
def test_cg_resume_static_bit_exact(native, cuda, dtype, kernel, fmt):
    if dtype == "mixed" and kernel == "per_step":
        pytest.skip("mixed precision runs in the persistent kernel only")
    prob = _problem(fmt)
    full = native.CgCheckpoint()
    x_full, res = _solve(native, cuda, prob, dtype, max_iter=60, static_iter=True, kernel=kernel, checkpoint=full)
    assert res["iterations"] == 60 and full.k == 60
    ck = native.CgCheckpoint()
    x1, r1 = _solve(native, cuda, prob, dtype, max_iter=23, static_iter=True, kernel=kernel, checkpoint=ck)
    assert r1["iterations"] == 23 and ck.k == 23
    # through host memory, as a checkpoint written to disk would go
    ck2 = native.CgCheckpoint.from_host(ck.to_host(), device=cuda)
    x2, r2 = _solve(native, cuda, prob, dtype, x0=x1, max_iter=60, static_iter=True, kernel=kernel,
                    checkpoint=ck2)
    assert r2["iterations"] == 60 and ck2.k == 60
    pairs = [(x2, x_full), (ck2.r, full.r), (ck2.p, full.p)] + ([(ck2.xs, full.xs)] if dtype == "mixed" else [])
    for a, b in pairs:
        assert bits_equal(a.cpu().numpy(), b.cpu().numpy())
    assert r2["rr"] == res["rr"] and ck2.state.rr_prev == full.state.rr_prev
    assert ck2.state.outer == full.state.outer and ck2.state.maxrr == full.state.maxrr


@pytest.mark.parametrize("kernel", ["persistent", "per_step"])
@pytest.mark.parametrize("dtype", ["fp64", "fp32", "mixed"])
def test_cg_resume_after_cap(native, cuda, dtype, kernel):
    if dtype == "mixed" and kernel == "per_step":
        pytest.skip("mixed precision runs in the persistent kernel only")
    prob = _problem("csr")
    tol = 1e-4 if dtype == "fp32" else 1e-10
    x_full, res = _solve(native, cuda, prob, dtype, tol=tol, kernel=kernel)
    K = res["iterations"]
    ck = native.CgCheckpoint()
    x1, r1 = _solve(native, cuda, prob, dtype, tol=tol, kernel=kernel, max_iter=K // 2, check=False,
                    checkpoint=ck)
    assert r1["status"] != 0 and ck.k == K // 2  # stopped by the cap, state saved
    x2, r2 = _solve(native, cuda, prob, dtype, x0=x1, tol=tol, kernel=kernel, checkpoint=ck)
    assert r2["iterations"] == K and ck.k == K
    assert bits_equal(x2.cpu().numpy(), x_full.cpu().numpy())
    # a converged state resumes to no further work
    x3, r3 = _solve(native, cuda, prob, dtype, x0=x2, tol=tol, kernel=kernel, checkpoint=ck)
    assert r3["iterations"] == K and bits_equal(x3.cpu().numpy(), x_full.cpu().numpy())


@pytest.mark.parametrize("kernel", ["persistent", "per_step"])
@pytest.mark.parametrize("fmt", ["csr", "dia"])
def test_cg_resume_matches_oracle(native, cuda, oracle, kernel, fmt):
    """A solve stopped by its iteration cap halfway and resumed from the
    checkpoint ends where the FP64 oracle's uninterrupted solve ends: the same
    iteration count (within 1), a true relative residual below the tolerance
    recomputed on the host with the oracle's SpMV, and the oracle's solution
    (this shifted Laplacian is well conditioned, so solutions that meet the
    tolerance agree closely)."""
    prob = _problem(fmt)
    (rp, ci, v), b, _ = prob
    xo, it, _, _ = oracle.cg(rp, ci, v, b, max_iter=5000, stop=1, tol=1e-10)
    ck = native.CgCheckpoint()
    x1, r1 = _solve(native, cuda, prob, "fp64", tol=1e-10, kernel=kernel, max_iter=it // 2, check=False,
                    checkpoint=ck)
    assert r1["status"] == -18 and ck.k == it // 2
    ck2 = native.CgCheckpoint.from_host(ck.to_host(), device=cuda)
    x2, r2 = _solve(native, cuda, prob, "fp64", x0=x1.cpu().numpy(), tol=1e-10, kernel=kernel, checkpoint=ck2)
    assert abs(r2["iterations"] - it) <= 1, (r2, it)
    x = x2.cpu().numpy()
    r = b - oracle.spmv_csr(rp, ci, v, x)
    assert np.linalg.norm(r) / np.linalg.norm(b) <= 1e-10 * 1.05
    assert np.allclose(x, xo, rtol=1e-8, atol=1e-10)


def test_cg_checkpoint_rejects_misuse(native, cuda):
    prob = _problem("csr")
    ck = native.CgCheckpoint()
    _solve(native, cuda, prob, "fp64", max_iter=5, static_iter=True, kernel="persistent", checkpoint=ck)
    with pytest.raises(native.PerksError):  # written by the persistent kernel
        _solve(native, cuda, prob, "fp64", max_iter=9, static_iter=True, kernel="per_step", checkpoint=ck)
    with pytest.raises(ValueError):  # FP64 state, FP32 solve
        _solve(native, cuda, prob, "fp32", checkpoint=ck)
    with pytest.raises(ValueError):  # FP64 state, mixed solve (FP32 r and p)
        _solve(native, cuda, prob, "mixed", checkpoint=ck)


@pytest.mark.parametrize("shape,dt", [("2ds9pt", np.float32), ("2d9pt", np.float64), ("3d7pt", np.float32),
                                      ("3d27pt", np.float64)])
@pytest.mark.parametrize("boundary", ["clamp", "dirichlet"])
def test_stencil_split_run_bit_exact(native, cuda, shape, dt, boundary):
    rng = np.random.default_rng(9)
    f = rng.random((300, 517) if shape.startswith("2d") else (40, 50, 70)).astype(dt)
    full, _ = run(native, cuda, f, shape, 9, boundary=boundary)
    half, _ = run(native, cuda, f, shape, 4, boundary=boundary)
    rest, _ = run(native, cuda, half, shape, 5, boundary=boundary, l2_sweep=True)
    assert bits_equal(rest, full)
