"""Device-side timeout path of the persistent kernels.

Every device-side wait (grid barrier, batch job barrier, bulk-copy mbarrier)
gives up after a clock budget, records an error bit in the kernel's status
word and leaves the kernel; the host maps that to PERKS_ERR_TIMEOUT and the
CUDA context stays usable. These tests shorten the budget to about 100 us
and make one CTA skip its first grid-barrier arrival, so the barrier can
never complete and every waiting CTA's budget runs out: the call must return
PERKS_ERR_TIMEOUT, and the next normal call must be bit-exact against the
oracle. No test faults, traps or hangs the GPU: each wait ends after its
budget."""
import contextlib

import numpy as np
import pytest

from test_stencil_gpu import bits_equal, run

pytestmark = pytest.mark.gpu

TIMEOUT = -15
BUDGET = 200_000  # SM clock cycles, about 100 us at 2 GHz


@contextlib.contextmanager
def wait_fault(native, skip_cta=0, budget=BUDGET):
    L = native.lib()
    assert L.perks_debug_set_wait_fault(budget, skip_cta) == 0
    try:
        yield
    finally:
        L.perks_debug_set_wait_fault(0, -1)


@pytest.mark.parametrize("shape,dims,dt", [("2ds9pt", (300, 1100), np.float32), ("2d5pt", (200, 700), np.float64),
                                           ("3d7pt", (20, 40, 70), np.float32), ("3d27pt", (16, 30, 70), np.float64)])
@pytest.mark.parametrize("skip_cta", [0, 5])
def test_stencil_barrier_timeout(native, cuda, oracle, shape, dims, dt, skip_cta):
    import torch
    f = np.random.default_rng(3).random(dims).astype(dt)
    t = torch.from_numpy(f).to(cuda)
    fn = native.stencil2d if len(dims) == 2 else native.stencil3d
    with wait_fault(native, skip_cta):
        with pytest.raises(native.PerksError) as e:
            fn(t, shape, 4, kernel="persistent")
    assert e.value.code == TIMEOUT, str(e.value)
    assert "budget" in native.last_error()
    g, _ = run(native, cuda, f, shape, 4)
    assert bits_equal(g, oracle.stencil(shape, f, 4))


@pytest.mark.parametrize("shape", ["3d7pt", "3d27pt"])
def test_stencil3d_resident_barrier_timeout(native, cuda, oracle, shape):
    """With resident planes (few CTAs, long z-runs) the 3D kernel leaves
    cleanly on a barrier timeout and writes none of its planes back."""
    import torch
    f = np.random.default_rng(9).random((40, 50, 70)).astype(np.float32)
    t = torch.from_numpy(f).to(cuda)
    with wait_fault(native, 1):
        with pytest.raises(native.PerksError) as e:
            native.stencil3d(t, shape, 4, kernel="persistent", ctas=3, cache_rows=-1)
    assert e.value.code == TIMEOUT, str(e.value)
    g, st = run(native, cuda, f, shape, 4, kernel="persistent", ctas=3, cache_rows=-1)
    assert st["cached_rows"] > 0
    assert bits_equal(g, oracle.stencil(shape, f, 4))


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_stencil_tma_barrier_timeout(native, cuda, oracle, dt):
    """The TMA-fed 2D kernel leaves cleanly when the grid barrier times out
    (no tensor copy is in flight between steps)."""
    import torch
    f = np.random.default_rng(8).random((300, 1100)).astype(dt)
    t = torch.from_numpy(f).to(cuda)
    with wait_fault(native, 5):
        with pytest.raises(native.PerksError) as e:
            native.stencil2d(t, "2ds9pt", 4, kernel="persistent", tma=True)
    assert e.value.code == TIMEOUT, str(e.value)
    g, _ = run(native, cuda, f, "2ds9pt", 4, tma=True)
    assert bits_equal(g, oracle.stencil("2ds9pt", f, 4))


@pytest.mark.parametrize("dtype,cluster", [("fp64", 1), ("mixed", 1), ("fp32", 1), ("fp64", 4), ("mixed", 8)])
def test_cg_barrier_timeout(native, cuda, oracle, dtype, cluster):
    """With clusters the hook makes one cluster's leader skip its arrival;
    every cluster barrier is still passed by all CTAs of a cluster."""
    from perks_gb300 import matrices as M
    rp, ci, v = M.laplacian_2d(64)
    b = np.random.default_rng(4).uniform(-1, 1, len(rp) - 1)
    tol = 1e-5 if dtype == "fp32" else 1e-10
    with wait_fault(native, skip_cta=3):
        x, res = native.cg_csr(rp, ci, v, b, dtype=dtype, tol=tol, device=cuda, check=False, cluster=cluster)
    assert res["status"] == TIMEOUT, native.last_error()
    x, res = native.cg_csr(rp, ci, v, b, dtype=dtype, tol=tol, device=cuda, cluster=cluster)
    assert res["status"] == 0
    if dtype == "fp64":
        _, it, _, _ = oracle.cg(rp, ci, v, b, max_iter=20000, stop=1, tol=1e-10)
        assert abs(res["iterations"] - it) <= 1
    assert res["true_rel_res"] <= tol * 1.05


def test_batch_job_barrier_timeout(native, cuda, oracle):
    """A stencil job large enough to be cut into row slices: the slice that
    skips its first job barrier makes the job time out; the plan's other jobs
    finish, and a plan made afterwards runs bit-exact."""
    import torch
    from perks_gb300.batch import BatchPlan, stencil_job
    f = np.random.default_rng(5).random((600, 900))
    small = np.random.default_rng(6).random((16, 16))  # far below the slicing unit: one work item
    ta, ts = torch.from_numpy(f).to(cuda), torch.from_numpy(small).to(cuda)
    oa, os_ = torch.empty_like(ta), torch.empty_like(ts)
    jobs = [stencil_job(ta, oa, "2d5pt", 5), stencil_job(ts, os_, "2d5pt", 5)]
    with wait_fault(native, skip_cta=1):
        plan = BatchPlan(jobs, threads=512, ctas_per_sm=1)
    with plan:
        st = plan.run()
        res = plan.results()
    assert st["sliced_jobs"] == 1
    assert res[0]["status"] == TIMEOUT and res[0]["iterations"] == 0
    assert res[1]["status"] == 0 and bits_equal(os_.cpu().numpy(), oracle.stencil("2d5pt", small, 5))
    with BatchPlan(jobs, threads=512, ctas_per_sm=1) as plan:
        plan.run()
        res = plan.results()
    assert res[0]["status"] == 0
    assert bits_equal(oa.cpu().numpy(), oracle.stencil("2d5pt", f, 5))
