"""Batched uneven workload (perks_batch_*) on the GPU: many independent
stencil and CG instances in one persistent launch from a device work queue.

Stencil jobs are bit-identical to the oracle (reference evaluation order,
clamp boundary) whether they stay in shared memory or stream through global
memory; CG jobs reach the requested relative residual with an iteration
count within 1% (or 1) of the FP64 oracle. A plan runs repeatedly with the
same results, and autotunes its launch shape when asked."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits_equal(a, b):
    na, nb = np.isnan(a), np.isnan(b)
    return a.shape == b.shape and np.array_equal(na, nb) and np.array_equal(a[~na].view(np.uint8), b[~nb].view(np.uint8))


def it_close(a, b):
    return abs(a - b) <= max(1, int(0.01 * max(a, b)))


def _build(cuda, torch, seed=7):
    from perks_gb300 import matrices as M
    from perks_gb300.batch import cg_job, stencil_job
    rng = np.random.default_rng(seed)
    stencils, cgs, jobs = [], [], []
    # (shape, dims, steps): small ones stay in shared memory, large ones stream
    cases = [("2d5pt", (48, 70), 7), ("2ds9pt", (33, 129), 3), ("2d9pt", (64, 64), 11), ("2d5pt", (300, 257), 5),
             ("2ds9pt", (513, 200), 2), ("2d9pt", (1, 37), 4), ("3d7pt", (20, 30, 17), 6), ("3d7pt", (40, 50, 61), 3),
             ("3d7pt", (1, 1, 1), 2), ("2d5pt", (96, 96), 0), ("2ds9pt", (1100, 700), 9)]
    for k, (shape, dims, steps) in enumerate(cases * 2):
        dt = np.float32 if k % 2 == 0 else np.float64
        f = rng.random(dims).astype(dt)
        a = torch.from_numpy(f).to(cuda)
        o = torch.empty_like(a)
        stencils.append((len(jobs), shape, f, steps, o))
        jobs.append(stencil_job(a, o, shape, steps))
    for k, (mat, dt, tol) in enumerate([("lap2d", np.float64, 1e-10), ("lap3d", np.float64, 1e-10),
                                         ("lap2d", np.float32, 1e-5), ("spd", np.float64, 1e-10),
                                         ("lap2d", "mixed", 1e-10), ("spd", "mixed", 1e-10),
                                         ("lap3d", "mixed", 1e-10)]):
        rp, ci, v = {"lap2d": lambda: M.laplacian_2d(40), "lap3d": lambda: M.laplacian_3d(14),
                     "spd": lambda: M.random_spd(3000, 2)}[mat]()
        rp, ci, v = M.shifted(rp, ci, v, 0.1 * (k + 1))
        b = rng.uniform(-1, 1, len(rp) - 1)
        tt = torch.float32 if dt == np.float32 else torch.float64
        dev = lambda a, t: torch.from_numpy(np.ascontiguousarray(a)).to(cuda, t)
        x = torch.empty(len(b), dtype=tt, device=cuda)
        cgs.append((len(jobs), rp, ci, v, b, tol, dt, x))
        jobs.append(cg_job(dev(rp, torch.int32), dev(ci, torch.int32), dev(v, tt), dev(b, tt), x, tol=tol, max_iter=5000,
                           mixed=dt == "mixed"))
    return jobs, stencils, cgs


@pytest.mark.parametrize("threads,ctas,slicing", [(0, 0, 0), (256, 2, 1), (1024, 1, 4), (512, 1, 2), (1024, 1, 16),
                                                   (1024, 1, 0)])
def test_batch_matches_oracle(native, cuda, oracle, threads, ctas, slicing):
    """Every launch shape and work granularity (slicing: stencil jobs costlier
    than total / (slicing x SMs) are cut into row slices), tuned or fixed."""
    import torch
    from perks_gb300.batch import BatchPlan
    jobs, stencils, cgs = _build(cuda, torch)
    with BatchPlan(jobs, threads=threads, ctas_per_sm=ctas, slicing=slicing) as plan:
        for rep in range(2):
            for _, _, _, _, o in stencils:
                o.fill_(float("nan"))
            st = plan.run()
            res = plan.results()
            torch.cuda.synchronize()
            assert st["resident_jobs"] > 0 and (st["sliced_jobs"] > 0 or st["slicing"] == 1)
            assert st["tuned"] == (1 if threads == 0 or slicing == 0 else 0)
            assert st["slicing"] in (1, 2, 4, 8, 16) and (slicing == 0 or st["slicing"] == slicing)
            for j, shape, f, steps, o in stencils:
                assert res[j]["status"] == 0 and res[j]["iterations"] == steps
                assert bits_equal(o.cpu().numpy(), oracle.stencil(shape, f, steps)), (shape, f.shape, f.dtype, steps, rep)
            for j, rp, ci, v, b, tol, dt, x in cgs:
                assert res[j]["status"] == 0, res[j]
                assert res[j]["rel_res"] <= tol
                xs = x.cpu().numpy().astype(np.float64)
                r = b - oracle.spmv_csr(rp, ci, np.asarray(v, np.float64), xs)
                assert np.linalg.norm(r) / np.linalg.norm(b) <= (1e-4 if dt == np.float32 else tol * 1.05)
                if dt != np.float32:
                    _, it, _, _ = oracle.cg(rp, ci, v, b, max_iter=5000, stop=1, tol=tol)
                    if dt == "mixed":  # FP32 inner iterations: more of them, the FP64 accuracy
                        assert res[j]["iterations"] <= 2 * it + 50, (res[j], it)
                    else:
                        assert it_close(res[j]["iterations"], it), (res[j], it)


def test_batch_rejects_bad_jobs(native, cuda):
    import torch
    from perks_gb300 import PerksError
    from perks_gb300.batch import BatchPlan, stencil_job
    a = torch.zeros((8, 8), device=cuda)
    with pytest.raises(PerksError):
        BatchPlan([stencil_job(a, torch.empty_like(a), "2d13pt", 2)])  # shape not in the batched set
    with pytest.raises(PerksError):
        BatchPlan([])
