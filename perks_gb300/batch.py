"""Batches of independent stencil and CG instances in one persistent launch
(libperks_gb300's perks_batch_* interface).

    jobs = [stencil_job(a, out_a, "2d5pt", 100), cg_job(rp, ci, v, b, x, tol=1e-10)]
    with BatchPlan(jobs) as plan:      # validates, orders, autotunes, captures the graph
        stats = plan.run()             # one graph launch
        results = plan.results()       # per job, in the order given

Device tensors (torch) own the memory; the plan keeps references to them.
"""
from __future__ import annotations

import ctypes

from . import _native as N


def _dtype_code(t):
    import torch
    if t.dtype == torch.float32:
        return N.FP32
    if t.dtype == torch.float64:
        return N.FP64
    raise TypeError("float32 or float64 tensors only")


def stencil_job(field_in, field_out, shape: str, steps: int) -> dict:
    """`steps` time steps of `shape` (2d5pt, 2ds9pt, 2d9pt or 3d7pt, clamp
    boundary, reference order) on a 2D (wy, wx) or 3D (h, wy, wx) CUDA tensor."""
    if field_in.shape != field_out.shape or field_in.dtype != field_out.dtype:
        raise ValueError("input and output must have the same shape and dtype")
    dims = tuple(field_in.shape)
    h, wy, wx = (1,) + dims if len(dims) == 2 else dims
    return {"kind": N.JOB_STENCIL, "shape": N.SHAPES[shape], "dtype": _dtype_code(field_in), "h": h, "wy": wy,
            "wx": wx, "steps": int(steps), "in": field_in.contiguous(), "out": field_out}


def cg_job(row_ptr, col, val, b, x, tol: float = 1e-10, max_iter: int = 100000, mixed: bool = False) -> dict:
    """CG on CSR device tensors (row_ptr, col int32; val, b, x of one float
    dtype); x receives the solution (it starts from 0). mixed=True (float64
    tensors): FP32 inner iteration with FP64 reliable updates."""
    dt = _dtype_code(val)
    if mixed:
        if dt != N.FP64:
            raise TypeError("a mixed-precision job takes float64 values, b and x")
        dt = N.MIXED
    return {"kind": N.JOB_CG, "dtype": dt, "n": int(b.numel()), "nnz": int(col.numel()),
            "rp": row_ptr, "ci": col, "val": val, "b": b, "x": x, "tol": float(tol), "max_iter": int(max_iter)}


class BatchPlan:
    def __init__(self, jobs: list[dict], threads: int = 0, ctas_per_sm: int = 0, stream=None, slicing: int = 0):
        """threads, ctas_per_sm: the launch shape (0: autotuned); slicing: the
        work granularity, a stencil job costlier than total / (slicing x SMs)
        is cut into row slices (1, 2, 4, 8 or 16; 0: autotuned over 2..16)."""
        import torch
        self._jobs = jobs  # keeps the tensors alive
        arr = (N.Job * len(jobs))()
        for i, j in enumerate(jobs):
            J = arr[i]
            J.kind, J.dtype = j["kind"], j["dtype"]
            if j["kind"] == N.JOB_STENCIL:
                J.shape, J.h, J.wy, J.wx, J.steps = j["shape"], j["h"], j["wy"], j["wx"], j["steps"]
                J.d_in, J.d_out = j["in"].data_ptr(), j["out"].data_ptr()
            else:
                J.n, J.nnz, J.tol, J.max_iter = j["n"], j["nnz"], j["tol"], j["max_iter"]
                J.d_row_ptr, J.d_col, J.d_val = j["rp"].data_ptr(), j["ci"].data_ptr(), j["val"].data_ptr()
                J.d_b, J.d_x = j["b"].data_ptr(), j["x"].data_ptr()
        o = N.BatchOpts()
        N.lib().perks_batch_default_opts(ctypes.byref(o))
        o.threads, o.ctas_per_sm, o.slicing = int(threads), int(ctas_per_sm), int(slicing)
        o.stream = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        self._plan = ctypes.c_void_p()
        N.check(N.lib().perks_batch_plan_create(arr, len(jobs), ctypes.byref(o), ctypes.byref(self._plan)))
        self._n = len(jobs)

    def run(self) -> dict:
        st = N.BatchStats()
        N.check(N.lib().perks_batch_plan_run(self._plan, None, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in N.BatchStats._fields_}

    def results(self) -> list[dict]:
        res = (N.JobResult * self._n)()
        N.check(N.lib().perks_batch_plan_results(self._plan, res))
        return [{k: getattr(r, k) for k, _ in N.JobResult._fields_} for r in res]

    def close(self):
        if self._plan:
            N.lib().perks_batch_plan_destroy(self._plan)
            self._plan = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def synthetic_workload(n_jobs: int = 512, steps: int = 100, seed: int = 42, device="cuda"):
    """The batched uneven workload of the benchmark: n_jobs instances, a third
    each of 2D 5/9-point stencils (64^2..1024^2, log-uniform), 3D 7-point
    stencils (32^3..128^3) and CG on 2D/3D Laplacians (n = 1e3..1e5,
    log-uniform) with a diagonal shift U(0, 0.5); stencils in FP32 and FP64
    storage alternating, CG in FP64 and mixed precision (FP32 inner
    iteration, FP64 reliable updates) alternating, every CG job to the FP64
    tolerance 1e-10; `steps` time steps per stencil. Seeded uniform [0,1)
    fields and uniform [-1,1) right-hand sides.

    Returns (jobs, alone): the batch jobs, and per job what the
    single-instance path needs: ("stencil", field, shape) or
    ("cg", (row_ptr, col, val, b), dtype, tol)."""
    import math

    import numpy as np
    import torch

    from . import matrices as M
    rng = np.random.default_rng(seed)
    gen = torch.Generator(device="cpu").manual_seed(seed)
    dev = torch.device(device)
    jobs, alone = [], []
    for k in range(n_jobs):
        kind, dt = k % 3, (torch.float32 if (k // 3) % 2 == 0 else torch.float64)
        if kind < 2:
            lo, hi = (64, 1024) if kind == 0 else (32, 128)
            m = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
            dims = (m, m) if kind == 0 else (m, m, m)
            shape = ("2d5pt" if rng.random() < 0.5 else "2ds9pt") if kind == 0 else "3d7pt"
            a = torch.rand(dims, generator=gen, dtype=dt).to(dev)
            jobs.append(stencil_job(a, torch.empty_like(a), shape, steps))
            alone.append(("stencil", a, shape))
        else:
            nt = math.exp(rng.uniform(math.log(1e3), math.log(1e5)))
            if rng.random() < 0.5:
                rp, ci, v = M.laplacian_2d(max(8, int(round(math.sqrt(nt)))))
            else:
                rp, ci, v = M.laplacian_3d(max(4, int(round(nt ** (1 / 3)))))
            rp, ci, v = M.shifted(rp, ci, v, rng.uniform(0, 0.5))
            b = rng.uniform(-1, 1, len(rp) - 1)
            mixed = dt == torch.float32
            t = lambda x, ty: torch.from_numpy(np.ascontiguousarray(x)).to(dev, ty)
            x = torch.empty(len(b), dtype=torch.float64, device=dev)
            jobs.append(cg_job(t(rp, torch.int32), t(ci, torch.int32), t(v, torch.float64), t(b, torch.float64), x,
                               tol=1e-10, max_iter=20000, mixed=mixed))
            alone.append(("cg", (rp, ci, v, b), "mixed" if mixed else "fp64", 1e-10))
    return jobs, alone
