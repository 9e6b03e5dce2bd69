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


def cg_job(row_ptr, col, val, b, x, tol: float = 1e-10, max_iter: int = 100000) -> dict:
    """CG on CSR device tensors (row_ptr, col int32; val, b, x of one float
    dtype); x receives the solution (it starts from 0)."""
    return {"kind": N.JOB_CG, "dtype": _dtype_code(val), "n": int(b.numel()), "nnz": int(col.numel()),
            "rp": row_ptr, "ci": col, "val": val, "b": b, "x": x, "tol": float(tol), "max_iter": int(max_iter)}


class BatchPlan:
    def __init__(self, jobs: list[dict], threads: int = 0, ctas_per_sm: int = 0, stream=None):
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
        o.threads, o.ctas_per_sm = int(threads), int(ctas_per_sm)
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
