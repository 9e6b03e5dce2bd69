"""One short, self-contained launch of a hot-path kernel, for profilers.

  python -m perks_gb300.profile stencil --shape 3d27pt --dims 256,256,256 --dtype f32 --order fast --steps 3
  python -m perks_gb300.profile cg --matrix lap2d --n 512 --dtype fp64 --iters 20
  python -m perks_gb300.profile batch --jobs 512 --steps 100
  python -m perks_gb300.profile sweep --steps 1000     # every stencil shape, one JSON line each
  python -m perks_gb300.profile fmapeak                # FP64 and FP32 FMA throughput of this GPU

Runs one warm-up call, then exactly one call of the requested size, and
prints its stats as one JSON line. The warm-up uses the same kernel with 2
time steps (stencil) or 2 iterations (CG), so an ncu filter of
`-k regex:<kernel> -s 1 -c 1` captures the second call. Fields are seeded
uniform [0,1); CG right-hand sides uniform [-1,1). `batch` builds the
benchmark's batched workload and runs it once with a fixed launch shape (the
autotuner's candidate runs would be captured otherwise): the only
batch_kernel launch, `-k regex:batch_kernel -c 1`.
"""
from __future__ import annotations

import argparse
import json
import sys


def _stencil(a):
    import torch
    from . import stencil as S
    dims = tuple(int(x) for x in a.dims.split(","))
    dt = {"f32": torch.float32, "f64": torch.float64}[a.dtype]
    g = torch.Generator(device="cpu").manual_seed(1)
    d = torch.rand(dims, generator=g, dtype=dt).cuda()
    o = torch.empty_like(d)
    kw = dict(kernel=a.kernel, order=a.order, l2_sweep=a.l2_sweep, cache_rows=a.cache_rows)
    fn = S.stencil2d if len(dims) == 2 else S.stencil3d
    fn(d, a.shape, 2, out=o, **kw)
    torch.cuda.synchronize()
    _, st = fn(d, a.shape, a.steps, out=o, **kw)
    torch.cuda.synchronize()
    return {"shape": a.shape, "dims": dims, "dtype": a.dtype, "order": a.order, "steps": a.steps, **st}


def _sweep(a):
    """The stencil sweep: every shape at its sizes, FP32 and FP64 storage,
    reference order, persistent vs one launch per step (a.steps time steps),
    and the FP32 result's error relative to the FP64 one after a.err_steps
    steps (the FP64 kernel is bit-identical to the CPU oracle in the tests,
    so it stands in for the oracle at these sizes; the reference weights do
    not sum to one, so over many steps the fields leave the floating-point
    range and only a short run gives a meaningful error)."""
    import torch
    from . import stencil as S
    cases = []
    if "2d" in a.which:
        cases += [(sh, (8192, 8192)) for sh in ("2d5pt", "2ds9pt", "2d13pt", "2d17pt", "2d21pt", "2ds25pt", "2d9pt",
                                               "2d25pt")]
    for n in (256, 512):
        if f"3d{n}" in a.which:
            cases += [(sh, (n, n, n)) for sh in ("3d7pt", "3d13pt", "3d17pt", "3d27pt", "poisson")]
    rows = []
    for shape, dims in cases:
        fn = S.stencil2d if len(dims) == 2 else S.stencil3d
        g = torch.Generator(device="cpu").manual_seed(1)
        f64 = torch.rand(dims, generator=g, dtype=torch.float64)
        res, outs = {}, {}
        for dtn, dt in (("f32", torch.float32), ("f64", torch.float64)):
            d = f64.to(dt).cuda()
            o = torch.empty_like(d)
            for kernel in ("persistent", "per_step") + (("naive",) if len(dims) == 2 else ()):
                fn(d, shape, 2, out=o, kernel=kernel)
                torch.cuda.synchronize()
                _, st = fn(d, shape, a.steps, out=o, kernel=kernel)
                torch.cuda.synchronize()
                res[f"{dtn}_{kernel}"] = round(st["gcells_per_s"], 2)
            fn(d, shape, a.err_steps, out=o)
            outs[dtn] = o.double()
            del d, o
        diff = (outs["f32"] - outs["f64"]).abs()
        ref = outs["f64"].abs()
        row = {"shape": shape, "dims": list(dims), "steps": a.steps, "gcells": res, "err_steps": a.err_steps,
               "f32_rel_max_err": float(diff.max() / ref.max()),
               "f32_rel_rms_err": float(diff.pow(2).mean().sqrt() / outs["f64"].pow(2).mean().sqrt())}
        del outs, diff, ref
        torch.cuda.empty_cache()
        print(json.dumps(row), flush=True)
        rows.append(row)
    return {"cases": len(rows)}


def _cg(a):
    import numpy as np
    from . import cg as C
    from . import matrices as M
    rp, ci, v = {"lap2d": lambda: M.laplacian_2d(a.n), "lap3d": lambda: M.laplacian_3d(a.n),
                 "spd": lambda: M.random_spd(a.n, 7)}[a.matrix]()
    b = np.random.default_rng(1).uniform(-1, 1, len(rp) - 1)
    kw = dict(dtype=a.dtype, tol=0.0, static_iter=True, check=False)
    if a.format == "dia":
        off, data = M.csr_to_dia(rp, ci, v)
        C.cg_dia(off, data, b, max_iter=2, **kw)
        _, res = C.cg_dia(off, data, b, max_iter=a.iters, **kw)
    else:
        C.cg_csr(rp, ci, v, b, max_iter=2, **kw)
        _, res = C.cg_csr(rp, ci, v, b, max_iter=a.iters, **kw)
    return {"matrix": a.matrix, "n": a.n, "format": a.format, "dtype": a.dtype, **res}


def _fmapeak(a):
    """FP64 and FP32 FMA throughput (perks_probe_fma_peak), best of a.reps."""
    from . import fma_peak
    out = {}
    for dt in ("fp64", "fp32"):
        runs = [fma_peak(dt) for _ in range(a.reps)]
        best = max(runs, key=lambda r: r["fma_per_s"])
        out[dt] = {"fma_per_s": best["fma_per_s"], "tflops": round(best["tflops"], 3),
                   "ms": round(best["ms"], 3), "runs": [round(r["tflops"], 3) for r in runs]}
    return out


def _batch(a):
    import torch
    from .batch import BatchPlan, synthetic_workload
    jobs, _ = synthetic_workload(a.jobs, a.steps, a.seed)
    with BatchPlan(jobs, threads=a.threads, ctas_per_sm=a.ctas, slicing=a.slicing) as plan:
        st = plan.run()
        bad = sum(1 for r in plan.results() if r["status"] != 0)
    torch.cuda.synchronize()
    return {"jobs": a.jobs, "steps": a.steps, "jobs_not_ok": bad, **st}


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m perks_gb300.profile")
    sub = ap.add_subparsers(dest="what", required=True)
    s = sub.add_parser("stencil")
    s.add_argument("--shape", required=True)
    s.add_argument("--dims", required=True, help="wy,wx or h,wy,wx")
    s.add_argument("--dtype", default="f32", choices=["f32", "f64"])
    s.add_argument("--order", default="reference", choices=["reference", "fast"])
    s.add_argument("--kernel", default="persistent", choices=["persistent", "per_step", "naive"])
    s.add_argument("--l2-sweep", action="store_true")
    s.add_argument("--steps", type=int, default=3)
    s.add_argument("--cache-rows", type=int, default=None,
                   help="rows (2D) / planes (3D) per CTA kept in shared memory: -1 as many as fit, 0 none "
                        "(default: the library's, 2D -1, 3D 0)")
    c = sub.add_parser("cg")
    c.add_argument("--matrix", default="lap2d", choices=["lap2d", "lap3d", "spd"])
    c.add_argument("--n", type=int, default=512, help="grid points per dimension (spd: rows)")
    c.add_argument("--format", default="csr", choices=["csr", "dia"])
    c.add_argument("--dtype", default="fp64", choices=["fp64", "fp32", "mixed"])
    c.add_argument("--iters", type=int, default=20)
    sw = sub.add_parser("sweep")
    sw.add_argument("--steps", type=int, default=1000)
    sw.add_argument("--err-steps", type=int, default=10)
    sw.add_argument("--which", default="2d,3d256,3d512", help="any of 2d, 3d256, 3d512")
    bt = sub.add_parser("batch")
    bt.add_argument("--jobs", type=int, default=512)
    bt.add_argument("--steps", type=int, default=100)
    bt.add_argument("--seed", type=int, default=42)
    bt.add_argument("--threads", type=int, default=1024, help="threads per CTA (0 = autotune)")
    bt.add_argument("--ctas", type=int, default=1, help="CTAs per SM (0 = autotune)")
    bt.add_argument("--slicing", type=int, default=2, help="work granularity 1, 2, 4, 8 or 16 (0 = autotune)")
    fp = sub.add_parser("fmapeak")
    fp.add_argument("--reps", type=int, default=5)
    a = ap.parse_args(argv)
    out = {"stencil": _stencil, "cg": _cg, "batch": _batch, "sweep": _sweep, "fmapeak": _fmapeak}[a.what](a)
    print(json.dumps(out, default=str), flush=True)


if __name__ == "__main__":
    sys.exit(main())
