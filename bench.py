"""Benchmark of the PERKS stencil time loop on GB300.

Headline workload (the reference's stencil sweep, 2D star 9-point):
2ds9pt, FP32 storage and arithmetic, 8192 x 8192 cells, 1000 time steps per
step of this benchmark, persistent kernel with shared-memory-resident rows,
reference evaluation order (bit-identical to the reference's CPU gold code).
Input: seeded uniform [0,1) field (synthetic; the reference has no dataset
for the stencils). The field (256 MiB) is larger than L2 (129 MB).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One JSON line on rank 0. N > 1 runs one independent replica per GPU
("replicas only": the reference runs on one GPU and the path has no exchange
between GPUs); value = cells*time_steps of all ranks / max rank time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SHAPE = "2ds9pt"
WY = WX = 8192
TSTEPS = 1000
DTYPE = "f32"
METRIC = "GCells/s per stencil & CG time-to-1e-10 rel. residual; mixed vs FP64 on GB300"
UNIT = "GCells/s"
# DRAM bytes (read + write) per cell per time step of the persistent kernel:
# dram__bytes_read.sum + dram__bytes_write.sum of one ncu capture of a 20-step
# launch on the same field (10.101 GB / (20 x 8192^2)), see
# profiles/stencil2d_2ds9pt_f32_8192.txt. The per-step traffic does not depend
# on the number of steps, so a 1000-step launch moves 1000 times as much.
TRAFFIC_PER_CELL_STEP = 7.53


def measured_hbm_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(x: float, ws: int, device=None) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device if device is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws: int):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def extra_cpu():
    """The CPU port on one thread as well as on all cores (the reference's
    CPU code is single-threaded), and the FP64 CPU CG per iteration on the
    2D Laplacian of 2048^2 cells (20 iterations, bounded sample)."""
    import numpy as np
    from oracle import oracle as O
    from perks_gb300 import matrices as M
    O.build()
    all_threads = O.num_threads()
    rng = np.random.default_rng(0)
    f = rng.random((WY, WX), dtype=np.float32)
    out = {}
    prev = O.set_num_threads(1)
    try:
        t0 = time.perf_counter()
        O.stencil(SHAPE, f, 2)
        dt = time.perf_counter() - t0
        out["cpu_port_1thread"] = {"value": WY * WX * 2 / dt / 1e9, "unit": UNIT, "cores": 1, "kind": "port",
                                   "sample": f"{SHAPE} fp32 {WY}x{WX}, 2 time steps, oracle C port, 1 thread"}
        rp, ci, v = M.laplacian_2d(2048)
        b = np.random.default_rng(1).uniform(-1, 1, len(rp) - 1)
        for threads in (1, all_threads):
            O.set_num_threads(threads)
            t0 = time.perf_counter()
            O.cg(rp, ci, v, b, max_iter=20, stop=1, tol=0.0, static_iter=True)
            dt = time.perf_counter() - t0
            out[f"cpu_cg_lap2d_2048_fp64_{threads}thread_ms_per_iter"] = round(dt * 1e3 / 20, 2)
    finally:
        O.set_num_threads(prev)
    return out


def cpu_baseline(seconds_budget: float = 15.0):
    """The oracle (C restatement of the reference's CPU gold code, OpenMP over
    rows) on this host's cores, on a bounded sample of the workload."""
    import numpy as np
    from oracle import oracle as O
    O.build()
    rng = np.random.default_rng(0)
    f = rng.random((WY, WX), dtype=np.float32)
    steps = 1
    t0 = time.perf_counter()
    O.stencil(SHAPE, f, steps)
    dt = time.perf_counter() - t0
    steps = max(1, min(50, int(seconds_budget / max(dt, 1e-3))))
    t0 = time.perf_counter()
    O.stencil(SHAPE, f, steps)
    dt = time.perf_counter() - t0
    return {"value": WY * WX * steps / dt / 1e9, "unit": UNIT, "cores": O.num_threads(), "kind": "port",
            "sample": f"{SHAPE} fp32 {WY}x{WX}, {steps} time steps (of {TSTEPS}), oracle C port, OpenMP"}


def headline_config(ws: int) -> dict:
    return {"workload": f"{SHAPE} {DTYPE} {WY}x{WX} x{TSTEPS} time steps, persistent, reference order",
            "shape": SHAPE, "cells": WY * WX, "time_steps_per_step": TSTEPS, "parallelism": f"replicas{ws}",
            "l2": "inputs larger than L2 (256 MiB field)"}


def run_reference(args, ws, rank):
    if rank != 0:
        return
    K, W = args.steps, args.warmup
    for _ in range(W):
        cpu_baseline(seconds_budget=2.0)
    vals = []
    t0 = time.perf_counter()
    last = None
    for _ in range(K):
        last = cpu_baseline(seconds_budget=max(2.0, 60.0 / max(K, 1)))
        vals.append(last["value"])
    el = time.perf_counter() - t0
    v = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": K,
            "warmup": W, "ms_per_step": el * 1e3 / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": DTYPE, "data": "synthetic (seeded uniform [0,1) field)",
            "config": headline_config(ws), "runs_on": "host cores (rank 0), no GPU",
            "cpu_baseline": {**last, "value": v},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-extra", action="store_true", help="skip the comparator measurements")
    ap.add_argument("--profile-steps", type=int, default=0,
                    help="profiling mode: one warm-up call, then one call of the headline kernel with this many "
                         "time steps, then exit (for ncu captures of a short launch)")
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend=backend)
    if args.impl == "reference":
        run_reference(args, ws, rank)
        if ws > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return

    import numpy as np
    import torch

    import perks_gb300 as P
    from perks_gb300 import _native as N

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    P.lib()
    stream = torch.cuda.current_stream(dev)
    g = torch.Generator(device="cpu").manual_seed(1234 + rank)
    host = torch.rand((WY, WX), generator=g, dtype=torch.float32).pin_memory()
    hout = torch.empty_like(host).pin_memory()
    d_in = host.to(dev)
    d_out = torch.empty_like(d_in)
    kw = dict(kernel="persistent", order="reference", l2_sweep=False)
    if args.profile_steps > 0:
        P.stencil2d(d_in, SHAPE, 2, out=d_out, **kw)
        torch.cuda.synchronize()
        _, st = P.stencil2d(d_in, SHAPE, args.profile_steps, out=d_out, **kw)
        torch.cuda.synchronize()
        print(json.dumps({"profile_steps": args.profile_steps, "kernel_ms": st["ms"],
                          "gcells_per_s": st["gcells_per_s"]}), flush=True)
        return

    def step():
        _, st = P.stencil2d(d_in, SHAPE, TSTEPS, out=d_out, **kw)
        return st

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    barrier(ws)
    P.reset_launch_count()
    kernel_ms = []
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        barrier(ws)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            st = step()
            kernel_ms.append(st["ms"])
        e1.record(stream)
        torch.cuda.synchronize()
        barrier(ws)
    launches = P.launch_count()
    ms = e0.elapsed_time(e1)
    ms_max = max_over_ranks(ms, ws, dev if ws > 1 else None)
    cells = WY * WX * TSTEPS
    value = cells * args.steps * ws / (ms_max * 1e-3) / 1e9

    # e2e: the reference-facing host-buffer entry point (jacobi_iterative),
    # pinned host buffers, H2D + D2H inside the timed region.
    lib = P.lib()
    hin_p = ctypes.c_void_p(host.data_ptr())
    hout_p = ctypes.c_void_p(hout.data_ptr())

    def e2e_step():
        rc = lib.perks_jacobi_iterative_f32(N.SHAPES[SHAPE], hin_p, WY, WX, hout_p, 256, 0, TSTEPS, 0, 1, 0, -1, 0)
        if rc != 0:
            raise RuntimeError(P.last_error())

    e2e_step()
    torch.cuda.synchronize()
    barrier(ws)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, ws, dev if ws > 1 else None)
    barrier(ws)
    e2e_val = cells * args.steps * ws / e2e_s / 1e9
    nbytes = WY * WX * 4

    peak, peak_src = measured_hbm_peak()
    kms = statistics.mean(kernel_ms)
    alg_bytes = 2 * 4 * cells  # reference formula: 2*sizeof(REAL)*cells per time step
    achieved = alg_bytes / (kms * 1e-3) / 1e9
    traffic = (TRAFFIC_PER_CELL_STEP * cells) if TRAFFIC_PER_CELL_STEP else None
    roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "peak_source": peak_src,
            "traffic": traffic,
            "algorithmic_bytes_per_launch": alg_bytes, "kernel_ms_per_launch": round(kms, 3)}
    if traffic:
        # DRAM bytes actually moved (resident rows are not re-read) per second
        dram = traffic / (kms * 1e-3) / 1e9
        roof["dram_achieved"] = round(dram, 1)
        roof["dram_frac"] = round(dram / peak, 4)

    extra = {}
    if not args.no_extra and rank == 0:
        # one-launch-per-step comparator and FP64 on the same shape and size
        _, st = P.stencil2d(d_in, SHAPE, 100, out=d_out, kernel="per_step")
        extra["per_step_fp32_gcells"] = round(st["gcells_per_s"], 2)
        _, st = P.stencil2d(d_in, SHAPE, 100, out=d_out, kernel="persistent", l2_sweep=True)
        extra["persistent_l2sweep_fp32_gcells"] = round(st["gcells_per_s"], 2)
        _, st = P.stencil2d(d_in, SHAPE, 100, out=d_out, kernel="persistent", order="fast")
        extra["persistent_fast_fp32_gcells"] = round(st["gcells_per_s"], 2)
        d64 = d_in.double()
        o64 = torch.empty_like(d64)
        _, st = P.stencil2d(d64, SHAPE, 50, out=o64, kernel="persistent")
        extra["persistent_ref_fp64_gcells"] = round(st["gcells_per_s"], 2)
        _, st = P.stencil2d(d64, SHAPE, 50, out=o64, kernel="persistent", order="fast")
        extra["persistent_fast_fp64_gcells"] = round(st["gcells_per_s"], 2)
        del d64, o64
        _, st = P.stencil2d(d_in, SHAPE, 20, out=d_out, kernel="naive")
        extra["naive_fp32_gcells"] = round(st["gcells_per_s"], 2)
        extra["cached_fraction"] = round(kernel_cached_fraction(P, d_in, d_out), 4)
        extra.update(host_link_gbs(torch, host, hout, d_in, d_out))
        extra.update(extra_fma_peak(P))
        extra.update(extra_config1(P, torch, extra.get("fma_peak", {})))
        extra.update(extra_min_domain(P, torch))
        extra.update(extra_3d(P, torch))
        extra.update(extra_cg(P, torch))
        extra.update(extra_cg_spd_sizes(P, torch))
        extra.update(extra_batch(P, torch))

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu = cpu_baseline()
        if not args.no_extra:
            extra.update(extra_cpu())

    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": max(3, args.warmup), "ms_per_step": round(ms_max / args.steps, 3),
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": DTYPE,
                "data": "synthetic (seeded uniform [0,1) field)",
                "config": headline_config(ws),
                "e2e": {"value": round(e2e_val, 3), "unit": UNIT, "h2d_bytes_per_step": nbytes,
                        "d2h_bytes_per_step": nbytes},
                "gpu_launches": int(launches),
                "roofline": roof,
                "cpu_baseline": cpu,
                "clocks": clk.summary(),
                "extra": extra}
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def host_link_gbs(torch, host, hout, d_in, d_out, reps=5):
    """Pinned host <-> device copy rate of one field (the ceiling of the e2e copies)."""
    out = {}
    for tag, dst, src in (("h2d_gbs", d_in, host), ("d2h_gbs", hout, d_out)):
        dst.copy_(src, non_blocking=True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            dst.copy_(src, non_blocking=True)
        e1.record()
        torch.cuda.synchronize()
        out[tag] = round(src.numel() * src.element_size() * reps / (e0.elapsed_time(e1) * 1e6), 1)
    return out


def extra_fma_peak(P):
    """Measured FMA throughput (perks_probe_fma_peak): the arithmetic roofline
    of the FP64 stencils and CG, bound by the FP64 pipe on GB300."""
    out = {}
    for dt in ("fp64", "fp32"):
        best = max((P.fma_peak(dt) for _ in range(3)), key=lambda r: r["fma_per_s"])
        out[dt] = {"fma_per_s": best["fma_per_s"], "tflops": round(best["tflops"], 3)}
    return {"fma_peak": out}


# FP64 arithmetic operations per cell of 2d5pt in reference order: five
# products of a weight and a neighbour, four sums, and the exact division by
# 118 (product with the reciprocal, remainder fma, correction fma); each takes
# one issue slot of the FP64 pipe, like one FMA.
FP64_OPS_2D5PT_REF = 12


def extra_config1(P, torch, peak, steps=1000):
    """The plain FP64 configuration: 2d5pt on 1024 x 1024 cells (clamp, the
    reference driver's check) and 1026 x 1026 with a fixed Dirichlet border,
    seeded uniform [0,1), 1000 time steps, reference order (bit-identical to
    the CPU oracle in the tests). Persistent kernel against one launch per
    step and the naive per-cell kernel; the FP64-pipe fraction counts
    FP64_OPS_2D5PT_REF operations per cell against the measured FP64 FMA rate.
    The field (8 MiB) lives in L2, so HBM is not the bound here."""
    g = torch.Generator(device="cpu").manual_seed(1)
    f = torch.rand((1026, 1026), generator=g, dtype=torch.float64).cuda()
    out = {}
    fma = (peak.get("fp64") or {}).get("fma_per_s")
    for tag, d, bnd in (("clamp_1024", f[1:-1, 1:-1].contiguous(), "clamp"), ("dirichlet_1026", f, "dirichlet")):
        o = torch.empty_like(d)
        row = {}
        for kernel in ("persistent", "per_step", "naive"):
            P.stencil2d(d, "2d5pt", 3, out=o, kernel=kernel, boundary=bnd)
            _, st = P.stencil2d(d, "2d5pt", steps, out=o, kernel=kernel, boundary=bnd)
            row[f"{kernel}_gcells"] = round(st["gcells_per_s"], 2)
            if kernel == "persistent":
                row["persistent_ms"] = round(st["ms"], 3)
                if fma:
                    row["fp64_pipe_frac"] = round(st["gcells_per_s"] * 1e9 * FP64_OPS_2D5PT_REF / fma, 4)
        out[f"config1_2d5pt_fp64_{tag}"] = {"steps": steps, **row}
    return out


def extra_min_domain(P, torch, steps=1000):
    """All-on-chip throughput: the headline shape at the largest 8192-wide
    field whose rows the persistent kernel keeps in shared memory (the
    reference's --small mode), against one launch per step at that size."""
    import numpy as np
    out = {}
    for dt, tag in ((torch.float32, "fp32"), (torch.float64, "fp64")):
        wy = P.min_domain_2d(SHAPE, WX, dtype=np.float64 if dt == torch.float64 else np.float32)
        d = torch.rand((wy, WX), dtype=dt, device="cuda")
        o = torch.empty_like(d)
        n = steps if tag == "fp32" else steps // 10
        P.stencil2d(d, SHAPE, 3, out=o)
        _, st = P.stencil2d(d, SHAPE, n, out=o)
        _, st1 = P.stencil2d(d, SHAPE, n, out=o, kernel="per_step")
        out[f"min_domain_{tag}"] = {"width_y": wy, "width_x": WX, "steps": n,
                                    "cached_fraction": round(st["cached_fraction"], 4),
                                    "persistent_gcells": round(st["gcells_per_s"], 2),
                                    "per_step_gcells": round(st1["gcells_per_s"], 2)}
        del d, o
    return out


def extra_3d(P, torch):
    """3D shapes of the stencil sweep at 512^3 (FP32 and FP64, 20 steps each)."""
    out = {}
    for dt, tag in ((torch.float32, "fp32"), (torch.float64, "fp64")):
        d = torch.rand((512, 512, 512), dtype=dt, device="cuda")
        o = torch.empty_like(d)
        for shape in ("3d7pt", "3d27pt"):
            P.stencil3d(d, shape, 2, out=o, order="fast")
            for order in ("reference", "fast"):
                _, st = P.stencil3d(d, shape, 20, out=o, order=order)
                out[f"{shape}_512_{tag}_{order}_gcells"] = round(st["gcells_per_s"], 2)
        del d, o
    return out


def extra_cg(P, torch):
    """CG time to a 1e-10 relative residual, RHS uniform [-1,1) seed 1, x0 = 0,
    FP64 vs mixed precision (FP32 inner, FP64 reliable updates): the 2D
    5-point Laplacian 2048^2 (4.19M rows, 20.96M nonzeros) in CSR and DIA, the
    3D 7-point Laplacian 160^3 and a random SPD matrix in CSR."""
    import numpy as np
    from perks_gb300 import matrices as M
    rp, ci, v = M.laplacian_2d(2048)
    b = np.random.default_rng(1).uniform(-1, 1, len(rp) - 1)
    off, data = M.csr_to_dia(rp, ci, v)
    out = {}
    for fmt in ("csr", "dia"):
        for dt in ("fp64", "mixed"):
            if fmt == "csr":
                x, res = P.cg_csr(rp, ci, v, b, dtype=dt, tol=1e-10)
                mb = cg_bytes_csr(len(b), len(ci), dt)
            else:
                x, res = P.cg_dia(off, data, b, dtype=dt, tol=1e-10)
                mb = cg_bytes_dia(len(b), len(off), dt)
            out[f"cg_lap2d_2048_{fmt}_{dt}"] = cg_summary(res, mb)
    # single-reduction CG (one barrier + one two-value reduction per iteration)
    x, res = P.cg_dia(off, data, b, dtype="fp64", tol=1e-10, algorithm="single_reduction")
    out["cg_lap2d_2048_dia_fp64_single_reduction"] = cg_summary(res, cg_bytes_dia(len(b), len(off), "fp64"))
    # 3D 7-point Laplacian 160^3 (4.1M rows), CSR input
    rp, ci, v = M.laplacian_3d(160)
    b = np.random.default_rng(1).uniform(-1, 1, len(rp) - 1)
    for dt in ("fp64", "mixed"):
        x, res = P.cg_csr(rp, ci, v, b, dtype=dt, tol=1e-10)
        out[f"cg_lap3d_160_csr_{dt}"] = cg_summary(res, cg_bytes_csr(len(b), len(ci), dt))
    return out


def extra_cg_spd_sizes(P, torch):
    """CG on the random sparse SPD matrices (power-law rows of 3..60 entries,
    mean about 14, N(0,1) off-diagonals, diagonally dominant), n = 1e5 to 2e6,
    CSR input, FP64 against mixed precision at the same 1e-10 relative
    residual."""
    import numpy as np
    from perks_gb300 import matrices as M
    out = {}
    for n, tag in ((100_000, "1e5"), (300_000, "3e5"), (1_000_000, "1e6"), (2_000_000, "2e6")):
        rp, ci, v = M.random_spd(n, 7)
        b = np.random.default_rng(1).uniform(-1, 1, n)
        for dt in ("fp64", "mixed"):
            P.cg_csr(rp, ci, v, b, dtype=dt, tol=1e-10)  # first call: setup of this size
            x, res = P.cg_csr(rp, ci, v, b, dtype=dt, tol=1e-10)
            out[f"cg_spd_{tag}_csr_{dt}"] = cg_summary(res, cg_bytes_csr(n, len(ci), dt))
        if tag == "1e6":
            x, res = P.cg_csr(rp, ci, v, b, dtype="fp64", tol=1e-10, algorithm="single_reduction")
            out["cg_spd_1e6_csr_fp64_single_reduction"] = cg_summary(res, cg_bytes_csr(n, len(ci), "fp64"))
    return out


def cg_bytes_csr(n, nnz, dtype):
    """Algorithmic bytes of one CG iteration, the reference's formula
    (conjugateGradient/cg_driver.cu:360-361): nnz (value + int32 column) +
    (n+1) row pointers + six vector passes, at the iteration's working
    precision (FP32 for the inner iterations of mixed precision)."""
    sv = 8 if dtype == "fp64" else 4
    return nnz * (sv + 4) + 4 * (n + 1) + 6 * n * sv


def cg_bytes_dia(n, ndiag, dtype):
    sv = 8 if dtype == "fp64" else 4
    return ndiag * n * sv + 6 * n * sv


def cg_summary(res, bytes_per_iter=None):
    it = max(1, res["iterations"])
    out = {"ms": round(res["ms"], 2), "iterations": res["iterations"],
           "us_per_iter": round(1e3 * res["ms"] / it, 2), "true_rel_res": res["true_rel_res"]}
    if bytes_per_iter:
        peak, src = measured_hbm_peak()
        gbs = bytes_per_iter * it / (res["ms"] * 1e-3) / 1e9
        out["roofline"] = {"bound": "hbm", "bytes_per_iter": bytes_per_iter, "achieved": round(gbs, 1),
                           "peak": peak, "unit": "GB/s", "frac": round(gbs / peak, 4), "peak_source": src}
    return out


def extra_batch(P, torch, n_jobs=512, steps=100, seed=42):
    """The batched uneven workload (perks_gb300.batch.synthetic_workload: 512
    instances of 2D/3D stencils in FP32/FP64 storage and shifted-Laplacian
    CG in FP64/mixed precision, every CG job to 1e-10) in one persistent
    launch (a CUDA graph, autotuned launch shape), against every instance run
    alone through the single-instance entry points in the same precisions,
    and against the plain FP64 path (every instance alone in FP64); sums of
    device times. The CG jobs' true relative residuals are recomputed on the
    host in FP64 (worst one reported)."""
    from perks_gb300.batch import BatchPlan, synthetic_workload
    jobs, alone = synthetic_workload(n_jobs, steps, seed)
    with BatchPlan(jobs) as plan:
        plan.run()
        runs = [plan.run() for _ in range(3)]
        res = plan.results()
    st = min(runs, key=lambda r: r["ms"])
    bad = sum(1 for r in res if r["status"] != 0)
    import numpy as np
    worst = 0.0
    for j, a in zip(jobs, alone):
        if a[0] == "cg":
            rp, ci, v, b = a[1]
            xs = j["x"].double().cpu().numpy()
            r = b - (np.add.reduceat(v * xs[ci], rp[:-1]) if len(ci) else 0.0)
            worst = max(worst, float(np.linalg.norm(r) / np.linalg.norm(b)))
    alone_ms, fp64_ms = 0.0, 0.0
    for a in alone:
        if a[0] == "stencil":
            fn = P.stencil2d if a[1].dim() == 2 else P.stencil3d
            _, s1 = fn(a[1], a[2], steps)
            alone_ms += s1["ms"]
            _, s2 = fn(a[1].double(), a[2], steps) if a[1].dtype != torch.float64 else (None, s1)
            fp64_ms += s2["ms"]
        else:
            rp, ci, v, b = a[1]
            _, r1 = P.cg_csr(rp, ci, v, b, dtype=a[2], tol=a[3], max_iter=20000, check=False)
            alone_ms += r1["ms"]
            if a[2] != "fp64":
                _, r1 = P.cg_csr(rp, ci, v, b, dtype="fp64", tol=a[3], max_iter=20000, check=False)
            fp64_ms += r1["ms"]
    torch.cuda.synchronize()
    return {"batch_512": {"jobs": n_jobs, "batch_ms": round(st["ms"], 2), "alone_ms_sum": round(alone_ms, 2),
                          "speedup": round(alone_ms / st["ms"], 2), "plain_fp64_alone_ms_sum": round(fp64_ms, 2),
                          "speedup_vs_plain_fp64": round(fp64_ms / st["ms"], 2),
                          "cg_worst_true_rel_res": worst, "threads": st["threads"],
                          "ctas_per_sm": st["ctas_per_sm"], "resident_stencil_jobs": st["resident_jobs"],
                          "sliced_stencil_jobs": st["sliced_jobs"], "slicing": st["slicing"],
                          "jobs_not_ok": bad}}


def kernel_cached_fraction(P, d_in, d_out):
    _, st = P.stencil2d(d_in, SHAPE, 2, out=d_out)
    return st["cached_fraction"]


if __name__ == "__main__":
    main()
