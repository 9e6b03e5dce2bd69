"""Build-time tuning of the 2D stencil kernels, written as a table.

The reference picks its register-cache depth per shape offline: it compiles
variants, reads the compiler's register and spill report and turns the
results into headers (stencil/2dstencil/ProcessCompilerLog.py,
ProcessRsts2cuh.py -> perksconfig.cuh). This tool does the same for the
GB300 kernels and adds a measurement, because here the choice that matters
(warps per CTA, rows in flight per warp, the form of the exact division)
changes speed without changing registers much:

  1. compile every candidate of every 2D translation unit with
     -DPERKS_TUNE_NW/_D/_FIN and -Xptxas -v, in parallel;
  2. drop a candidate for a shape when its kernel spills more than the
     built-in choice does;
  3. link one library per candidate and time every shape on the GPU
     (8192^2 field by default), after checking that its output is
     bit-identical to the built-in kernel's;
  4. keep the fastest candidate per (dtype, order, shape) when it beats the
     built-in choice by more than the noise margin, and write the table into
     csrc/tune2d.cuh (with --write).

    python -m perks_gb300.autotune [--write] [--dtypes f32,f64] [--orders ref,fast]

Candidates differ only in template arguments, so their kernels have
distinct names and can be linked next to the default build.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import ctypes
import itertools
import json
import os
import re
import subprocess
import sys
import time

from . import build as B
from . import _native as N

SHAPES2D = ["2d5pt", "2ds9pt", "2d13pt", "2d17pt", "2d21pt", "2ds25pt", "2d9pt", "2d25pt"]
TUNE_DIR = os.path.join(B.HERE, "_build", "tune")
TABLE = os.path.join(B.CSRC, "tune2d.cuh")
SPILL_RE = re.compile(r"(\d+) bytes spill stores")
REGS_RE = re.compile(r"Used (\d+) registers")
KERNEL_RE = re.compile(r"Function properties for _ZN5perks16stencil2d_kernelI[fd]Li(\d+)E")


def candidates(order: str, nws, ds, fins):
    for nw, d in itertools.product(nws, ds):
        for fin in (fins if order == "ref" else [0]):
            yield nw, d, fin


def compile_variant(tu: str, nw: int, d: int, fin: int) -> dict:
    """Compile one candidate of a translation unit; report per-shape registers and spills."""
    name = f"{tu}_nw{nw}_d{d}_f{fin}"
    obj = os.path.join(TUNE_DIR, name + ".o")
    cmd = ([B.nvcc()] + B.ARCH + B.NVCC_FLAGS +
           [f"-DPERKS_TUNE_NW={nw}", f"-DPERKS_TUNE_D={d}", f"-DPERKS_TUNE_FIN={fin}", "-Xptxas", "-v",
            "-c", os.path.join(B.CSRC, tu + ".cu"), "-o", obj])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return {"name": name, "ok": False, "error": (r.stderr or r.stdout)[-2000:]}
    return {"name": name, "ok": True, "obj": obj, "shapes": ptxas_report(r.stderr), "tu": tu, "nw": nw, "d": d,
            "fin": fin}


def compile_default(tu: str) -> dict:
    """Registers and spills of the built-in choice (no PERKS_TUNE_* overrides)."""
    cmd = [B.nvcc()] + B.ARCH + B.NVCC_FLAGS + ["-Xptxas", "-v", "-c", os.path.join(B.CSRC, tu + ".cu"),
                                                 "-o", os.path.join(TUNE_DIR, tu + "_default.o")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {tu}:\n{r.stderr[-2000:]}")
    return {"name": f"{tu}_default", "shapes": ptxas_report(r.stderr)}


def ptxas_report(text: str) -> dict:
    """{shape index: {"regs": R, "spill": bytes}} of the 2D kernels in -Xptxas -v output."""
    shapes, cur = {}, None
    for line in text.splitlines():
        m = KERNEL_RE.search(line)
        if m:
            cur = int(m.group(1))
            continue
        m = SPILL_RE.search(line)
        if m and cur is not None:
            shapes.setdefault(cur, {})["spill"] = int(m.group(1))
        m = REGS_RE.search(line)
        if m and cur is not None:
            shapes.setdefault(cur, {})["regs"] = int(m.group(1))
            cur = None
    return shapes


def link_variant(v: dict) -> str:
    lib = os.path.join(TUNE_DIR, v["name"] + ".so")
    objs = [o for o in (os.path.join(B.OBJ, os.path.basename(s) + ".o") for s in B._sources())
            if not o.endswith(v["tu"] + ".cu.o")]
    cmd = [B.nvcc()] + B.ARCH + ["-shared", "-o", lib] + objs + [v["obj"], "-lcudart_static", "-ldl", "-lrt",
                                                                  "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed for {v['name']}:\n{r.stderr}")
    return lib


class Lib:
    """A library build driven through its C ABI (only the calls timing needs)."""

    def __init__(self, path: str):
        self.L = ctypes.CDLL(path)
        self.L.perks_stencil_default_opts.argtypes = [ctypes.POINTER(N.StencilOpts), ctypes.c_int, ctypes.c_int]
        self.L.perks_stencil2d.argtypes = [ctypes.POINTER(N.StencilOpts), ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(N.StencilStats)]
        self.L.perks_last_error.restype = ctypes.c_char_p

    def run(self, shape: str, dt: int, order: int, src, dst, steps: int, stream) -> N.StencilStats:
        o = N.StencilOpts()
        self.L.perks_stencil_default_opts(ctypes.byref(o), N.SHAPES[shape], dt)
        o.order = order
        o.stream = stream
        st = N.StencilStats()
        rc = self.L.perks_stencil2d(ctypes.byref(o), src.data_ptr(), dst.data_ptr(), src.shape[0], src.shape[1],
                                    steps, ctypes.byref(st))
        if rc != 0:
            raise RuntimeError(self.L.perks_last_error().decode())
        return st


def measure(libs: dict, dtypes, orders, size: int, steps: dict, reps: int) -> dict:
    import torch
    dev = torch.device("cuda:0")
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    out = {}
    for dtn in dtypes:
        tdt = torch.float32 if dtn == "f32" else torch.float64
        dt = N.FP32 if dtn == "f32" else N.FP64
        g = torch.Generator(device="cpu").manual_seed(1234)
        big = torch.rand((size, size), generator=g, dtype=tdt).to(dev)
        small = torch.rand((700, 2100), generator=g, dtype=tdt).to(dev)
        o_big, o_ref, o_var = torch.empty_like(big), torch.empty_like(small), torch.empty_like(small)
        for ordn in orders:
            order = N.ORDER_REFERENCE if ordn == "ref" else N.ORDER_FAST
            for shape in SHAPES2D:
                key = f"{dtn}/{ordn}/{shape}"
                base = libs["default"]
                base.run(shape, dt, order, small, o_ref, 7, stream)
                res = {}
                for name, lib in libs.items():
                    if name != "default" and not lib_applies(name, dtn, ordn):
                        continue
                    if name != "default":
                        try:
                            lib.run(shape, dt, order, small, o_var, 7, stream)
                        except RuntimeError as e:  # e.g. shared memory budget
                            res[name] = {"error": str(e)}
                            continue
                        torch.cuda.synchronize()
                        if not torch.equal(o_var.view(torch.int32 if dtn == "f32" else torch.int64),
                                           o_ref.view(torch.int32 if dtn == "f32" else torch.int64)):
                            res[name] = {"error": "output differs from the built-in kernel"}
                            continue
                    lib.run(shape, dt, order, big, o_big, max(3, steps[dtn] // 10), stream)
                    best = 0.0
                    for _ in range(reps):
                        best = max(best, lib.run(shape, dt, order, big, o_big, steps[dtn], stream).gcells_per_s)
                    res[name] = {"gcells": round(best, 2)}
                out[key] = res
                print(key, json.dumps(res), flush=True)
        del big, small, o_big, o_ref, o_var
    return out


def lib_applies(name: str, dtn: str, ordn: str) -> bool:
    return name.startswith(f"s2d_{dtn}_{ordn}_")


def choose(results: dict, spills: dict, margin: float) -> dict:
    """Fastest candidate per key that spills no more than the built-in kernel
    and beats it by more than `margin` (relative)."""
    table = {}
    for key, res in results.items():
        dtn, ordn, shape = key.split("/")
        base = res.get("default", {}).get("gcells", 0.0)
        best, best_v = base * (1.0 + margin), None
        for name, r in res.items():
            if name == "default" or "gcells" not in r:
                continue
            sp = spills.get(name, {}).get(SHAPES2D.index(shape))
            if sp is None or sp["spill"] > spills[f"s2d_{dtn}_{ordn}_default"][SHAPES2D.index(shape)]["spill"]:
                continue
            if r["gcells"] > best:
                best, best_v = r["gcells"], name
        if best_v:
            m = re.search(r"_nw(\d+)_d(\d+)_f(\d+)$", best_v)
            table[key] = {"nw": int(m.group(1)), "d": int(m.group(2)), "fin": int(m.group(3)),
                          "gcells": best, "default_gcells": base}
    return table


def write_table(table: dict, path: str = TABLE) -> None:
    rows = []
    for dtn in ("f32", "f64"):
        orows = []
        for ordn in ("ref", "fast"):
            cells = []
            for shape in SHAPES2D:
                t = table.get(f"{dtn}/{ordn}/{shape}")
                cells.append(f"{{{t['nw']}, {t['d']}, {t['fin']}}}" if t else "{0, 0, 0}")
            orows.append("{" + ", ".join(cells) + "}")
        rows.append("{" + ",\n   ".join(orows) + "}")
    body = "constexpr Tune2D kTune2D[2][2][8] = {\n  " + ",\n  ".join(rows) + "};\n"
    src = open(path).read()
    a, b = src.index("// BEGIN TABLE\n") + len("// BEGIN TABLE\n"), src.index("// END TABLE")
    with open(path, "w") as f:
        f.write(src[:a] + body + src[b:])


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--dtypes", default="f32,f64")
    ap.add_argument("--orders", default="ref,fast")
    ap.add_argument("--nw", default="8,12,16,24")
    ap.add_argument("--d", default="4,6")
    ap.add_argument("--fin", default="0,1")
    ap.add_argument("--size", type=int, default=8192)
    ap.add_argument("--steps-f32", type=int, default=200)
    ap.add_argument("--steps-f64", type=int, default=20)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--margin", type=float, default=0.01, help="relative gain needed to leave the built-in choice")
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 4)
    ap.add_argument("--write", action="store_true", help="rewrite csrc/tune2d.cuh with the chosen table")
    ap.add_argument("--json", default="", help="write candidates, spills and timings here")
    ap.add_argument("--apply", default="", help="only rewrite csrc/tune2d.cuh from the table of a --json file")
    a = ap.parse_args(argv)
    if a.apply:
        with open(a.apply) as f:
            write_table(json.load(f)["table"])
        print("wrote", TABLE)
        return 0
    dtypes, orders = a.dtypes.split(","), a.orders.split(",")
    nws, ds, fins = ([int(x) for x in s.split(",")] for s in (a.nw, a.d, a.fin))

    B.build()
    os.makedirs(TUNE_DIR, exist_ok=True)
    jobs = [(f"s2d_{dt}_{o}", nw, d, fin) for dt in dtypes for o in orders for nw, d, fin in candidates(o, nws, ds, fins)]
    t0 = time.time()
    with cf.ThreadPoolExecutor(max_workers=a.jobs) as ex:
        built = list(ex.map(lambda j: compile_variant(*j), jobs))
        # the built-in choice of each unit, for its spill figures
        defaults = list(ex.map(compile_default, sorted({j[0] for j in jobs})))
    print(f"compiled {len(built)} candidates in {time.time() - t0:.0f}s", flush=True)
    spills = {v["name"]: v["shapes"] for v in built if v["ok"]}
    spills.update({d["name"]: d["shapes"] for d in defaults})
    for v in built:
        if not v["ok"]:
            print("compile failed:", v["name"], v["error"][-400:], file=sys.stderr)
    libs = {"default": Lib(B.LIB)}
    with cf.ThreadPoolExecutor(max_workers=a.jobs) as ex:
        paths = list(ex.map(link_variant, [v for v in built if v["ok"]]))
    for v, p in zip([v for v in built if v["ok"]], paths):
        libs[v["name"]] = Lib(p)
    results = measure(libs, dtypes, orders, a.size, {"f32": a.steps_f32, "f64": a.steps_f64}, a.reps)
    table = choose(results, spills, a.margin)
    print(json.dumps(table, indent=1))
    if a.json:
        with open(a.json, "w") as f:
            json.dump({"spills": spills, "results": results, "table": table}, f, indent=1)
    if a.write:
        write_table(table)
        print("wrote", TABLE)
    return 0


if __name__ == "__main__":
    sys.exit(main())
