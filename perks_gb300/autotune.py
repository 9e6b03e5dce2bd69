"""Build-time tuning of the stencil kernels, written as tables.

The reference picks its register-cache depth per shape offline: it compiles
variants, reads the compiler's register and spill report and turns the
results into headers (stencil/2dstencil/ProcessCompilerLog.py,
ProcessRsts2cuh.py -> perksconfig.cuh). This tool does the same for the
GB300 kernels and adds a measurement, because here the choices that matter
change speed without changing registers much. 2D: warps per CTA, rows in
flight per warp, the form of the exact division, rows per copy wait. 3D:
compute warps per CTA, rows per compute warp, KB of planes in flight; 2D
also the 16-byte vectors each lane holds per row (fewer cells per lane: a
smaller register window, so more warps fit).

  1. compile every candidate of every translation unit of the kind with
     -DPERKS_TUNE_* and -Xptxas -v, in parallel (a 2D knob given as 0 keeps
     each shape's table value, so one knob can be swept alone);
  2. record each kernel's spill bytes; a candidate that spills more than the
     built-in choice must win by a wider margin (5 % instead of 1 %);
  3. link one library per candidate and time every shape on the GPU
     (8192^2 / 512^3 fields by default), after checking that its output on a
     ragged field is bit-identical to the built-in kernel's;
  4. keep the fastest candidate per (dtype, order, shape) when it beats the
     kernel the table already selects by more than that margin, and write it
     over that entry.

    python -m perks_gb300.autotune --kind 2d --json t.json   # measure
    python -m perks_gb300.autotune --kind 2d --apply t.json  # write csrc/tune2d.cuh

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
SHAPES3D = ["3d7pt", "3d13pt", "3d17pt", "3d27pt", "poisson"]
TUNE_DIR = os.path.join(B.HERE, "_build", "tune")
SPILL_RE = re.compile(r"(\d+) bytes spill stores")
REGS_RE = re.compile(r"Used (\d+) registers")

KINDS = {
    "2d": {"prefix": "s2d", "shapes": SHAPES2D, "base": 0, "table": os.path.join(B.CSRC, "tune2d.cuh"),
           "decl": "constexpr Tune2D kTune2D[2][2][8]",
           "knobs": [("nw", "PERKS_TUNE_NW"), ("d", "PERKS_TUNE_D"), ("fin", "PERKS_TUNE_FIN"),
                     ("rp", "PERKS_TUNE_RP"), ("nv", "PERKS_TUNE_NV")],
           "kernel_re": re.compile(r"Function properties for _ZN5perks16stencil2d_kernelI[fd]Li(\d+)E")},
    "3d": {"prefix": "s3d", "shapes": SHAPES3D, "base": 16, "table": os.path.join(B.CSRC, "tune3d.cuh"),
           "decl": "constexpr Tune3D kTune3D[2][2][5]",
           "knobs": [("nwc", "PERKS_TUNE3_NWC"), ("ry", "PERKS_TUNE3_RY"), ("dkb", "PERKS_TUNE3_DKB")],
           "kernel_re": re.compile(r"Function properties for _ZN5perks16stencil3d_kernelI[fd]Li(\d+)E")},
}
TABLE = KINDS["2d"]["table"]


def candidates(kind: str, order: str, values: dict):
    """Knob settings to try; the 2D division form only matters in reference order."""
    names = [k for k, _ in KINDS[kind]["knobs"]]
    lists = [[0] if (kind == "2d" and k == "fin" and order != "ref") else values[k] for k in names]
    for combo in itertools.product(*lists):
        yield dict(zip(names, combo))


def variant_name(tu: str, knobs: dict) -> str:
    return tu + "".join(f"_{k}{v}" for k, v in knobs.items())


def parse_variant(name: str) -> dict:
    """Knob values from a variant name such as s3d_f32_ref_nwc11_ry3_dkb72."""
    tail = name.split("_", 3)[3]
    return {k: int(v) for k, v in re.findall(r"([a-z]+)(\d+)", tail)}


def ptxas_report(text: str, kind: str = "2d") -> dict:
    """{shape position: {"regs": R, "spill": bytes}} of the stencil kernels in -Xptxas -v output."""
    K = KINDS[kind]
    shapes, cur = {}, None
    for line in text.splitlines():
        m = K["kernel_re"].search(line)
        if m:
            cur = int(m.group(1)) - K["base"]
            continue
        m = SPILL_RE.search(line)
        if m and cur is not None:
            shapes.setdefault(cur, {})["spill"] = int(m.group(1))
        m = REGS_RE.search(line)
        if m and cur is not None:
            shapes.setdefault(cur, {})["regs"] = int(m.group(1))
            cur = None
    return shapes


def compile_variant(kind: str, tu: str, knobs: dict | None) -> dict:
    """Compile one candidate (knobs=None: the built-in choice) of a translation
    unit; report per-shape registers and spills."""
    name = variant_name(tu, knobs) if knobs else f"{tu}_default"
    obj = os.path.join(TUNE_DIR, name + ".o")
    macros = [f"-D{m}={knobs[k]}" for k, m in KINDS[kind]["knobs"]] if knobs else []
    cmd = ([B.nvcc()] + B.ARCH + B.NVCC_FLAGS + macros +
           ["-Xptxas", "-v", "-c", os.path.join(B.CSRC, tu + ".cu"), "-o", obj])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return {"name": name, "ok": False, "error": (r.stderr or r.stdout)[-2000:]}
    return {"name": name, "ok": True, "obj": obj, "tu": tu, "shapes": ptxas_report(r.stderr, kind)}


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
        P = ctypes.POINTER
        self.L.perks_stencil_default_opts.argtypes = [P(N.StencilOpts), ctypes.c_int, ctypes.c_int]
        self.L.perks_stencil2d.argtypes = [P(N.StencilOpts), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_int, P(N.StencilStats)]
        self.L.perks_stencil3d.argtypes = [P(N.StencilOpts), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_int, ctypes.c_int, P(N.StencilStats)]
        self.L.perks_last_error.restype = ctypes.c_char_p

    def run(self, shape: str, dt: int, order: int, src, dst, steps: int, stream) -> N.StencilStats:
        o = N.StencilOpts()
        self.L.perks_stencil_default_opts(ctypes.byref(o), N.SHAPES[shape], dt)
        o.order = order
        o.stream = stream
        st = N.StencilStats()
        if src.dim() == 2:
            rc = self.L.perks_stencil2d(ctypes.byref(o), src.data_ptr(), dst.data_ptr(), src.shape[0], src.shape[1],
                                        steps, ctypes.byref(st))
        else:
            rc = self.L.perks_stencil3d(ctypes.byref(o), src.data_ptr(), dst.data_ptr(), src.shape[0], src.shape[1],
                                        src.shape[2], steps, ctypes.byref(st))
        if rc != 0:
            raise RuntimeError(self.L.perks_last_error().decode())
        return st


def measure(kind: str, libs: dict, dtypes, orders, size: int, steps: dict, reps: int, only=()) -> dict:
    import torch
    dev = torch.device("cuda:0")
    stream = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    big_dims = (size, size) if kind == "2d" else (size, size, size)
    small_dims = (700, 2100) if kind == "2d" else (20, 45, 300)
    out = {}
    for dtn in dtypes:
        tdt = torch.float32 if dtn == "f32" else torch.float64
        idt = torch.int32 if dtn == "f32" else torch.int64
        dt = N.FP32 if dtn == "f32" else N.FP64
        g = torch.Generator(device="cpu").manual_seed(1234)
        big = torch.rand(big_dims, generator=g, dtype=tdt).to(dev)
        small = torch.rand(small_dims, generator=g, dtype=tdt).to(dev)
        o_big, o_ref, o_var = torch.empty_like(big), torch.empty_like(small), torch.empty_like(small)
        for ordn in orders:
            order = N.ORDER_REFERENCE if ordn == "ref" else N.ORDER_FAST
            for shape in KINDS[kind]["shapes"]:
                if only and shape not in only:
                    continue
                key = f"{dtn}/{ordn}/{shape}"
                libs["default"].run(shape, dt, order, small, o_ref, 7, stream)
                res = {}
                for name, lib in libs.items():
                    if name != "default" and not name.startswith(f"{KINDS[kind]['prefix']}_{dtn}_{ordn}_"):
                        continue
                    try:
                        if name != "default":
                            lib.run(shape, dt, order, small, o_var, 7, stream)
                            torch.cuda.synchronize()
                            if not torch.equal(o_var.view(idt), o_ref.view(idt)):
                                res[name] = {"error": "output differs from the built-in kernel"}
                                continue
                        lib.run(shape, dt, order, big, o_big, max(2, steps[dtn] // 10), stream)
                        best = 0.0
                        for _ in range(reps):
                            best = max(best, lib.run(shape, dt, order, big, o_big, steps[dtn], stream).gcells_per_s)
                    except RuntimeError as e:  # e.g. a ring larger than shared memory
                        res[name] = {"error": str(e)}
                        continue
                    res[name] = {"gcells": round(best, 2)}
                out[key] = res
                print(key, json.dumps(res), flush=True)
        del big, small, o_big, o_ref, o_var
        torch.cuda.empty_cache()
    return out


def choose(results: dict, spills: dict, margin: float, kind: str = "2d", spill_margin: float = 0.05) -> dict:
    """Fastest candidate per key that beats the current kernel by more than
    `margin` (relative), or by more than `spill_margin` when it spills more
    than the built-in choice (its speed then depends more on the memory
    system than the measurement shows)."""
    K = KINDS[kind]
    table = {}

    def spill_of(name, si):
        sh = spills.get(name, {})
        return (sh.get(si) or sh.get(str(si)) or {}).get("spill")

    for key, res in results.items():
        dtn, ordn, shape = key.split("/")
        si = K["shapes"].index(shape)
        base = res.get("default", {}).get("gcells", 0.0)
        ref_spill = spill_of(f"{K['prefix']}_{dtn}_{ordn}_default", si) or 0
        best, best_v = 0.0, None
        for name, r in res.items():
            if name == "default" or "gcells" not in r:
                continue
            sp = spill_of(name, si)
            if sp is None:
                continue
            need = base * (1.0 + (spill_margin if sp > ref_spill else margin))
            if r["gcells"] > need and r["gcells"] > best:
                best, best_v = r["gcells"], name
        if best_v:
            table[key] = dict(parse_variant(best_v), gcells=best, default_gcells=base)
    return table


def read_table(path: str = TABLE, kind: str = "2d") -> dict:
    """The entries of a table header, keyed like choose()'s result (all-zero entries left out)."""
    K = KINDS[kind]
    src = open(path).read()
    body = src[src.index("// BEGIN TABLE\n"):src.index("// END TABLE")]
    body = body[body.index("= {") + 3:]
    cells = re.findall(r"\{([\d,\s]+)\}", body)
    names = [k for k, _ in K["knobs"]]
    out = {}
    keys = [f"{d}/{o}/{sh}" for d in ("f32", "f64") for o in ("ref", "fast") for sh in K["shapes"]]
    for key, cell in zip(keys, cells):
        vals = [int(x) for x in cell.split(",")]
        if any(vals):
            out[key] = dict(zip(names, vals + [0] * (len(names) - len(vals))))
    return out


def merge_table(path: str, kind: str, table: dict) -> dict:
    """The header's table with the new winners written over it. Candidates
    are measured against the kernels the header already selects, so an entry
    without a winner keeps its current value, and a winner's knob of 0 (the
    kernels then keep the table's value; the 2D division form has no such
    value) keeps the entry's current one."""
    merged = read_table(path, kind)
    for k, v in table.items():
        old = merged.get(k, {})
        merged[k] = {n: (v[n] if (v[n] or n == "fin") else old.get(n, 0)) for n, _ in KINDS[kind]["knobs"]}
    return merged


def write_table(table: dict, path: str = TABLE, kind: str = "2d") -> None:
    K = KINDS[kind]
    names = [k for k, _ in K["knobs"]]
    zero = "{" + ", ".join("0" for _ in names) + "}"
    rows = []
    for dtn in ("f32", "f64"):
        orows = []
        for ordn in ("ref", "fast"):
            cells = []
            for shape in K["shapes"]:
                t = table.get(f"{dtn}/{ordn}/{shape}")
                cells.append("{" + ", ".join(str(t.get(k, 0)) for k in names) + "}" if t else zero)
            orows.append("{" + ", ".join(cells) + "}")
        rows.append("{" + ",\n   ".join(orows) + "}")
    body = K["decl"] + " = {\n  " + ",\n  ".join(rows) + "};\n"
    src = open(path).read()
    a, b = src.index("// BEGIN TABLE\n") + len("// BEGIN TABLE\n"), src.index("// END TABLE")
    with open(path, "w") as f:
        f.write(src[:a] + body + src[b:])


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--kind", default="2d", choices=sorted(KINDS))
    ap.add_argument("--dtypes", default="f32,f64")
    ap.add_argument("--orders", default="ref,fast")
    ap.add_argument("--nw", default="8,12,16,24", help="2D warps per CTA")
    ap.add_argument("--d", default="4,6", help="2D rows in flight per warp")
    ap.add_argument("--fin", default="0,1,2", help="2D division form (reference order)")
    ap.add_argument("--rp", default="1,2", help="2D rows per copy wait")
    ap.add_argument("--nv", default="0", help="2D 16-byte vectors per lane (0 = built-in)")
    ap.add_argument("--shapes", default="", help="only these shapes (comma-separated)")
    ap.add_argument("--nwc", default="6,8,11,15", help="3D compute warps per CTA")
    ap.add_argument("--ry", default="2,3,4", help="3D rows per compute warp")
    ap.add_argument("--dkb", default="72", help="3D KB of planes in flight")
    ap.add_argument("--size", type=int, default=0, help="field edge (default 8192 for 2D, 512 for 3D)")
    ap.add_argument("--steps-f32", type=int, default=0)
    ap.add_argument("--steps-f64", type=int, default=0)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--margin", type=float, default=0.01, help="relative gain needed to leave the built-in choice")
    ap.add_argument("--jobs", type=int, default=os.cpu_count() or 4)
    ap.add_argument("--write", action="store_true", help="rewrite the kind's table header with the chosen values")
    ap.add_argument("--json", default="", help="write candidates, spills and timings here")
    ap.add_argument("--apply", default="", help="only rewrite the table header from the table of a --json file")
    ap.add_argument("--rechoose", action="store_true", help="with --apply: choose again from the file's timings")
    a = ap.parse_args(argv)
    if a.apply:
        with open(a.apply) as f:
            d = json.load(f)
        kind = d.get("kind", "2d")
        path = KINDS[kind]["table"]
        table = choose(d["results"], d["spills"], a.margin, kind) if a.rechoose else d["table"]
        write_table(merge_table(path, kind, table), path, kind)
        print("wrote", KINDS[kind]["table"])
        return 0
    K = KINDS[a.kind]
    dtypes, orders = a.dtypes.split(","), a.orders.split(",")
    values = {k: [int(x) for x in getattr(a, k).split(",")] for k, _ in K["knobs"]}
    size = a.size or (8192 if a.kind == "2d" else 512)
    steps = {"f32": a.steps_f32 or (200 if a.kind == "2d" else 20),
             "f64": a.steps_f64 or (20 if a.kind == "2d" else 5)}

    B.build()
    os.makedirs(TUNE_DIR, exist_ok=True)
    tus = [f"{K['prefix']}_{dt}_{o}" for dt in dtypes for o in orders]
    jobs = [(a.kind, tu, kn) for tu in tus for kn in candidates(a.kind, tu.split("_")[2], values)]
    jobs += [(a.kind, tu, None) for tu in tus]
    t0 = time.time()
    with cf.ThreadPoolExecutor(max_workers=a.jobs) as ex:
        built = list(ex.map(lambda j: compile_variant(*j), jobs))
    print(f"compiled {len(built)} units in {time.time() - t0:.0f}s", flush=True)
    for v in built:
        if not v["ok"]:
            print("compile failed:", v["name"], v["error"][-400:], file=sys.stderr)
    spills = {v["name"]: v["shapes"] for v in built if v["ok"]}
    cands = [v for v in built if v["ok"] and not v["name"].endswith("_default")]
    with cf.ThreadPoolExecutor(max_workers=a.jobs) as ex:
        paths = list(ex.map(link_variant, cands))
    libs = {"default": Lib(B.LIB)}
    for v, p in zip(cands, paths):
        libs[v["name"]] = Lib(p)
    results = measure(a.kind, libs, dtypes, orders, size, steps, a.reps,
                      tuple(s for s in a.shapes.split(",") if s))
    table = choose(results, spills, a.margin, a.kind)
    print(json.dumps(table, indent=1))
    if a.json:
        with open(a.json, "w") as f:
            json.dump({"kind": a.kind, "spills": spills, "results": results, "table": table}, f, indent=1)
    if a.write:
        write_table(merge_table(K["table"], a.kind, table), K["table"], a.kind)
        print("wrote", K["table"])
    return 0


if __name__ == "__main__":
    sys.exit(main())
