"""ORACLE — test infrastructure only.

ctypes access to the CPU restatement (``liboracle.so``, built from
stencil_oracle.c / cg_oracle.c) and, where it was built, to the reference's
own CPU gold code (``_ref/libref_<shape>.so``, compiled unmodified from the
reference sources by this directory's Makefile).

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline import this
module, to check results against and to time the CPU path.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")

SHAPES_2D = {"2d5pt": 0, "2ds9pt": 1, "2d13pt": 2, "2d17pt": 3, "2d21pt": 4,
             "2ds25pt": 5, "2d9pt": 6, "2d25pt": 7}
SHAPES_3D = {"3d7pt": 16, "3d13pt": 17, "3d17pt": 18, "3d27pt": 19, "poisson": 20}
SHAPES = {**SHAPES_2D, **SHAPES_3D}
HALO = {"2d5pt": 1, "2ds9pt": 2, "2d13pt": 3, "2d17pt": 4, "2d21pt": 5, "2ds25pt": 6,
        "2d9pt": 1, "2d25pt": 2, "3d7pt": 1, "3d13pt": 2, "3d17pt": 1, "3d27pt": 1,
        "poisson": 1}

_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double


def reference_dir() -> str | None:
    """The reference checkout whose CPU code builds _ref: $PERKS_REFERENCE_DIR,
    else a checkout named ``reference`` beside this repository; None when
    neither holds the reference's sources."""
    for d in (os.environ.get("PERKS_REFERENCE_DIR"),
              os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")):
        if d and os.path.exists(os.path.join(d, "stencil", "2dstencil", "2d5pt", "jacobi_gold_gen.cpp")):
            return os.path.abspath(d)
    return None


def build(quiet: bool = True) -> None:
    """Run the oracle Makefile (the restatement always; _ref when the
    reference sources are found, see reference_dir)."""
    cmd = ["make", "-C", HERE, "-j8"]
    ref = reference_dir()
    if ref:
        cmd.append("REF=" + ref)
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        _lib = ctypes.CDLL(path)
        for name in ("oracle_stencil2d_f32", "oracle_stencil2d_f64"):
            getattr(_lib, name).argtypes = [_I, _P, _I, _I, _P, _I, _I]
        for name in ("oracle_stencil3d_f32", "oracle_stencil3d_f64"):
            getattr(_lib, name).argtypes = [_I, _P, _I, _I, _I, _P, _I, _I]
        for name in ("oracle_cg_f32", "oracle_cg_f64"):
            getattr(_lib, name).argtypes = [_I, _P, _P, _P, _P, _P, _I, _I, _D, _I, _P, _P]
        _lib.oracle_cg_dia_f64.argtypes = [_I, _I, _P, _P, _P, _P, _I, _I, _D, _I, _P, _P]
        _lib.oracle_spmv_csr_f64.argtypes = [_I, _P, _P, _P, _P, _P]
        _lib.oracle_spmv_csr_f32.argtypes = [_I, _P, _P, _P, _P, _P]
        _lib.oracle_spmv_dia_f64.argtypes = [_I, _I, _P, _P, _P, _P]
        _lib.oracle_gen_tridiag_f32.argtypes = [_I, ctypes.c_uint, _P, _P, _P]
        _lib.oracle_gen_tridiag_f64.argtypes = [_I, ctypes.c_uint, _P, _P, _P]
    return _lib


def _ptr(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def _sfx(dtype) -> str:
    return "f32" if np.dtype(dtype) == np.float32 else "f64"


def stencil(shape: str, field: np.ndarray, steps: int, boundary: int = 0) -> np.ndarray:
    """Run `steps` Jacobi steps of `shape` on a 2D (wy, wx) or 3D (h, wy, wx)
    float32/float64 array with the CPU restatement."""
    field = np.ascontiguousarray(field)
    out = np.empty_like(field)
    sid = SHAPES[shape]
    if field.ndim == 2:
        fn = getattr(lib(), "oracle_stencil2d_" + _sfx(field.dtype))
        rc = fn(sid, _ptr(field), field.shape[0], field.shape[1], _ptr(out), steps, boundary)
    else:
        fn = getattr(lib(), "oracle_stencil3d_" + _sfx(field.dtype))
        rc = fn(sid, _ptr(field), field.shape[0], field.shape[1], field.shape[2], _ptr(out),
                steps, boundary)
    if rc != 0:
        raise ValueError(f"oracle stencil failed ({rc})")
    return out


def num_threads() -> int:
    lib().oracle_num_threads.restype = _I
    return lib().oracle_num_threads()


def set_num_threads(n: int) -> int:
    """Threads of the oracle's parallel loops from now on (n <= 0: all
    cores); returns the previous count."""
    L = lib()
    L.oracle_set_num_threads.restype = _I
    L.oracle_set_num_threads.argtypes = [_I]
    return L.oracle_set_num_threads(int(n))


def ref_available(shape: str | None = None) -> bool:
    name = "libref_cg.so" if shape is None else f"libref_{shape}.so"
    return os.path.exists(os.path.join(REF_DIR, name))


_ref_libs: dict = {}


def _ref_lib(name: str) -> ctypes.CDLL:
    if name not in _ref_libs:
        path = os.path.join(REF_DIR, f"libref_{name}.so")
        # RTLD_LOCAL: every shape defines the same template symbols.
        _ref_libs[name] = ctypes.CDLL(path, mode=ctypes.RTLD_LOCAL)
    return _ref_libs[name]


def ref_stencil(shape: str, field: np.ndarray, steps: int) -> np.ndarray:
    """Run the reference's own CPU gold code (clamp boundary only)."""
    field = np.ascontiguousarray(field).copy()  # the reference takes a non-const pointer
    out = np.zeros_like(field)
    L = _ref_lib(shape)
    if field.ndim == 2:
        fn = getattr(L, "ref_stencil2d_" + _sfx(field.dtype))
        fn.argtypes = [_P, _I, _I, _P, _I]
        fn(_ptr(field), field.shape[0], field.shape[1], _ptr(out), steps)
    else:
        fn = getattr(L, "ref_stencil3d_" + _sfx(field.dtype))
        fn.argtypes = [_P, _I, _I, _I, _P, _I]
        fn(_ptr(field), field.shape[0], field.shape[1], field.shape[2], _ptr(out), steps)
    return out


# ----------------------------------------------------------------------- CG
def cg(row_ptr, col, val, b, x0=None, max_iter=1000, stop=0, tol=1e-10, static_iter=False,
       trace=False):
    """CPU CG restatement. float32 values -> the reference float build,
    float64 -> FP64 oracle. Returns (x, iterations, rr, trace|None)."""
    val = np.ascontiguousarray(val)
    dt = val.dtype
    n = len(row_ptr) - 1
    rp = np.ascontiguousarray(row_ptr, dtype=np.int32)
    ci = np.ascontiguousarray(col, dtype=np.int32)
    b = np.ascontiguousarray(b, dtype=dt)
    x = np.zeros(n, dt) if x0 is None else np.ascontiguousarray(x0, dtype=dt).copy()
    rr = np.zeros(1, np.float64)
    tr = np.zeros(max_iter + 1, np.float64) if trace else None
    fn = getattr(lib(), "oracle_cg_" + _sfx(dt))
    it = fn(n, _ptr(rp), _ptr(ci), _ptr(val), _ptr(b), _ptr(x), max_iter, stop, tol,
            int(static_iter), _ptr(rr), _ptr(tr) if trace else None)
    if tr is not None and it >= 0:
        tr = tr[: it + 1]
    return x, it, float(rr[0]), tr


def cg_dia(offsets, data, b, x0=None, max_iter=1000, stop=0, tol=1e-10, static_iter=False):
    data = np.ascontiguousarray(data, dtype=np.float64)
    off = np.ascontiguousarray(offsets, dtype=np.int32)
    n = data.shape[1]
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros(n) if x0 is None else np.ascontiguousarray(x0, dtype=np.float64).copy()
    rr = np.zeros(1)
    it = lib().oracle_cg_dia_f64(n, len(off), _ptr(off), _ptr(data), _ptr(b), _ptr(x), max_iter,
                                 stop, tol, int(static_iter), _ptr(rr), None)
    return x, it, float(rr[0])


def spmv_csr(row_ptr, col, val, x):
    val = np.ascontiguousarray(val)
    n = len(row_ptr) - 1
    rp = np.ascontiguousarray(row_ptr, dtype=np.int32)
    ci = np.ascontiguousarray(col, dtype=np.int32)
    x = np.ascontiguousarray(x, dtype=val.dtype)
    y = np.empty(n, val.dtype)
    getattr(lib(), "oracle_spmv_csr_" + _sfx(val.dtype))(n, _ptr(rp), _ptr(ci), _ptr(val), _ptr(x), _ptr(y))
    return y


def spmv_dia(offsets, data, x):
    data = np.ascontiguousarray(data, dtype=np.float64)
    off = np.ascontiguousarray(offsets, dtype=np.int32)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty(data.shape[1])
    lib().oracle_spmv_dia_f64(data.shape[1], len(off), _ptr(off), _ptr(data), _ptr(x), _ptr(y))
    return y


def gen_tridiag(n: int, seed: int, dtype=np.float32):
    rp = np.zeros(n + 1, np.int32)
    ci = np.zeros(3 * n - 2, np.int32)
    v = np.zeros(3 * n - 2, dtype)
    getattr(lib(), "oracle_gen_tridiag_" + _sfx(dtype))(n, seed, _ptr(rp), _ptr(ci), _ptr(v))
    return rp, ci, v


def ref_gen_tridiag(n: int, seed: int, dtype=np.float32):
    L = _ref_lib("cg")
    rp = np.zeros(n + 1, np.int32)
    ci = np.zeros(3 * n - 2, np.int32)
    v = np.zeros(3 * n - 2, dtype)
    fn = getattr(L, "ref_gen_tridiag_" + _sfx(dtype))
    fn.argtypes = [_I, ctypes.c_uint, _P, _P, _P]
    fn(n, seed, _ptr(rp), _ptr(ci), _ptr(v))
    return rp, ci, v


def ref_cg_steps(row_ptr, col, val, b, iters: int):
    """The reference's float CG loop body (its own helper functions) for
    `iters` iterations from x0 = 0; returns (x, trace of r.r)."""
    L = _ref_lib("cg")
    n = len(row_ptr) - 1
    rp = np.ascontiguousarray(row_ptr, dtype=np.int32)
    ci = np.ascontiguousarray(col, dtype=np.int32)
    v = np.ascontiguousarray(val, dtype=np.float32)
    x = np.zeros(n, np.float32)
    Ax = np.zeros(n, np.float32)
    p = np.zeros(n, np.float32)
    r = np.ascontiguousarray(b, dtype=np.float32).copy()
    tr = np.zeros(iters + 1)
    L.ref_cg_steps.argtypes = [_P] * 7 + [_I, _I, _I, _P]
    L.ref_cg_steps(_ptr(rp), _ptr(ci), _ptr(v), _ptr(x), _ptr(Ax), _ptr(p), _ptr(r), len(v), n,
                   iters, _ptr(tr))
    return x, tr


def ref_cpu_cg(row_ptr, col, val, b):
    """cpuConjugateGrad exactly as shipped (fixed MAXITER iterations)."""
    L = _ref_lib("cg")
    n = len(row_ptr) - 1
    rp = np.ascontiguousarray(row_ptr, dtype=np.int32)
    ci = np.ascontiguousarray(col, dtype=np.int32)
    v = np.ascontiguousarray(val, dtype=np.float32)
    x = np.zeros(n, np.float32)
    Ax = np.zeros(n, np.float32)
    p = np.zeros(n, np.float32)
    r = np.ascontiguousarray(b, dtype=np.float32).copy()
    L.ref_cpu_cg.argtypes = [_P] * 7 + [_I, _I, ctypes.c_float]
    L.ref_cpu_cg(_ptr(rp), _ptr(ci), _ptr(v), _ptr(x), _ptr(Ax), _ptr(p), _ptr(r), len(v), n, 1e-10)
    L.ref_max_iter.restype = _I
    return x, L.ref_max_iter()
