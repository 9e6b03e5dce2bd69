"""ctypes binding of libperks_gb300.so (the C ABI in include/perks.h).

The library is built in-tree by perks_gb300/build.py. Loading never falls
back to anything else: if the library is missing or does not load, the
import of the compute entry points raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libperks_gb300.so")

c_int, c_double, c_void_p = ctypes.c_int, ctypes.c_double, ctypes.c_void_p

# enums (include/perks.h)
PERKS_OK = 0
ERR = {
    -10: "PERKS_ERR_INVALID_ARG", -11: "PERKS_ERR_UNSUPPORTED", -12: "PERKS_ERR_NO_DEVICE",
    -13: "PERKS_ERR_CUDA", -14: "PERKS_ERR_OOM", -15: "PERKS_ERR_TIMEOUT", -16: "PERKS_ERR_LAUNCH",
    -17: "PERKS_ERR_BREAKDOWN", -18: "PERKS_ERR_NOT_CONVERGED",
}
SHAPES = {"2d5pt": 0, "2ds9pt": 1, "2d13pt": 2, "2d17pt": 3, "2d21pt": 4, "2ds25pt": 5,
          "2d9pt": 6, "2d25pt": 7, "3d7pt": 16, "3d13pt": 17, "3d17pt": 18, "3d27pt": 19,
          "poisson": 20}
HALO = {"2d5pt": 1, "2ds9pt": 2, "2d13pt": 3, "2d17pt": 4, "2d21pt": 5, "2ds25pt": 6,
        "2d9pt": 1, "2d25pt": 2, "3d7pt": 1, "3d13pt": 2, "3d17pt": 1, "3d27pt": 1, "poisson": 1}
FP32, FP64, MIXED = 0, 1, 2
CLAMP, DIRICHLET = 0, 1
ORDER_REFERENCE, ORDER_FAST = 0, 1
KERNEL_PERSISTENT, KERNEL_PER_STEP, KERNEL_NAIVE = 0, 1, 2
STOP_ABS_RR, STOP_REL = 0, 1
CG_PLAIN, CG_SINGLE_REDUCTION = 0, 1


class StencilOpts(ctypes.Structure):
    _fields_ = [("shape", c_int), ("dtype", c_int), ("boundary", c_int), ("order", c_int),
                ("kernel", c_int), ("cache_rows", c_int), ("l2_sweep", c_int), ("tile_x", c_int),
                ("tile_y", c_int), ("ctas", c_int), ("stream", c_void_p), ("tma", c_int)]


class StencilStats(ctypes.Structure):
    _fields_ = [("ms", c_double), ("gcells_per_s", c_double), ("cached_fraction", c_double),
                ("grid_x", c_int), ("grid_y", c_int), ("grid_z", c_int), ("tile_x", c_int),
                ("tile_y", c_int), ("cached_rows", c_int), ("launches", c_int)]


class CgState(ctypes.Structure):
    _fields_ = [("d_r", c_void_p), ("d_p", c_void_p), ("d_xs", c_void_p), ("rr", c_double), ("rr_prev", c_double),
                ("bb", c_double), ("maxrr", c_double), ("outer", c_int), ("since", c_int), ("k", c_int),
                ("kernel", c_int), ("dtype", c_int), ("n", c_int)]


class CgOpts(ctypes.Structure):
    _fields_ = [("dtype", c_int), ("stop", c_int), ("tol", c_double), ("max_iter", c_int),
                ("static_iter", c_int), ("kernel", c_int), ("replace_every", c_int), ("ctas", c_int),
                ("stream", c_void_p), ("checkpoint", ctypes.POINTER(CgState)), ("cache_vectors", c_int),
                ("cluster", c_int), ("algorithm", c_int)]


class CgResult(ctypes.Structure):
    _fields_ = [("iterations", c_int), ("outer", c_int), ("rr", c_double), ("true_rel_res", c_double),
                ("ms", c_double), ("launches", c_int), ("layout", c_int), ("ctas", c_int)]


class Job(ctypes.Structure):
    _fields_ = [("kind", c_int), ("dtype", c_int), ("shape", c_int), ("h", c_int), ("wy", c_int), ("wx", c_int),
                ("steps", c_int), ("d_in", c_void_p), ("d_out", c_void_p), ("n", c_int), ("nnz", c_int),
                ("d_row_ptr", c_void_p), ("d_col", c_void_p), ("d_val", c_void_p), ("d_b", c_void_p),
                ("d_x", c_void_p), ("tol", c_double), ("max_iter", c_int)]


class JobResult(ctypes.Structure):
    _fields_ = [("iterations", c_int), ("status", c_int), ("rel_res", c_double)]


class BatchOpts(ctypes.Structure):
    _fields_ = [("threads", c_int), ("ctas_per_sm", c_int), ("stream", c_void_p), ("slicing", c_int)]


class BatchStats(ctypes.Structure):
    _fields_ = [("ms", c_double), ("threads", c_int), ("ctas_per_sm", c_int), ("grid", c_int),
                ("resident_jobs", c_int), ("tuned", c_int), ("sliced_jobs", c_int), ("slicing", c_int)]


JOB_STENCIL, JOB_CG = 0, 1

# Every function the header declares, with its ctypes signature.
SIGNATURES = {
    "perks_stencil_default_opts": (None, [ctypes.POINTER(StencilOpts), c_int, c_int]),
    "perks_stencil2d": (c_int, [ctypes.POINTER(StencilOpts), c_void_p, c_void_p, c_int, c_int, c_int,
                                ctypes.POINTER(StencilStats)]),
    "perks_stencil3d": (c_int, [ctypes.POINTER(StencilOpts), c_void_p, c_void_p, c_int, c_int, c_int, c_int,
                                ctypes.POINTER(StencilStats)]),
    "perks_stencil2d_noalloc": (c_int, [ctypes.POINTER(StencilOpts), c_void_p, c_void_p, c_int, c_int, c_int,
                                        ctypes.POINTER(StencilStats)]),
    "perks_stencil2d_min_domain": (c_int, [ctypes.POINTER(StencilOpts), c_int, ctypes.POINTER(c_int)]),
    "perks_stencil3d_min_domain": (c_int, [ctypes.POINTER(StencilOpts), c_int, c_int, ctypes.POINTER(c_int)]),
    "perks_get_min_width_y": (c_int, [c_int] * 8),
    "perks_jacobi_iterative_f32": (c_int, [c_int, c_void_p, c_int, c_int, c_void_p] + [c_int] * 8),
    "perks_jacobi_iterative_f64": (c_int, [c_int, c_void_p, c_int, c_int, c_void_p] + [c_int] * 8),
    "perks_j3d_iterative_f32": (c_int, [c_int, c_void_p, c_int, c_int, c_int, c_void_p] + [c_int] * 8),
    "perks_j3d_iterative_f64": (c_int, [c_int, c_void_p, c_int, c_int, c_int, c_void_p] + [c_int] * 8),
    "perks_cg_default_opts": (None, [ctypes.POINTER(CgOpts)]),
    "perks_cg_csr": (c_int, [c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                             ctypes.POINTER(CgOpts), ctypes.POINTER(CgResult)]),
    "perks_cg_dia": (c_int, [c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                             ctypes.POINTER(CgOpts), ctypes.POINTER(CgResult)]),
    "perks_spmv_csr": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                               c_void_p]),
    "perks_spmv_dia": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "perks_batch_default_opts": (None, [ctypes.POINTER(BatchOpts)]),
    "perks_batch_plan_create": (c_int, [ctypes.POINTER(Job), c_int, ctypes.POINTER(BatchOpts),
                                        ctypes.POINTER(c_void_p)]),
    "perks_batch_plan_run": (c_int, [c_void_p, c_void_p, ctypes.POINTER(BatchStats)]),
    "perks_batch_plan_results": (c_int, [c_void_p, ctypes.POINTER(JobResult)]),
    "perks_batch_plan_destroy": (None, [c_void_p]),
    "perks_mtx_size": (c_int, [ctypes.c_char_p, ctypes.POINTER(c_int), ctypes.POINTER(c_int),
                               ctypes.POINTER(ctypes.c_longlong)]),
    "perks_mtx_read_csr": (c_int, [ctypes.c_char_p, c_int, ctypes.c_longlong, c_void_p, c_void_p, c_void_p,
                                   ctypes.POINTER(ctypes.c_longlong)]),
    "perks_probe_fma_peak": (c_int, [c_int, ctypes.POINTER(c_double), ctypes.POINTER(c_double)]),
    "perks_last_error": (ctypes.c_char_p, []),
    "perks_status_string": (ctypes.c_char_p, [c_int]),
    "perks_abi_version": (c_int, []),
    "perks_debug_set_wait_fault": (c_int, [ctypes.c_longlong, c_int]),
    "perks_debug_workspace_allocs": (ctypes.c_longlong, []),
    "perks_debug_div_check": (c_int, [c_int, c_int, ctypes.POINTER(ctypes.c_longlong), ctypes.POINTER(ctypes.c_uint)]),
    "perks_launch_count": (ctypes.c_longlong, []),
    "perks_reset_launch_count": (None, []),
}

_lib = None
ABI_VERSION = 3  # PERKS_ABI_VERSION of include/perks.h that the structures above follow


class PerksError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERR.get(code, code)}: {msg}")
        self.code = code


def lib() -> ctypes.CDLL:
    """Load libperks_gb300.so (building it first when absent)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from . import build as _b
            _b.build()
        L = ctypes.CDLL(LIB_PATH)
        L.perks_abi_version.restype = c_int
        if L.perks_abi_version() != ABI_VERSION:
            raise ImportError(f"{LIB_PATH} has ABI version {L.perks_abi_version()}, these bindings need "
                              f"{ABI_VERSION}: rebuild it (perks_gb300.build.build())")
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int) -> int:
    if rc != PERKS_OK:
        msg = lib().perks_last_error().decode(errors="replace")
        raise PerksError(rc, msg)
    return rc
