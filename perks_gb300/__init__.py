"""perks_gb300 — GB300 (sm_103a) implementation of the PERKS stencil time
loop and conjugate-gradient iteration behind the reference's host API.

The compute lives in libperks_gb300.so (CUDA kernels + C ABI, include/perks.h);
this package is its ctypes host mirror.
"""
from . import _native
from ._native import PerksError, SHAPES, HALO, lib
from .stencil import (getMinWidthY, j3d_iterative, jacobi_iterative, last_error, min_domain_2d, min_domain_3d,
                      stencil2d, stencil3d)
from .cg import CgCheckpoint, cg_csr, cg_dia, spmv_csr, spmv_dia
from .batch import BatchPlan, cg_job, stencil_job

__all__ = ["PerksError", "SHAPES", "HALO", "lib", "jacobi_iterative", "j3d_iterative", "stencil2d",
           "stencil3d", "last_error", "cg_csr", "cg_dia", "spmv_csr", "spmv_dia", "BatchPlan", "cg_job",
           "stencil_job"]


def launch_count() -> int:
    """Kernels this thread launched through the library since the last reset."""
    return int(_native.lib().perks_launch_count())


def reset_launch_count() -> None:
    _native.lib().perks_reset_launch_count()


def fma_peak(dtype: str = "fp64") -> dict:
    """Measured FMA throughput of the current GPU in 'fp64' or 'fp32'
    (perks_probe_fma_peak): fused multiply-adds per second, the FLOP rate
    (twice that) in TFLOP/s, and the timed launch's milliseconds."""
    import ctypes
    rate, ms = ctypes.c_double(), ctypes.c_double()
    _native.check(_native.lib().perks_probe_fma_peak(_native.FP64 if dtype == "fp64" else _native.FP32,
                                                     ctypes.byref(rate), ctypes.byref(ms)))
    return {"dtype": dtype, "fma_per_s": rate.value, "tflops": 2e-12 * rate.value, "ms": ms.value}
