"""perks_gb300 — GB300 (sm_103a) implementation of the PERKS stencil time
loop and conjugate-gradient iteration behind the reference's host API.

The compute lives in libperks_gb300.so (CUDA kernels + C ABI, include/perks.h);
this package is its ctypes host mirror.
"""
from . import _native
from ._native import PerksError, SHAPES, HALO, lib
from .stencil import (getMinWidthY, j3d_iterative, jacobi_iterative, last_error, min_domain_2d, stencil2d,
                      stencil3d)
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
