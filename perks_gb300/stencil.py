"""Host-side mirror of the reference's stencil interface.

* ``jacobi_iterative`` / ``j3d_iterative`` keep the argument list of the
  reference's host API (stencil/2dstencil/common/jacobi_cuda.cuh:6-10,
  stencil/3dstencil/common/jacobi_cuda.cuh:6-10) over host (numpy) arrays and
  return its int status; the shape, fixed per executable in the reference by
  -D macros, is a keyword argument.
* ``stencil2d`` / ``stencil3d`` run on device tensors (torch is used only to
  own device memory and streams) and return the output and launch stats.

Every call goes through libperks_gb300.so; there is no other code path.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N


def _opts(shape: str, dtype, order="reference", kernel="persistent", boundary="clamp", cache_rows=None,
          l2_sweep=False, ctas=0, stream=None, tma=False) -> N.StencilOpts:
    """Options for one call; cache_rows None keeps the library's default
    (2D: as many resident rows as fit; 3D: no resident planes)."""
    if shape not in N.SHAPES:
        raise ValueError(f"unknown shape {shape!r}")
    o = N.StencilOpts()
    dt = N.FP64 if np.dtype(dtype) == np.float64 else N.FP32
    N.lib().perks_stencil_default_opts(ctypes.byref(o), N.SHAPES[shape], dt)
    o.order = {"reference": N.ORDER_REFERENCE, "fast": N.ORDER_FAST}[order]
    o.kernel = {"persistent": N.KERNEL_PERSISTENT, "per_step": N.KERNEL_PER_STEP, "naive": N.KERNEL_NAIVE}[kernel]
    o.boundary = {"clamp": N.CLAMP, "dirichlet": N.DIRICHLET}[boundary]
    if cache_rows is not None:
        o.cache_rows = int(cache_rows)
    o.l2_sweep = int(bool(l2_sweep))
    o.ctas = int(ctas)
    o.stream = stream
    o.tma = int(bool(tma))
    return o


def _stats(st: N.StencilStats) -> dict:
    return {k: getattr(st, k) for k, _ in N.StencilStats._fields_}


def _torch_dtype_np(t):
    import torch
    if t.dtype == torch.float32:
        return np.float32
    if t.dtype == torch.float64:
        return np.float64
    raise TypeError("stencil fields must be float32 or float64")


def stencil2d(field, shape: str, steps: int, out=None, **kw):
    """`steps` Jacobi steps of a 2D shape on a CUDA tensor (wy, wx)."""
    import torch
    if field.dim() != 2 or not field.is_cuda:
        raise ValueError("field must be a 2D CUDA tensor")
    field = field.contiguous()
    out = torch.empty_like(field) if out is None else out
    if "stream" not in kw:
        kw["stream"] = ctypes.c_void_p(torch.cuda.current_stream(field.device).cuda_stream)
    o = _opts(shape, _torch_dtype_np(field), **kw)
    st = N.StencilStats()
    N.check(N.lib().perks_stencil2d(ctypes.byref(o), field.data_ptr(), out.data_ptr(), field.shape[0],
                                    field.shape[1], int(steps), ctypes.byref(st)))
    return out, _stats(st)


def stencil3d(field, shape: str, steps: int, out=None, **kw):
    """`steps` Jacobi steps of a 3D shape on a CUDA tensor (h, wy, wx)."""
    import torch
    if field.dim() != 3 or not field.is_cuda:
        raise ValueError("field must be a 3D CUDA tensor")
    field = field.contiguous()
    out = torch.empty_like(field) if out is None else out
    if "stream" not in kw:
        kw["stream"] = ctypes.c_void_p(torch.cuda.current_stream(field.device).cuda_stream)
    o = _opts(shape, _torch_dtype_np(field), **kw)
    st = N.StencilStats()
    N.check(N.lib().perks_stencil3d(ctypes.byref(o), field.data_ptr(), out.data_ptr(), field.shape[0],
                                    field.shape[1], field.shape[2], int(steps), ctypes.byref(st)))
    return out, _stats(st)


def min_domain_2d(shape: str, width_x: int, dtype=np.float32, **kw) -> int:
    """Largest width_y that the persistent 2D kernel keeps on chip between
    steps for this width_x (the reference's --small mode, getMinWidthY,
    stencil/2dstencil/jacobi-2d.cu:79-136); 0 when the options cache nothing."""
    o = _opts(shape, dtype, **kw)
    wy = ctypes.c_int(0)
    N.check(N.lib().perks_stencil2d_min_domain(ctypes.byref(o), int(width_x), ctypes.byref(wy)))
    return wy.value


def min_domain_3d(shape: str, width_y: int, width_x: int, dtype=np.float32, **kw) -> int:
    """Largest height at which the persistent 3D kernel keeps every plane
    tile that no other CTA reads on chip between steps (the reference's
    getminHeight, stencil/3dstencil/j3d.driver.cpp:62-144); 0 when no plane
    tile fits or the options cache nothing."""
    o = _opts(shape, dtype, **kw)
    h = ctypes.c_int(0)
    N.check(N.lib().perks_stencil3d_min_domain(ctypes.byref(o), int(width_y), int(width_x), ctypes.byref(h)))
    return h.value


def getMinWidthY(width_x: int, bdimx: int = 256, registers: int = 0, useSM: bool = True, blkpsm: int = 0,
                 isDoubleTile: bool = False, *, shape: str = "2d5pt", dtype=np.float32) -> int:
    """Reference signature (stencil/2dstencil/common/jacobi_cuda.cuh:14): the
    minimum-domain width_y, or a negative status."""
    dt = N.FP64 if np.dtype(dtype) == np.float64 else N.FP32
    return N.lib().perks_get_min_width_y(N.SHAPES[shape], dt, int(width_x), bdimx, registers, int(useSM),
                                         blkpsm, int(isDoubleTile))


def jacobi_iterative(h_input: np.ndarray, width_y: int, width_x: int, output: np.ndarray, bdimx: int = 256,
                     blkpsm: int = 0, iteration: int = 3, async_: bool = False, useSM: bool = True,
                     usewarmup: bool = False, warmupiteration: int = -1, isDoubleTile: bool = False, *,
                     shape: str = "2d5pt") -> int:
    """Reference host API (jacobi-2d.cu:371): host arrays in and out, int status."""
    if h_input.dtype not in (np.float32, np.float64) or output.dtype != h_input.dtype:
        raise TypeError("float32 or float64 arrays of one dtype")
    if not (h_input.flags["C_CONTIGUOUS"] and output.flags["C_CONTIGUOUS"]):
        raise ValueError("arrays must be C-contiguous")
    fn = N.lib().perks_jacobi_iterative_f64 if h_input.dtype == np.float64 else N.lib().perks_jacobi_iterative_f32
    return fn(N.SHAPES[shape], h_input.ctypes.data, width_y, width_x, output.ctypes.data, bdimx, blkpsm,
              iteration, int(async_), int(useSM), int(usewarmup), warmupiteration, int(isDoubleTile))


def j3d_iterative(h_input: np.ndarray, height: int, width_y: int, width_x: int, output: np.ndarray,
                  bdimx: int = 256, blkpsm: int = 0, iteration: int = 3, useSM: bool = True,
                  usewarmup: bool = False, warmupiteration: int = -1, isDoubleTile: bool = False,
                  getminHeight: bool = False, *, shape: str = "3d7pt") -> int:
    """Reference host API (j3d.cu:129): host arrays in and out, int status."""
    if getminHeight:
        is64 = h_input is not None and np.dtype(h_input.dtype) == np.float64
        fn = N.lib().perks_j3d_iterative_f64 if is64 else N.lib().perks_j3d_iterative_f32
        return fn(N.SHAPES[shape], None, height, width_y, width_x, None, bdimx, blkpsm, iteration,
                  int(useSM), 0, warmupiteration, int(isDoubleTile), 1)
    if h_input.dtype not in (np.float32, np.float64) or output.dtype != h_input.dtype:
        raise TypeError("float32 or float64 arrays of one dtype")
    fn = N.lib().perks_j3d_iterative_f64 if h_input.dtype == np.float64 else N.lib().perks_j3d_iterative_f32
    return fn(N.SHAPES[shape], h_input.ctypes.data, height, width_y, width_x, output.ctypes.data, bdimx,
              blkpsm, iteration, int(useSM), int(usewarmup), warmupiteration, int(isDoubleTile),
              int(getminHeight))


def last_error() -> str:
    return N.lib().perks_last_error().decode(errors="replace")
