"""Host-side mirror of the reference's CG path.

``cg_csr`` / ``cg_dia`` solve A x = b on the GPU through libperks_gb300.so
(perks_cg_csr / perks_cg_dia), the replacement for the reference's
DispatchCG::ProcessDispatchCG (conjugateGradient/cg_dispatcher.cuh:559-916).
Inputs may be numpy arrays (copied to the device) or CUDA tensors; torch is
used only to own device memory.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N

_DT = {"fp64": N.FP64, "fp32": N.FP32, "mixed": N.MIXED}


def _dev(a, dtype, device):
    import torch
    if isinstance(a, torch.Tensor):
        return a.to(device=device, dtype=dtype).contiguous()
    return torch.from_numpy(np.ascontiguousarray(a)).to(device=device, dtype=dtype)


class CgCheckpoint:
    """CG iteration state between two iterations (perks_cg_state): residual r,
    last search direction p, r.r of the last two iterations, b.b and the
    iteration count; for mixed precision also the FP32 solution increment
    x_s and the reliable-update bookkeeping. Pass it as ``checkpoint=`` to
    cg_csr / cg_dia: a solve resumes from it when it holds a state (k > 0; x0
    must then be the iterate saved with it) and leaves its final state in it.
    ``to_host`` / ``from_host`` move it to numpy (for example to np.savez it
    with x)."""

    _SCALARS = ("rr", "rr_prev", "bb", "maxrr")
    _INTS = ("outer", "since", "k", "kernel", "dtype", "n")

    def __init__(self):
        self.r = None
        self.p = None
        self.xs = None
        self.state = N.CgState()

    @property
    def k(self) -> int:
        return self.state.k

    def _bind(self, n, dtype, device, mixed=False):
        import torch
        if self.r is None:
            self.r = torch.zeros(n, dtype=dtype, device=device)
            self.p = torch.zeros(n, dtype=dtype, device=device)
        if self.r.numel() != n or self.r.dtype != dtype:
            raise ValueError("checkpoint holds a state of another size or dtype")
        if mixed and self.xs is None:
            self.xs = torch.zeros(n, dtype=torch.float32, device=device)
        self.state.d_r = self.r.data_ptr()
        self.state.d_p = self.p.data_ptr()
        self.state.d_xs = self.xs.data_ptr() if self.xs is not None else None
        return ctypes.pointer(self.state)

    def to_host(self) -> dict:
        st = self.state
        d = {"r": self.r.cpu().numpy(), "p": self.p.cpu().numpy()}
        if self.xs is not None:
            d["xs"] = self.xs.cpu().numpy()
        for f in self._SCALARS + self._INTS:
            d[f] = getattr(st, f)
        return d

    @classmethod
    def from_host(cls, d: dict, device="cuda") -> "CgCheckpoint":
        import torch
        c = cls()
        c.r = torch.from_numpy(np.ascontiguousarray(d["r"])).to(device)
        c.p = torch.from_numpy(np.ascontiguousarray(d["p"])).to(device)
        if "xs" in d:
            c.xs = torch.from_numpy(np.ascontiguousarray(d["xs"])).to(device)
        for f in cls._SCALARS:
            setattr(c.state, f, float(d[f]))
        for f in cls._INTS:
            setattr(c.state, f, int(d[f]))
        return c


def _opts(dtype="fp64", stop="rel", tol=1e-10, max_iter=100000, static_iter=False, kernel="persistent",
          replace_every=0, ctas=0, stream=None, cache_vectors=-1, cluster=1, algorithm="plain"):
    o = N.CgOpts()
    N.lib().perks_cg_default_opts(ctypes.byref(o))
    o.dtype = _DT[dtype]
    o.stop = {"abs": N.STOP_ABS_RR, "rel": N.STOP_REL}[stop]
    o.tol = float(tol)
    o.max_iter = int(max_iter)
    o.static_iter = int(bool(static_iter))
    o.kernel = {"persistent": N.KERNEL_PERSISTENT, "per_step": N.KERNEL_PER_STEP}[kernel]
    o.replace_every = int(replace_every)
    o.ctas = int(ctas)
    o.stream = stream
    o.cache_vectors = int(cache_vectors)
    o.cluster = int(cluster)
    o.algorithm = {"plain": N.CG_PLAIN, "single_reduction": N.CG_SINGLE_REDUCTION}[algorithm]
    return o


def _result(r: N.CgResult) -> dict:
    return {k: getattr(r, k) for k, _ in N.CgResult._fields_}


def cg_csr(row_ptr, col, val, b, x0=None, *, dtype="fp64", device="cuda", check=True, checkpoint=None, **kw):
    """Solve with CSR A. dtype: 'fp64', 'fp32' (the reference's float build)
    or 'mixed' (FP32 inner CG, FP64 solution/residual). `checkpoint`: a
    CgCheckpoint to resume from and to save into. Returns (x, result)."""
    import torch
    vdt = torch.float32 if dtype == "fp32" else torch.float64
    rp = _dev(row_ptr, torch.int32, device)
    ci = _dev(col, torch.int32, device)
    v = _dev(val, vdt, device)
    bb = _dev(b, vdt, device)
    n = rp.numel() - 1
    x = torch.zeros(n, dtype=vdt, device=device) if x0 is None else _dev(x0, vdt, device).clone()
    if "stream" not in kw:
        kw["stream"] = ctypes.c_void_p(torch.cuda.current_stream(x.device).cuda_stream)
    o = _opts(dtype, **kw)
    if checkpoint is not None:
        wdt = torch.float64 if dtype == "fp64" else torch.float32  # the iteration's working type
        o.checkpoint = checkpoint._bind(n, wdt, x.device, mixed=dtype == "mixed")
    res = N.CgResult()
    rc = N.lib().perks_cg_csr(n, ci.numel(), rp.data_ptr(), ci.data_ptr(), v.data_ptr(), bb.data_ptr(),
                              x.data_ptr(), ctypes.byref(o), ctypes.byref(res))
    if check:
        N.check(rc)
    out = _result(res)
    out["status"] = rc
    return x, out


def cg_dia(offsets, data, b, x0=None, *, dtype="fp64", device="cuda", check=True, checkpoint=None, **kw):
    """Solve with DIA A (offsets[ndiag], data[ndiag][n], diagonal-major)."""
    import torch
    vdt = torch.float32 if dtype == "fp32" else torch.float64
    off = np.ascontiguousarray(offsets, dtype=np.int32)
    d = _dev(data, vdt, device)
    bb = _dev(b, vdt, device)
    n = d.shape[1]
    x = torch.zeros(n, dtype=vdt, device=device) if x0 is None else _dev(x0, vdt, device).clone()
    if "stream" not in kw:
        kw["stream"] = ctypes.c_void_p(torch.cuda.current_stream(x.device).cuda_stream)
    o = _opts(dtype, **kw)
    if checkpoint is not None:
        wdt = torch.float64 if dtype == "fp64" else torch.float32  # the iteration's working type
        o.checkpoint = checkpoint._bind(n, wdt, x.device, mixed=dtype == "mixed")
    res = N.CgResult()
    rc = N.lib().perks_cg_dia(n, len(off), off.ctypes.data, d.data_ptr(), bb.data_ptr(), x.data_ptr(),
                              ctypes.byref(o), ctypes.byref(res))
    if check:
        N.check(rc)
    out = _result(res)
    out["status"] = rc
    return x, out


def spmv_csr(row_ptr, col, val, x, device="cuda"):
    import torch
    vdt = torch.float32 if np.dtype(getattr(val, "dtype", np.float64)) == np.float32 else torch.float64
    rp, ci = _dev(row_ptr, torch.int32, device), _dev(col, torch.int32, device)
    v, xx = _dev(val, vdt, device), _dev(x, vdt, device)
    y = torch.empty(rp.numel() - 1, dtype=vdt, device=device)
    dt = N.FP32 if vdt == torch.float32 else N.FP64
    N.check(N.lib().perks_spmv_csr(dt, y.numel(), ci.numel(), rp.data_ptr(), ci.data_ptr(), v.data_ptr(),
                                   xx.data_ptr(), y.data_ptr(), None))
    return y


def spmv_dia(offsets, data, x, device="cuda"):
    import torch
    vdt = torch.float32 if np.dtype(getattr(data, "dtype", np.float64)) == np.float32 else torch.float64
    off = np.ascontiguousarray(offsets, dtype=np.int32)
    d, xx = _dev(data, vdt, device), _dev(x, vdt, device)
    y = torch.empty(d.shape[1], dtype=vdt, device=device)
    dt = N.FP32 if vdt == torch.float32 else N.FP64
    N.check(N.lib().perks_spmv_dia(dt, y.numel(), len(off), off.ctypes.data, d.data_ptr(), xx.data_ptr(),
                                   y.data_ptr(), None))
    return y
