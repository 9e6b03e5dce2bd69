"""perks_stencil2d_noalloc, the entry point for callers that may not allocate
device memory (their device-memory footprint is fixed at start-up, or another
framework's memory manager owns the GPU, so cudaMalloc mid-run is not
allowed): it must give exactly what perks_stencil2d gives, call after call,
from its shared static scratch array.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test. It also passes alone in a
fresh process (the first call resolves the scratch array's address)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(native, fn, field, shape, steps, out=None, **kw):
    import torch
    from perks_gb300 import _native as N
    from perks_gb300.stencil import _opts, _torch_dtype_np
    out = torch.empty_like(field) if out is None else out
    o = _opts(shape, _torch_dtype_np(field), stream=ctypes.c_void_p(torch.cuda.current_stream().cuda_stream),
              **kw)
    st = N.StencilStats()
    rc = getattr(N.lib(), fn)(ctypes.byref(o), field.data_ptr(), out.data_ptr(), field.shape[0], field.shape[1],
                              steps, ctypes.byref(st))
    torch.cuda.synchronize()
    return rc, out


def test_noalloc_matches_allocating_entry_point(native, cuda):
    import torch
    g = torch.Generator(device="cpu").manual_seed(5)
    cases = [("2d5pt", torch.float64, (1024, 1024), 9, {}),
             ("2ds9pt", torch.float32, (700, 1500), 7, {"kernel": "per_step"}),
             ("2d25pt", torch.float64, (333, 901), 5, {"l2_sweep": True})]
    for shape, dt, dims, steps, kw in cases:
        f = torch.rand(dims, generator=g, dtype=dt).to(cuda)
        # two calls in a row: the second must not see the first call's state
        for call in range(2):
            rc_a, a = _call(native, "perks_stencil2d", f, shape, steps, **kw)
            rc_b, b = _call(native, "perks_stencil2d_noalloc", f, shape, steps, **kw)
            assert rc_a == 0 and rc_b == 0, native.last_error()
            assert torch.equal(a.view(torch.uint8), b.view(torch.uint8)), (shape, call)
            f = a  # next call starts from a different field


def test_noalloc_rejects_oversized_field(native, cuda):
    import torch
    f = torch.zeros((4096, 4096), dtype=torch.float64, device=cuda)  # 2 x 128 MiB of scratch needed
    rc, _ = _call(native, "perks_stencil2d_noalloc", f, "2d5pt", 2)
    assert rc == -10
    assert "bytes of scratch" in native.last_error()


def test_noalloc_allocates_nothing(native, cuda):
    """After a first call (which may load the kernel's code), further calls,
    also on a larger field than any before, make no workspace allocation and
    leave the device's free memory where it was."""
    import torch
    L = native.lib()
    g = torch.Generator(device="cpu").manual_seed(8)
    small = torch.rand((200, 900), generator=g, dtype=torch.float32).to(cuda)
    big = torch.rand((1900, 2000), generator=g, dtype=torch.float32).to(cuda)
    out_big = torch.empty_like(big)
    rc, _ = _call(native, "perks_stencil2d_noalloc", small, "2ds9pt", 3)
    assert rc == 0, native.last_error()
    torch.cuda.synchronize()
    allocs0 = L.perks_debug_workspace_allocs()
    free0, _ = torch.cuda.mem_get_info()
    for steps in (5, 6, 1):
        rc, _ = _call(native, "perks_stencil2d_noalloc", big, "2ds9pt", steps, out=out_big)
        assert rc == 0, native.last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert L.perks_debug_workspace_allocs() == allocs0
    # every buffer of the calls exists before free0 is read, so the device's
    # free memory only moves if the entry point allocated something
    assert free1 == free0, (free0, free1)
    rc, ref = _call(native, "perks_stencil2d", big, "2ds9pt", 1)
    assert rc == 0, native.last_error()
    assert torch.equal(ref.view(torch.uint8), out_big.view(torch.uint8))
