"""The C-ABI library: it loads without a GPU, exports every function that
include/perks.h declares, its struct layouts agree with a C compiler's, and
argument checks fail with status codes (never a crash or exit)."""
import ctypes
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "perks.h")


def declared_functions():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"PERKS_API\s+[\w\s\*]+?\b(perks_\w+)\s*\(", src)))


def test_header_declares_functions():
    names = declared_functions()
    assert "perks_stencil2d" in names and "perks_cg_csr" in names and len(names) >= 15


def test_every_declared_symbol_exported(native):
    L = native.lib()
    out = subprocess.run(["nm", "-D", "--defined-only", native._native.LIB_PATH], capture_output=True, text=True)
    exported = set(re.findall(r"\bT (perks_\w+)", out.stdout))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    for n in declared_functions():
        assert getattr(L, n) is not None
    # the Python binding covers every declared function
    assert set(declared_functions()) == set(native._native.SIGNATURES)


def test_struct_layout_matches_c(native):
    N = native._native
    code = r'''
#include <stdio.h>
#include <stddef.h>
#include "perks.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu\n", sizeof(perks_stencil_opts), sizeof(perks_stencil_stats),
         sizeof(perks_cg_opts), sizeof(perks_cg_result), sizeof(perks_cg_state));
  printf("%zu %zu %zu %zu\n", offsetof(perks_stencil_opts, stream), offsetof(perks_cg_opts, stream),
         offsetof(perks_cg_result, launches), offsetof(perks_cg_state, n));
  return 0;
}'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "p.c")
        open(c, "w").write(code)
        exe = os.path.join(d, "p")
        subprocess.run(["gcc", "-I" + os.path.dirname(HEADER), c, "-o", exe], check=True)
        lines = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    sizes = [int(x) for x in lines[0].split()]
    offs = [int(x) for x in lines[1].split()]
    assert sizes == [ctypes.sizeof(N.StencilOpts), ctypes.sizeof(N.StencilStats), ctypes.sizeof(N.CgOpts),
                     ctypes.sizeof(N.CgResult), ctypes.sizeof(N.CgState)]
    assert offs == [N.StencilOpts.stream.offset, N.CgOpts.stream.offset, N.CgResult.launches.offset,
                    N.CgState.n.offset]


def test_enum_values_match_header(native):
    src = open(HEADER).read()
    N = native._native
    for name, val in N.SHAPES.items():
        key = "PERKS_" + name.upper()
        m = re.search(rf"\b{key}\s*=\s*(\d+)", src)
        assert m and int(m.group(1)) == val, name


def test_status_strings_and_version(native):
    L = native.lib()
    assert L.perks_abi_version() == native._native.ABI_VERSION == 3
    assert L.perks_status_string(0) == b"ok"
    assert L.perks_status_string(-15) == b"device-side wait timed out"


def test_argument_errors_are_status_codes(native):
    L = native.lib()
    N = native._native
    o = N.StencilOpts()
    L.perks_stencil_default_opts(ctypes.byref(o), 0, N.FP64)
    # null pointers and a 3D shape on the 2D entry point: INVALID_ARG, no GPU needed
    assert L.perks_stencil2d(ctypes.byref(o), None, None, 4, 4, 1, None) == -10
    o.shape = 16
    assert L.perks_stencil2d(ctypes.byref(o), 1, 1, 4, 4, 1, None) == -10
    assert b"not a 2D shape" in L.perks_last_error()
    o.shape = 0
    assert L.perks_stencil2d(ctypes.byref(o), 1, 1, 0, 4, 1, None) == -10
    o.order = 7
    assert L.perks_stencil2d(ctypes.byref(o), 1, 1, 4, 4, 1, None) == -10
    assert L.perks_stencil3d(None, 1, 1, 4, 4, 4, 1, None) == -10
    # the copy-engine switch: 0 or 1; the no-allocation entry point runs cp.async only
    L.perks_stencil_default_opts(ctypes.byref(o), 0, N.FP32)
    assert o.tma == 0
    o.tma = 2
    assert L.perks_stencil2d(ctypes.byref(o), 1, 1, 4, 4, 1, None) == -10
    o.tma = 1
    assert L.perks_stencil2d_noalloc(ctypes.byref(o), 1, 1, 4, 4, 1, None) == -11


def test_reference_signature_errors(native):
    a = np.zeros((4, 4), np.float32)
    b = np.zeros_like(a)
    # a 3D shape through the 2D drop-in
    assert native.jacobi_iterative(a, 4, 4, b, shape="3d7pt") == -10
    c = np.zeros((2, 4, 4))
    # reference codes: -2 unsupported widths, -4 height too small
    assert native.j3d_iterative(c, 2, 0, 4, c.copy(), shape="3d7pt") == -2
    assert native.j3d_iterative(c, 0, 4, 4, c.copy(), shape="3d7pt") == -4


def test_no_device_is_reported(native):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    a = np.random.rand(8, 8)
    b = np.zeros_like(a)
    rc = native.jacobi_iterative(a, 8, 8, b, iteration=1)
    assert rc in (-12, -13)
    assert native.last_error()


def test_checkpoint_of_another_solve_rejected_before_launch(native):
    """A checkpoint holds n elements of the writer's working type in d_r and
    d_p: resuming it with another dtype or size is refused by the argument
    checks, before any device access (the pointers here are never used)."""
    L = native.lib()
    N = native._native
    st = N.CgState()
    st.d_r, st.d_p, st.k, st.kernel = 16, 16, 5, N.KERNEL_PERSISTENT
    st.dtype, st.n = N.FP32, 10
    o = N.CgOpts()
    L.perks_cg_default_opts(ctypes.byref(o))
    o.checkpoint = ctypes.pointer(st)
    fake = ctypes.c_void_p(16)
    res = N.CgResult()
    o.dtype = N.FP64  # FP32 state, FP64 solve
    assert L.perks_cg_csr(10, 28, fake, fake, fake, fake, fake, ctypes.byref(o), ctypes.byref(res)) == -10
    assert b"another dtype" in L.perks_last_error()
    o.dtype = N.FP32
    assert L.perks_cg_csr(12, 34, fake, fake, fake, fake, fake, ctypes.byref(o), ctypes.byref(res)) == -10
    assert b"rows" in L.perks_last_error()
    st.kernel = N.KERNEL_PER_STEP  # written by the other kernel kind
    assert L.perks_cg_csr(10, 28, fake, fake, fake, fake, fake, ctypes.byref(o), ctypes.byref(res)) == -10


def test_single_reduction_cg_unsupported_combinations(native):
    """The single-reduction CG is a persistent-kernel FP64/FP32 solver without
    checkpoints: other combinations are refused before any device access."""
    L = native.lib()
    N = native._native
    fake = ctypes.c_void_p(16)
    res = N.CgResult()
    for dtype, kernel in ((N.MIXED, N.KERNEL_PERSISTENT), (N.FP64, N.KERNEL_PER_STEP)):
        o = N.CgOpts()
        L.perks_cg_default_opts(ctypes.byref(o))
        o.algorithm, o.dtype, o.kernel = N.CG_SINGLE_REDUCTION, dtype, kernel
        assert L.perks_cg_csr(10, 28, fake, fake, fake, fake, fake, ctypes.byref(o), ctypes.byref(res)) == -11
    o = N.CgOpts()
    L.perks_cg_default_opts(ctypes.byref(o))
    o.algorithm = 7
    assert L.perks_cg_csr(10, 28, fake, fake, fake, fake, fake, ctypes.byref(o), ctypes.byref(res)) == -10


def test_division_check_rejects_unknown_divisor(native):
    L = native.lib()
    bad = (ctypes.c_longlong * 2)()
    assert L.perks_debug_div_check(7, 0, bad, None) == -10
    assert L.perks_debug_div_check(118, 4, bad, None) == -10
    assert L.perks_debug_div_check(118, 0, None, None) == -10


def test_min_domain_3d_argument_errors(native):
    L = native.lib()
    N = native._native
    o = N.StencilOpts()
    L.perks_stencil_default_opts(ctypes.byref(o), 16, N.FP32)
    h = ctypes.c_int(-1)
    assert L.perks_stencil3d_min_domain(None, 8, 8, ctypes.byref(h)) == -10
    assert L.perks_stencil3d_min_domain(ctypes.byref(o), 0, 8, ctypes.byref(h)) == -10
    o.shape = 0
    assert L.perks_stencil3d_min_domain(ctypes.byref(o), 8, 8, ctypes.byref(h)) == -10
