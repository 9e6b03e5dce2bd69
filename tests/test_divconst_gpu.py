"""The stencil kernels' exact FP32 division by a constant (divconst.cuh),
every one of the 2^32 inputs, against IEEE round-to-nearest division on the
GPU, per element and on packed pairs, all four finish forms (form 2: the
short path wherever its flag test is clear; form 3: the branch-free short
finish). Bit-exact, signs of zero
included; any NaN equals any NaN."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("divisor", [118, 159])
@pytest.mark.parametrize("form", [0, 1, 2, 3])
def test_division_all_inputs(native, cuda, divisor, form):
    L = native.lib()
    bad = (ctypes.c_longlong * 2)()
    first = (ctypes.c_uint * 2)()
    assert L.perks_debug_div_check(divisor, form, bad, first) == 0, native.last_error()
    assert list(bad) == [0, 0], [hex(f) for f in first]
