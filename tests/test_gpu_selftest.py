"""Device arithmetic the kernels rely on for bit-exact results.

The direction kernels divide diagonal drops by sqrtf(2) with a
three-instruction correctly rounded division (Markstein's correction step
for a constant divisor) instead of the IEEE division of the reference
(src/flow_routing.c:42-43,69).  It must give the same bits as the IEEE
division for every float32 input, which this test checks exhaustively
(2^32 inputs, on the GPU).
"""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu


def test_div_by_sqrt2_matches_ieee_division_everywhere(gpu):
    from libtopotoolbox_gb300 import _native

    bad = C.c_uint64(123)
    first = C.c_uint32(0)
    st = _native.lib().tt_cuda_selftest_div_sqrt2(C.byref(bad), C.byref(first))
    assert st == 0
    assert bad.value == 0, f"{bad.value} inputs differ, first bit pattern {first.value:#010x}"
    assert first.value == 0xFFFFFFFF
