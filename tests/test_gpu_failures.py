"""Failure detection without faulting the GPU.

Every failure here is made on the host or by input data the kernels check:
an iteration cap that runs out (status, not a hang), a device allocation
refused by the host-side fault switch, and direction grids with cycles or
with receivers off the grid.  Each call must come back with the documented
status and leave the context usable.
"""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from conftest import same_float

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def _status():
    from libtopotoolbox_gb300 import _native

    return _native.last_status()


def test_round_cap_reports_not_converged(gpu, port):
    from libtopotoolbox_gb300 import _native, api, dems

    dem, bc, _ = dems.plain_512(seed=3, size=256)
    lib = _native.lib()
    lib.tt_cuda_set_max_rounds(2)
    try:
        with pytest.raises(_native.TTCudaError) as e:
            api.fillsinks(dem, bc)
        assert e.value.status == 4
    finally:
        lib.tt_cuda_set_max_rounds(0)
    # the context is still usable and the next call is exact
    assert same_float(api.fillsinks(dem, bc), port.fillsinks(dem, bc))


def test_partial_result_is_an_upper_bound(gpu, port):
    """A capped fill returns a valid intermediate state: f >= final fill."""
    import ctypes as C

    from libtopotoolbox_gb300 import _native, dems

    dem, bc, _ = dems.plain_512(seed=4, size=256)
    lib = _native.lib()
    out = np.empty_like(dem, order="F")
    dp, keep = _native.dims_arg(dem.shape)
    lib.tt_cuda_set_max_rounds(3)
    try:
        lib.tt_cuda_fillsinks(C.c_void_p(out.ctypes.data), C.c_void_p(dem.ctypes.data),
                              C.c_void_p(bc.ctypes.data), dp)
        assert _status() == 4
    finally:
        lib.tt_cuda_set_max_rounds(0)
    exact = port.fillsinks(dem, bc)
    assert np.all(out >= exact)


def test_allocation_failure_reports_status(gpu):
    code = (
        "import numpy as np, sys; sys.path.insert(0, %r);"
        "from libtopotoolbox_gb300 import api, _native;"
        "d = np.zeros((64, 64), np.float32, order='F'); b = np.ones((64, 64), np.uint8, order='F');"
        "\ntry:\n api.fillsinks(d, b)\nexcept _native.TTCudaError as e:\n print('STATUS', e.status)"
    ) % str(ROOT)
    env = dict(os.environ, TT_CUDA_FAIL_ALLOC="1")
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                       timeout=300)
    assert "STATUS 2" in r.stdout, r.stdout + r.stderr


def _dir_grid(m, n):
    # every pixel flows to (i+1, j) (bit 2), the last row is an outlet
    d = np.full((m, n), 4, dtype=np.uint8, order="F")
    d[-1, :] = 0
    return d


def test_cycle_inside_a_tile(gpu):
    from libtopotoolbox_gb300 import _native, api

    d = _dir_grid(40, 40)
    d[5, 5] = 4   # (5,5) -> (6,5)
    d[6, 5] = 64  # (6,5) -> (5,5): bit 6 is (i-1, j)
    with pytest.raises(_native.TTCudaError) as e:
        api.flow_accumulation(d)
    assert e.value.status == 5
    with pytest.raises(_native.TTCudaError) as e:
        api.flow_accumulation_backward(d, np.ones(d.shape, np.float32))
    assert e.value.status == 5
    # usable afterwards
    ok = api.flow_accumulation(_dir_grid(40, 40))
    assert ok[-1, 0] == 40


def test_cycle_across_tiles(gpu):
    from libtopotoolbox_gb300 import _native, api

    d = _dir_grid(70, 70)
    d[31, 10] = 4   # (31,10) -> (32,10): crosses the tile edge at i = 32
    d[32, 10] = 64  # (32,10) -> (31,10)
    with pytest.raises(_native.TTCudaError) as e:
        api.flow_accumulation(d)
    assert e.value.status == 5
    with pytest.raises(_native.TTCudaError) as e:
        api.flow_accumulation_backward(d, np.ones(d.shape, np.float32))
    assert e.value.status == 5


def test_direction_off_the_grid(gpu):
    from libtopotoolbox_gb300 import _native, api

    d = _dir_grid(20, 20)
    d[-1, 3] = 4  # last row points below the grid
    with pytest.raises(_native.TTCudaError) as e:
        api.flow_accumulation(d)
    assert e.value.status == 1


def test_invalid_arguments(gpu):
    import ctypes as C

    from libtopotoolbox_gb300 import _native

    lib = _native.lib()
    dp, keep = _native.dims_arg((0, 5))
    lib.tt_cuda_fillsinks(None, None, None, dp)
    assert _status() == 1
    d = np.zeros((4, 4), np.float32, order="F")
    dp, keep = _native.dims_arg((4, 4))
    lib.tt_cuda_flow_routing_d8_carve(C.c_void_p(d.ctypes.data), C.c_void_p(d.ctypes.data),
                                      C.c_void_p(d.ctypes.data), C.c_void_p(d.ctypes.data),
                                      C.c_void_p(d.ctypes.data), dp, 7)
    assert _status() == 1
