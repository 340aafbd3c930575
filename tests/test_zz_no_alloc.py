"""tt_cuda_fillsinks_noalloc_dev: the fill for callers that cannot allocate.

Some callers cannot call cudaMalloc while they run (their own memory pool
already owns the device, or they cannot afford the device-wide
synchronisation an allocation can cause).  This entry point keeps its
scratch in a static device array instead.  The test calls it through the C
ABI twice in a row and compares each result with tt_cuda_fillsinks_dev bit
for bit (the fill is exact), and checks that a grid beyond the static
scratch is refused.  It lives in its own file, collected last, and needs no
state from other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(lib, name, out, dem, bc, dims, stream):
    from libtopotoolbox_gb300 import _native

    dp, keep = _native.dims_arg(dims)
    return getattr(lib, name)(C.c_void_p(out.data_ptr()), C.c_void_p(dem.data_ptr()),
                              C.c_void_p(bc.data_ptr()), dp, C.c_void_p(stream))


def test_noalloc_fill_matches_dev_fill(gpu):
    torch = gpu
    from libtopotoolbox_gb300 import _native, dems

    lib = _native.lib()
    dv = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dv).cuda_stream
    cases = []
    d, b, _ = dems.plain_512(seed=11, size=512)
    cases.append((d, b))
    d, b, _ = dems.plain_4096(seed=12, size=300)
    cases.append((d, b))
    for dem, bc in cases:  # two calls in a row on the shared static scratch
        m, n = dem.shape
        t_dem = torch.from_numpy(np.ascontiguousarray(dem.T)).to(dv)
        t_bc = torch.from_numpy(np.ascontiguousarray(bc.T)).to(dv)
        ref = torch.empty_like(t_dem)
        got = torch.full_like(t_dem, float("nan"))
        assert _call(lib, "tt_cuda_fillsinks_dev", ref, t_dem, t_bc, (m, n), stream) == 0
        assert _call(lib, "tt_cuda_fillsinks_noalloc_dev", got, t_dem, t_bc, (m, n), stream) == 0
        torch.cuda.synchronize()
        a, r = got.cpu().numpy(), ref.cpu().numpy()
        assert np.all((a == r) | (np.isnan(a) & np.isnan(r)))


def test_noalloc_fill_rejects_oversized_grid(gpu):
    torch = gpu
    from libtopotoolbox_gb300 import _native

    lib = _native.lib()
    small = torch.zeros((4, 4), dtype=torch.float32, device="cuda")
    small_bc = torch.zeros((4, 4), dtype=torch.uint8, device="cuda")
    # 8192 x 8224 pixels need 256 x 257 tiles, more than the static scratch holds
    st = _call(lib, "tt_cuda_fillsinks_noalloc_dev", small, small, small_bc, (8192, 8224), 0)
    assert st == 1
    assert _native.last_status() == 1
