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


def test_noalloc_fill_allocates_nothing(gpu):
    """Free device memory is unchanged across calls (after the first, which
    loads the kernels), and in a fresh process whose library workspace
    refuses every allocation (TT_CUDA_FAIL_ALLOC) the allocating fill fails
    while this one succeeds and matches the oracle."""
    torch = gpu
    import os
    import subprocess
    import sys
    from pathlib import Path

    from libtopotoolbox_gb300 import _native, dems

    lib = _native.lib()
    dv = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dv).cuda_stream
    dem, bc, _ = dems.plain_4096(seed=13, size=640)
    m, n = dem.shape
    t_dem = torch.from_numpy(np.ascontiguousarray(dem.T)).to(dv)
    t_bc = torch.from_numpy(np.ascontiguousarray(bc.T)).to(dv)
    out = torch.empty_like(t_dem)
    assert _call(lib, "tt_cuda_fillsinks_noalloc_dev", out, t_dem, t_bc, (m, n), stream) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(dv)
    for _ in range(2):
        assert _call(lib, "tt_cuda_fillsinks_noalloc_dev", out, t_dem, t_bc, (m, n), stream) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(dv)
    assert free1 == free0, (free0, free1)

    root = Path(__file__).resolve().parent.parent
    script = f"""
import sys
sys.path.insert(0, {str(root)!r}); sys.path.insert(0, {str(root / 'oracle')!r})
import ctypes as C, numpy as np, torch, pyoracle
from libtopotoolbox_gb300 import _native, dems
lib = _native.lib()
dem, bc, _ = dems.plain_4096(seed=14, size=320)
m, n = dem.shape
t = lambda a: torch.from_numpy(np.ascontiguousarray(a.T)).cuda()
d_dem, d_bc = t(dem), t(bc)
out = torch.empty_like(d_dem)
dp, keep = _native.dims_arg((m, n))
P = lambda x: C.c_void_p(x.data_ptr())
st = torch.cuda.current_stream().cuda_stream
assert lib.tt_cuda_fillsinks_dev(P(out), P(d_dem), P(d_bc), dp, C.c_void_p(st)) == 2
assert lib.tt_cuda_fillsinks_noalloc_dev(P(out), P(d_dem), P(d_bc), dp, C.c_void_p(st)) == 0
torch.cuda.synchronize()
a = out.cpu().numpy().T
r = pyoracle.Oracle("port").fillsinks(dem, bc)
assert np.all((a == r) | (np.isnan(a) & np.isnan(r)))
print("ok")
"""
    env = dict(os.environ, TT_CUDA_FAIL_ALLOC="1")
    res = subprocess.run([sys.executable, "-c", script], env=env, capture_output=True, text=True,
                         timeout=600)
    assert res.returncode == 0 and "ok" in res.stdout, res.stdout + res.stderr


def test_noalloc_fill_beside_other_work(gpu):
    """A long run of other kernels on another stream does not starve the
    fill's persistent kernel (a cooperative launch): the call converges and
    its result is exact."""
    torch = gpu
    from libtopotoolbox_gb300 import _native, dems

    lib = _native.lib()
    dv = torch.device("cuda", 0)
    dem, bc, _ = dems.plain_512(seed=15, size=512)
    m, n = dem.shape
    t_dem = torch.from_numpy(np.ascontiguousarray(dem.T)).to(dv)
    t_bc = torch.from_numpy(np.ascontiguousarray(bc.T)).to(dv)
    ref = torch.empty_like(t_dem)
    assert _call(lib, "tt_cuda_fillsinks_dev", ref, t_dem, t_bc, (m, n),
                 torch.cuda.current_stream(dv).cuda_stream) == 0
    busy = torch.cuda.Stream(dv)
    mine = torch.cuda.Stream(dv)
    a = torch.randn(4096, 4096, device=dv)
    torch.cuda.synchronize()
    with torch.cuda.stream(busy):
        for _ in range(40):
            a = torch.tanh(a @ a * 1e-3)
    got = torch.empty_like(t_dem)
    with torch.cuda.stream(mine):
        st = _call(lib, "tt_cuda_fillsinks_noalloc_dev", got, t_dem, t_bc, (m, n),
                   mine.cuda_stream)
    torch.cuda.synchronize()
    assert st == 0
    g, r = got.cpu().numpy(), ref.cpu().numpy()
    assert np.all((g == r) | (np.isnan(g) & np.isnan(r)))
