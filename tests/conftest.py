import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def port():
    import pyoracle

    return pyoracle.Oracle("port")


@pytest.fixture(scope="session")
def ref():
    import pyoracle

    if not pyoracle.REF_LIB.exists():
        if pyoracle.build_ref() is None:
            pytest.skip("reference sources not available on this host")
    return pyoracle.Oracle("ref")


@pytest.fixture(scope="session")
def gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from libtopotoolbox_gb300 import _native

    _native.lib()
    return torch


def same_float(a, b):
    """Bit-exact float equality with NaN == NaN and +0 == -0."""
    a = np.asarray(a)
    b = np.asarray(b)
    return a.shape == b.shape and bool(np.all((a == b) | (np.isnan(a) & np.isnan(b))))


def topo_positions_ok(node, direction, order=0):
    """Every donor precedes its receiver in `node` (test/d8.c:36-79 style)."""
    node = np.asarray(node).ravel(order="F")
    d = np.asarray(direction).ravel(order="F").astype(np.int64)
    m = direction.shape[0]
    N = node.size
    if not np.array_equal(np.sort(node), np.arange(N)):
        return False
    pos = np.empty(N, dtype=np.int64)
    pos[node] = np.arange(N)
    src = np.nonzero(d)[0]
    k = np.floor(np.log2(d[src])).astype(np.int64)
    a = np.array([0, 1, 1, 1, 0, -1, -1, -1])
    b = np.array([1, 1, 0, -1, -1, -1, 0, 1])
    di, dj = (a, b) if order == 0 else (b, a)
    tgt = (src // m + dj[k]) * m + (src % m + di[k])
    return bool(np.all(pos[src] < pos[tgt]))


@pytest.fixture
def seeded():
    return np.random.default_rng(12345)


def reconstruct_cases():
    """(name, marker, mask) pairs for grayscale reconstruction
    (src/reconstruct.c:270-312): markers below the mask by random amounts
    with seed pixels at the mask, NaN holes in the mask, fill-like markers
    (-INF but for a few seeds), a marker above the mask in places (both the
    reference and the GPU path clamp it to the mask first), plateaus and
    ragged shapes."""
    from libtopotoolbox_gb300 import dems

    out = []
    rng = np.random.default_rng(2024)
    for s, shp in enumerate([(100, 200), (37, 53), (65, 31), (3, 3), (5, 2), (1, 1), (256, 96)]):
        mask = dems.pcg4d_dem(shp, 40 + s)
        marker = mask - rng.uniform(0, 30, shp).astype(np.float32)
        seeds = rng.random(shp) < 0.01
        marker[seeds] = mask[seeds]
        out.append((f"hmax_{shp[0]}x{shp[1]}", np.asfortranarray(marker), mask))
    d, _, _ = dems.plain_4096(seed=9, size=256)
    mk = np.asfortranarray(d - np.float32(3))
    out.append(("rounded_plateaus_256", mk, d))
    holes = np.array(d, order="F", copy=True)
    holes[rng.random(d.shape) < 0.03] = np.nan
    out.append(("nan_mask_256", np.asfortranarray(d - rng.uniform(0, 10, d.shape).astype(np.float32)),
                holes))
    z = dems.pcg4d_dem((128, 160), 77)
    fl = np.full(z.shape, -np.inf, dtype=np.float32, order="F")
    pick = rng.random(z.shape) < 0.002
    fl[pick] = z[pick]
    out.append(("seeded_ninf_128x160", fl, z))
    hi = np.array(z - 2, order="F", copy=True)
    hi[rng.random(z.shape) < 0.02] += 50  # above the mask in places
    out.append(("marker_above_mask", hi, z))
    d, bc, _ = dems.plain_16384(seed=5, size=640)
    nanm = np.asfortranarray(d)
    out.append(("nodata_640", np.asfortranarray(np.where(np.isnan(d), 0, d) - np.float32(20)), nanm))
    return out
