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
