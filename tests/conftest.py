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


def mfd_edges(dem, order="topological", seed=0):
    """Multiple-flow-direction edge list of a DEM: every pixel drains to each
    lower neighbour with fraction proportional to the drop over the
    distance (fractions of a pixel sum to 1).  Sources are listed from the
    highest pixel down (a topological order); "shuffled" permutes the list."""
    m, n = dem.shape
    z = np.asarray(dem, np.float64).ravel(order="F")
    src, tgt, w = [], [], []
    ii, jj = np.meshgrid(np.arange(m), np.arange(n), indexing="ij")
    ii, jj = ii.ravel(order="F"), jj.ravel(order="F")
    for di in (-1, 0, 1):
        for dj in (-1, 0, 1):
            if di == 0 and dj == 0:
                continue
            ok = (ii + di >= 0) & (ii + di < m) & (jj + dj >= 0) & (jj + dj < n)
            p = np.nonzero(ok)[0]
            q = (jj[p] + dj) * m + (ii[p] + di)
            drop = (z[p] - z[q]) / np.hypot(di, dj)
            keep = drop > 0
            src.append(p[keep])
            tgt.append(q[keep])
            w.append(drop[keep])
    src, tgt, w = np.concatenate(src), np.concatenate(tgt), np.concatenate(w)
    tot = np.bincount(src, weights=w, minlength=m * n)
    frac = (w / tot[src]).astype(np.float32)
    key = np.lexsort((tgt, -z[src]))
    src, tgt, frac = src[key], tgt[key], frac[key]
    if order == "shuffled":
        perm = np.random.default_rng(seed).permutation(src.size)
        src, tgt, frac = src[perm], tgt[perm], frac[perm]
    return src.astype(np.int64), tgt.astype(np.int64), frac


def edge_list_cases(port):
    """(name, source, target, fraction, shape) edge lists for
    flow_accumulation_edgelist / traverse_down_f32_add_mul."""
    from libtopotoolbox_gb300 import dems

    out = []
    d = dems.pcg4d_dem((100, 200), 3)
    r = port.pipeline(d, dems.border_bc(d.shape))
    s, t = port.flow_routing_d8_edgelist(r["node"], r["direction"])
    out.append(("d8_unit", s, t, np.ones(len(s), np.float32), d.shape))
    rng = np.random.default_rng(17)
    out.append(("d8_fractions", s, t, rng.uniform(0.2, 1.0, len(s)).astype(np.float32), d.shape))
    perm = rng.permutation(len(s))
    out.append(("d8_unit_shuffled", s[perm], t[perm], np.ones(len(s), np.float32), d.shape))
    for shp, sd in [((64, 48), 1), ((37, 53), 2), ((1, 40), 3)]:
        z = dems.pcg4d_dem(shp, sd)
        a, b, f = mfd_edges(z)
        out.append((f"mfd_{shp[0]}x{shp[1]}", a, b, f, shp))
    z = dems.pcg4d_dem((80, 90), 4)
    a, b, f = mfd_edges(z, "shuffled", seed=5)
    out.append(("mfd_shuffled", a, b, f, z.shape))
    # repeated edges and self-loops among 50 nodes, random order
    a = rng.integers(0, 50, 400)
    b = rng.integers(0, 50, 400)
    b[:20] = a[:20]
    out.append(("random_dups_loops", a.astype(np.int64), b.astype(np.int64),
                rng.uniform(0, 0.5, 400).astype(np.float32), (10, 5)))
    # a fan: one edge into node 1, then 300 edges out of it, then onwards
    # (more ready edges at once than a walker's private stack holds)
    fa = [0] + [1] * 300 + list(range(2, 302))
    fb = [1] + list(range(2, 302)) + [302] * 300
    out.append(("fan_300", np.array(fa, np.int64), np.array(fb, np.int64),
                np.full(len(fa), 0.5, np.float32), (303, 1)))
    out.append(("empty", np.zeros(0, np.int64), np.zeros(0, np.int64),
                np.zeros(0, np.float32), (7, 9)))
    return out
