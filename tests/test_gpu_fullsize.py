"""Full-size workloads.

* 4096 x 4096 (rounded fractal with Gaussian pits, extensive flats): the whole
  pipeline bit-exact against the CPU oracle, output by output.
* 16384 x 16384 (5 % NaN nodata disks, -INF/bc convention, 1000 closed
  depressions): size-independent properties, since the serial oracle would
  take tens of minutes -- fixpoint and idempotence of the fill, Bellman
  optimality of gwdt, bit-exact directions and flats on random crops (they
  depend only on 3 x 3 / 5 x 5 neighbourhoods), a topological node order and
  the accumulation checksum (outlet totals sum to the pixel count).
"""
import numpy as np
import pytest

from conftest import same_float, topo_positions_ok

pytestmark = pytest.mark.gpu


def _dev_pipeline(torch, dem, bc):
    from libtopotoolbox_gb300 import api

    dv = torch.device("cuda", 0)
    d = torch.from_numpy(np.ascontiguousarray(dem.T)).to(dv)
    b = torch.from_numpy(np.ascontiguousarray(bc.T)).to(dv)
    o = api.dev.d8_pipeline(d, b)
    torch.cuda.synchronize()
    return {k: v.cpu().numpy().T for k, v in o.items()}


def test_plain_4096_bit_exact(gpu, port):
    from libtopotoolbox_gb300 import dems

    dem, bc, cs = dems.plain_4096()
    got = _dev_pipeline(gpu, dem, bc)
    exp = port.pipeline(dem, bc, hybrid=True)
    assert same_float(got["filled"], exp["filled"])
    assert np.array_equal(got["flats"], exp["flats"])
    assert same_float(got["dist"], exp["dist"])
    assert np.array_equal(got["direction"], exp["direction"])
    assert topo_positions_ok(got["node"], got["direction"])
    assert np.array_equal(got["acc"], exp["acc"])


NB = [(-1, -1), (-1, 0), (-1, 1), (0, -1), (0, 1), (1, -1), (1, 0), (1, 1)]


def _shift(a, di, dj, fill):
    """b[i, j] = a[i + di, j + dj] (fill outside)."""
    out = np.full_like(a, fill)
    m, n = a.shape
    si = slice(max(0, -di), m - max(0, di))
    sj = slice(max(0, -dj), n - max(0, dj))
    ti = slice(max(0, di), m - max(0, -di))
    tj = slice(max(0, dj), n - max(0, -dj))
    out[si, sj] = a[ti, tj]
    return out


@pytest.mark.timeout(1800)
def test_plain_16384_properties(gpu, port):
    torch = gpu
    from libtopotoolbox_gb300 import api, dems

    raw, bc0, cs = dems.plain_16384()
    dem, bc, nanmask = dems.nan_to_outlets(raw, bc0)
    del raw
    got = _dev_pipeline(torch, dem, bc)
    f = got["filled"]
    m, n = dem.shape

    # fill >= dem, fixed cells unchanged, fixpoint f = max(dem, min 3x3 f)
    assert np.all(f >= dem)
    fixed = bc == 1
    assert same_float(f[fixed], dem[fixed])
    lo = f.copy()
    for di, dj in NB:
        np.fmin(lo, _shift(f, di, dj, np.float32(np.inf)), out=lo)
    fp = np.where(lo > dem, lo, dem)
    assert same_float(np.where(fixed, f, fp), f)
    del lo, fp
    # idempotence
    dv = torch.device("cuda", 0)
    ft = torch.from_numpy(np.ascontiguousarray(f.T)).to(dv)
    bt = torch.from_numpy(np.ascontiguousarray(bc.T)).to(dv)
    f2 = api.dev.fillsinks(ft, bt).cpu().numpy().T
    assert same_float(f2, f)
    del ft, bt, f2

    # flats and directions bit-exact on random crops (interior margin 3)
    rng = np.random.default_rng(0)
    for _ in range(6):
        i0, j0 = rng.integers(0, m - 600), rng.integers(0, n - 600)
        sl = (slice(i0, i0 + 600), slice(j0, j0 + 600))
        cf, _ = port.identifyflats(f[sl])
        assert np.array_equal(cf[3:-3, 3:-3], got["flats"][sl][3:-3, 3:-3])
        _, cd = port.flow_routing_d8_carve(f[sl], got["dist"][sl], got["flats"][sl], 0)
        assert np.array_equal(cd[3:-3, 3:-3], got["direction"][sl][3:-3, 3:-3])

    # gwdt: sources at 1, every other reached flat achieves its distance
    # through some flat neighbour, and no flat neighbour improves it.
    fl = (got["flats"] & 1) > 0
    pre = (got["flats"] & 4) > 0
    d = got["dist"]
    assert np.all(d[pre] == 1.0)
    assert np.all(d[~fl] == 0.0)
    costs = port.gwdt_computecosts(got["flats"], dem, f)[0]
    best = np.full(d.shape, np.inf, np.float32)
    for di, dj in NB:
        ch = np.float32(1.41421356237309504880) if di and dj else np.float32(1.0)
        dn = _shift(d, di, dj, np.float32(np.inf))
        cn = _shift(costs, di, dj, np.float32(0))
        fn = _shift(fl, di, dj, False)
        prop = dn + (ch * (costs + cn)) / np.float32(2)
        prop = np.where(fn & fl, prop, np.float32(np.inf)).astype(np.float32)
        np.fmin(best, prop, out=best)
    reach = fl & ~pre & np.isfinite(d)
    assert np.array_equal(best[reach], d[reach])
    assert np.all(best[fl & ~pre] >= d[fl & ~pre])
    del best, costs

    # node order and accumulation checksum
    assert topo_positions_ok(got["node"], got["direction"])
    out = got["direction"] == 0
    total = float(np.sum(got["acc"][out].astype(np.float64)))
    assert abs(total - m * n) <= 1e-6 * m * n
    assert np.all(got["acc"] >= 1.0)
