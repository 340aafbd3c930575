"""Per-cell accuracy of weighted flow accumulation when the weights span many
orders of magnitude (src/flow_accumulation.c:32-80 against an FP64 sum over
the same receivers).

Tolerance, stated per result: every cell whose FP64 total is nonzero is
within 1e-5 relative of it, |a - b| / |b| <= 1e-5; every cell whose FP64
total is zero is exactly zero.  Weights here are of one sign, so no total
cancels.  The sums are also bit-identical from run to run.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5


@pytest.fixture(scope="module")
def forest_8192(gpu):
    """Directions and node order of the 8192 x 8192 differentiation DEM
    (fractal, Hurst 0.7, 800 m relief), computed on the GPU."""
    torch = gpu
    from libtopotoolbox_gb300 import dems
    from libtopotoolbox_gb300.api import dev

    dem, bc, _, _ = dems.grad_8192()
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a.T)).cuda()  # noqa: E731
    d_dem, d_bc = t(dem), t(bc)
    o = dev.d8_pipeline(d_dem, d_bc)
    torch.cuda.synchronize()
    return d_dem, d_bc, o["direction"], o["node"].cpu().numpy().T, o["direction"].cpu().numpy().T


def _weights(kind, shape):
    rng = np.random.default_rng(8192 + len(kind))
    if kind == "decades":  # 10^U(-8, 0): 8 orders of magnitude, 20 % zeros
        w = 10.0 ** rng.uniform(-8.0, 0.0, size=shape)
        w[rng.random(shape) < 0.2] = 0.0
    else:  # headwater: unit weights, 30 % of the cells at 1e-6 and 1 % at 1e-12
        w = np.ones(shape)
        w[rng.random(shape) < 0.3] = 1e-6
        w[rng.random(shape) < 0.01] = 1e-12
    return np.asfortranarray(w.astype(np.float32))


def _check(got, exp):
    zero = exp == 0
    assert np.all(got[zero] == 0), "cells with a zero FP64 total must be exactly zero"
    nz = ~zero
    rel = np.abs(got[nz].astype(np.float64) - exp[nz]) / np.abs(exp[nz])
    worst = float(rel.max(initial=0.0))
    assert worst <= REL_TOL, f"max per-cell relative error {worst:.3e}"
    return worst


@pytest.mark.parametrize("kind", ["decades", "headwater"])
def test_wide_range_weights_8192(gpu, port, forest_8192, kind):
    torch = gpu
    from libtopotoolbox_gb300.api import dev

    d_dem, d_bc, d_dir, node, direction = forest_8192
    w = _weights(kind, direction.shape)
    d_w = torch.from_numpy(np.ascontiguousarray(w.T)).cuda()
    acc = dev.flow_accumulation(d_dir, d_w)
    acc2 = dev.flow_accumulation(d_dir, d_w)
    torch.cuda.synchronize()
    assert torch.equal(acc, acc2), "weighted accumulation is not run-to-run identical"
    got = acc.cpu().numpy().T
    exp = port.flow_accumulation_f64(node, direction, w)
    _check(got, exp)
    # the fused pipeline entry (node order and accumulation from one
    # contraction) gives the same bits
    o = dev.d8_pipeline(d_dem, d_bc, weights=d_w)
    torch.cuda.synchronize()
    assert torch.equal(o["acc"], acc)


def test_wide_range_weights_small(gpu, port):
    """The same rule on small grids with ragged tiles, through the
    host-pointer entry point."""
    from libtopotoolbox_gb300 import api, dems

    for shp in [(300, 257), (33, 1000), (1, 700)]:
        dem = dems.pcg4d_dem(shp, 5)
        r = port.pipeline(dem, dems.border_bc(shp))
        w = _weights("decades", shp)
        got = api.flow_accumulation(r["direction"], w)
        exp = port.flow_accumulation_f64(r["node"], r["direction"], w)
        _check(got, exp)
