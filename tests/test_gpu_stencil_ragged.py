"""GPU parity of the flat labelling and directions stencils on ragged grids.

Both must equal the oracle bit for bit (src/identifyflats.c:33-121,
src/flow_routing.c:15-76) on shapes that cut the 32 x 32 tiles at every
edge, with NaN and -INF cells, and on integer DEMs dense in equal
neighbours (sills and presills everywhere).
"""
import numpy as np
import pytest

from libtopotoolbox_gb300 import dems

pytestmark = pytest.mark.gpu

SHAPES = [(4, 70), (8, 8), (4, 4), (36, 260), (132, 97), (260, 300), (1028, 1060), (64, 33),
          (97, 131), (33, 2)]


def _dem(shape, seed):
    rng = np.random.default_rng(seed)
    z = np.round(rng.uniform(0, 4, size=shape)).astype(np.float32)
    z = np.asfortranarray(z)
    k = max(1, z.size // 50)
    z.flat[rng.choice(z.size, k, replace=False)] = np.nan
    z.flat[rng.choice(z.size, k, replace=False)] = -np.inf
    return z


@pytest.mark.parametrize("shape", SHAPES)
def test_identifyflats_ragged(gpu, port, shape):
    from libtopotoolbox_gb300 import api

    for seed in range(2):
        z = _dem(shape, seed)
        ef, en = port.identifyflats(z)
        gf, gn = api.identifyflats(z)
        assert np.array_equal(gf, ef), (shape, seed)
        assert gn == en


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("order", [0, 1])
def test_directions_ragged(gpu, port, shape, order):
    from libtopotoolbox_gb300 import api

    rng = np.random.default_rng(7)
    z = np.asfortranarray(np.round(rng.uniform(0, 6, size=shape)).astype(np.float32))
    z.flat[rng.choice(z.size, max(1, z.size // 40), replace=False)] = np.nan
    d, bc, _ = dems.nan_to_outlets(z, dems.border_bc(shape))
    filled = port.fillsinks(d, bc)
    flats, _ = port.identifyflats(filled)
    costs, _ = port.gwdt_computecosts(flats, d, filled)
    dist = port.gwdt(costs, flats, want_prev=False)
    _, ed = port.flow_routing_d8_carve(filled, dist, flats, order)
    _, gd = api.flow_routing_d8_carve(filled, dist, flats, order)
    assert np.array_equal(gd, ed), (shape, order)
