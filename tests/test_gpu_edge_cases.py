"""GPU parity of the whole D8 pipeline on edge-case grids.

Each case goes through `tt_cuda_d8_pipeline` and is compared with the
oracle's call sequence (test/random_dem.cpp:682-724): filled DEM, flat
flags, gwdt distances and directions bit for bit, unit accumulation exact,
node a topological order.
- Thin grids: one or two pixels across, so every tile is cut and most
  pixels lie on the boundary.
- One flat basin drained through a single outlet, whose distances must
  cross ~80 tiles.
- A DEM that is all NaN.
"""
import numpy as np
import pytest

from conftest import same_float, topo_positions_ok
from libtopotoolbox_gb300 import dems

pytestmark = pytest.mark.gpu


def _check(port, dem, bc, name):
    from libtopotoolbox_gb300 import api

    r = port.pipeline(dem, bc)
    got = api.d8_pipeline(dem, bc)
    assert same_float(got["filled"], r["filled"]), name
    assert np.array_equal(got["flats"], r["flats"]), name
    assert same_float(got["dist"], r["dist"]), name
    assert np.array_equal(got["direction"], r["direction"]), name
    assert topo_positions_ok(got["node"], got["direction"]), name
    assert np.array_equal(got["acc"], r["acc"]), name


@pytest.mark.parametrize("shape", [(1, 300), (300, 1), (2, 257), (257, 2), (3, 1000),
                                   (1000, 3)])
def test_thin_grids(gpu, port, shape):
    rng = np.random.default_rng(sum(shape))
    dem = np.asfortranarray(np.round(rng.uniform(0, 5, size=shape)).astype(np.float32))
    _check(port, dem, dems.border_bc(shape), f"thin {shape}")


def test_single_outlet_basin(gpu, port):
    """A 1500 x 1300 flat floor at 0 inside a rim at 10, drained by one rim
    pixel at 0: the floor is one flat whose only presills touch the outlet,
    so gwdt distances grow across the whole basin."""
    m, n = 1500, 1300
    dem = np.zeros((m, n), dtype=np.float32, order="F")
    dem[0, :] = dem[-1, :] = 10
    dem[:, 0] = dem[:, -1] = 10
    dem[0, n // 2] = 0  # the outlet
    _check(port, dem, dems.border_bc((m, n)), "single outlet")


def test_all_nan_dem(gpu, port):
    """Every pixel NaN: every pixel is its own outlet, nothing is flat, no
    direction is set."""
    shape = (40, 70)
    dem = np.full(shape, np.nan, dtype=np.float32, order="F")
    _check(port, dem, dems.border_bc(shape), "all NaN")
