"""Graphflood's single-flow graph on the GPU against the oracle.

compute_sfgraph (src/graphflood/sfgraph.c:27-113): receivers, distances,
donor counts, the listed donors and the Braun-Willett stack bit-identical,
D8 and D4, on the oracle-pin DEMs with graphflood boundary codes and on the
full 4096 x 4096 workload.  compute_drainage_area_single_flow
(src/graphflood/gf_flowacc.c:19-35): exact for an integer cell size, within
1e-12 relative for a cell size whose area is not a dyadic number.
"""
import numpy as np
import pytest

from test_oracle_pins import GF

pytestmark = pytest.mark.gpu


def _same_graph(a, b, name):
    rcv, dist, don, ndon, stack = a
    assert np.array_equal(rcv, b[0]), name
    assert np.array_equal(dist, b[1]), name
    assert np.array_equal(ndon, b[3]), name
    assert np.array_equal(stack, b[4]), name
    k = don.shape[1]
    mask = np.arange(k)[None, :] < ndon[:, None]
    assert np.array_equal(don[mask], b[2][mask]), name


@pytest.mark.parametrize("idx", range(len(GF)))
@pytest.mark.parametrize("d8", [True, False])
def test_sfgraph_matches_oracle(gpu, port, idx, d8):
    from libtopotoolbox_gb300 import api

    name, topo, bcs = GF[idx]
    got = api.compute_sfgraph(topo, bcs, 30.0, d8)
    _same_graph(got, port.compute_sfgraph(topo, bcs, 30.0, d8), name)
    area = api.compute_drainage_area_single_flow(got[0], topo.shape, 30.0)
    assert np.array_equal(area, port.compute_drainage_area_single_flow(got[0], got[4],
                                                                       topo.shape, 30.0)), name
    a2 = api.compute_drainage_area_single_flow(got[0], topo.shape, 0.1)
    r2 = port.compute_drainage_area_single_flow(got[0], got[4], topo.shape, 0.1)
    assert np.max(np.abs(a2 - r2) / np.maximum(np.abs(r2), 1e-300)) <= 1e-12, name


def test_sfgraph_donor_slots_untouched(gpu):
    """Slots past each donor count keep what the caller passed."""
    import ctypes as C

    from libtopotoolbox_gb300 import _native as N

    name, topo, bcs = GF[0]
    n = topo.size
    don = np.full(n * 8, 0xABCD, np.uint64)
    rcv, stack = np.empty(n, np.uint64), np.empty(n, np.uint64)
    dist, ndon = np.empty(n, np.float64), np.empty(n, np.uint8)
    dim = (C.c_size_t * 2)(*topo.shape)
    N.lib().tt_cuda_compute_sfgraph(topo.ctypes.data, rcv.ctypes.data, dist.ctypes.data,
                                    don.ctypes.data, ndon.ctypes.data, stack.ctypes.data,
                                    bcs.ctypes.data, C.cast(dim, C.c_void_p), 30.0, True)
    assert N.last_status() == 0
    don = don.reshape(n, 8)
    mask = np.arange(8)[None, :] >= ndon[:, None]
    assert np.all(don[mask] == 0xABCD)


def test_sfgraph_full_size(gpu, port):
    from libtopotoolbox_gb300 import api, dems

    dem, bc, cs = dems.plain_4096()
    topo = np.ascontiguousarray(np.asarray(dem, np.float64).T)
    bcs = np.ones(topo.shape, np.uint8)
    bcs[0, :] = bcs[-1, :] = bcs[:, 0] = bcs[:, -1] = 3
    got = api.compute_sfgraph(topo, bcs, float(cs), True)
    _same_graph(got, port.compute_sfgraph(topo, bcs, float(cs), True), "plain_4096")
    area = api.compute_drainage_area_single_flow(got[0], topo.shape, float(cs))
    ref = port.compute_drainage_area_single_flow(got[0], got[4], topo.shape, float(cs))
    assert np.max(np.abs(area - ref) / np.maximum(np.abs(ref), 1e-300)) <= 1e-12
