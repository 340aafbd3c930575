"""Edge-list forms on the GPU (the callers of the path's outputs).

For the same node order and direction grid, flow_routing_d8_edgelist is
bit-identical to the oracle (src/flow_routing.c:258-312); drainagebasins on
the same edge list is bit-identical to the oracle's reverse sweep
(src/drainagebasins.c:6-27); edgelist_degree equals the oracle's counters
(src/streamquad.c:209-224); flow_accumulation_edgelist of a D8 forest with
unit fractions is within 1e-5 of the FP64 sweep and equal, bit for bit, to
flow_accumulation of the same forest.  Both memory orders.
"""
import numpy as np
import pytest

from test_gpu_parity import _cases, rel_err, REL_TOL

pytestmark = pytest.mark.gpu

CASES = _cases()


def _flow(case, order):
    from libtopotoolbox_gb300 import api

    name, dem, bc = case
    filled = api.fillsinks(dem, bc)
    flats, _ = api.identifyflats(filled)
    costs, _ = api.gwdt_computecosts(flats, dem, filled)
    dist = api.gwdt(costs, flats)
    node, direction = api.flow_routing_d8_carve(filled, dist, flats, order)
    return node, direction


@pytest.mark.parametrize("idx", range(len(CASES)))
@pytest.mark.parametrize("order", [0, 1])
def test_edgelist_basins_degree(gpu, port, idx, order):
    from libtopotoolbox_gb300 import api

    name, dem, bc = CASES[idx]
    node, direction = _flow(CASES[idx], order)
    src, tgt = api.flow_routing_d8_edgelist(node, direction, order)
    osrc, otgt = port.flow_routing_d8_edgelist(node, direction, order)
    assert np.array_equal(src, osrc) and np.array_equal(tgt, otgt), name
    assert np.array_equal(api.drainagebasins(src, tgt, dem.shape),
                          port.drainagebasins(osrc, otgt, dem.shape)), name
    for a, b in zip(api.edgelist_degree(src, tgt, dem.size),
                    port.edgelist_degree(osrc, otgt, dem.size)):
        assert np.array_equal(a, b), name


@pytest.mark.parametrize("idx", range(len(CASES)))
def test_accumulation_edgelist(gpu, port, idx):
    from libtopotoolbox_gb300 import api

    name, dem, bc = CASES[idx]
    node, direction = _flow(CASES[idx], 0)
    src, tgt = api.flow_routing_d8_edgelist(node, direction, 0)
    fr = np.ones(len(src), np.float32)
    rng = np.random.default_rng(idx)
    w = np.asfortranarray(rng.lognormal(0.0, 0.5, dem.shape).astype(np.float32))
    for weights in (None, w):
        got = api.flow_accumulation_edgelist(src, tgt, fr, dem.shape, weights)
        ref64 = port.flow_accumulation_edgelist(src, tgt, fr, dem.shape, weights, f64=True)
        assert rel_err(got, ref64, tau=1.0) <= REL_TOL, name
        assert np.array_equal(got, api.flow_accumulation(direction, weights)), name


def test_device_forms_match_host(gpu, port):
    from libtopotoolbox_gb300 import api
    from libtopotoolbox_gb300.api import dev

    torch = gpu
    name, dem, bc = CASES[5]
    node, direction = _flow(CASES[5], 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(np.asarray(a).T)).cuda()  # noqa: E731
    d_node, d_dir = t(node), t(direction)
    s, g = dev.flow_routing_d8_edgelist(d_node, d_dir)
    hs, hg = api.flow_routing_d8_edgelist(node, direction)
    assert np.array_equal(s.cpu().numpy(), hs) and np.array_equal(g.cpu().numpy(), hg)
    like = torch.empty(d_dir.shape, dtype=torch.float32, device="cuda")
    fr = torch.ones(s.numel(), dtype=torch.float32, device="cuda")
    acc = dev.flow_accumulation_edgelist(s, g, fr, like).cpu().numpy().T
    assert np.array_equal(acc, api.flow_accumulation(direction))
    b = dev.drainagebasins(s, g, like).cpu().numpy().T
    assert np.array_equal(b, port.drainagebasins(hs, hg, dem.shape))


def test_edge_lists_the_forest_cannot_take(gpu):
    """Refused with TT_CUDA_ERR_INVALID_ARGUMENT (1) or TT_CUDA_ERR_CYCLE (5)."""
    from libtopotoolbox_gb300 import _native, api

    shape = (8, 8)
    src = np.array([0, 1], np.int64)
    with pytest.raises(_native.TTCudaError) as e:  # a source listed twice
        api.flow_accumulation_edgelist(np.array([0, 0]), np.array([1, 8]),
                                       np.ones(2, np.float32), shape)
    assert e.value.status == 1
    with pytest.raises(_native.TTCudaError) as e:  # not a neighbour
        api.flow_accumulation_edgelist(src, np.array([5, 30]), np.ones(2, np.float32), shape)
    assert e.value.status == 1
    with pytest.raises(_native.TTCudaError) as e:  # a fraction other than 1
        api.flow_accumulation_edgelist(src, np.array([1, 2]),
                                       np.array([1.0, 0.5], np.float32), shape)
    assert e.value.status == 1
    with pytest.raises(_native.TTCudaError) as e:  # a two-cycle
        api.drainagebasins(np.array([0, 1]), np.array([1, 0]), shape)
    assert e.value.status == 5


def test_edgelist_full_size_properties(gpu):
    """4096 x 4096 workload: one edge per pixel with a direction, sources
    distinct and topologically ordered, basins = the roots with donors."""
    from libtopotoolbox_gb300 import api, dems

    dem, bc, _ = dems.plain_4096()
    res = api.d8_pipeline(dem, bc)
    node, direction = res["node"], res["direction"]
    src, tgt = api.flow_routing_d8_edgelist(node, direction)
    assert len(src) == int(np.count_nonzero(direction))
    pos = np.full(direction.size, -1, np.int64)
    pos[src] = np.arange(len(src))
    assert len(np.unique(src)) == len(src)
    later = pos[tgt]
    assert np.all((later == -1) | (later > np.arange(len(src))))
    basins = api.drainagebasins(src, tgt, dem.shape).ravel(order="F")
    roots_with_donors = np.unique(tgt[pos[tgt] == -1])
    assert basins.max() == len(roots_with_donors)
    assert np.array_equal(np.sort(np.unique(basins[basins > 0])),
                          np.arange(1, len(roots_with_donors) + 1))
    assert np.all(basins[src] == basins[tgt])
