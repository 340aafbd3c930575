"""Edge-list forms on the GPU (the callers of the path's outputs).

For the same node order and direction grid, flow_routing_d8_edgelist is
bit-identical to the oracle (src/flow_routing.c:258-312); drainagebasins on
the same edge list is bit-identical to the oracle's reverse sweep
(src/drainagebasins.c:6-27); edgelist_degree equals the oracle's counters
(src/streamquad.c:209-224); flow_accumulation_edgelist of a D8 forest with
unit fractions is within 1e-5 of the FP64 sweep and equal, bit for bit, to
flow_accumulation of the same forest; any other edge list (fractions,
several targets, any order) is within 1e-5 of the FP64 list-order sweep, as
is traverse_down_f32_add_mul; the or/and sweeps (traverse_down_u32_or_and,
traverse_up_u32_or_and) are bit-identical to the oracle, and the upward one
labels the same drainage basins.  Both memory orders.
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


def test_edge_list_errors(gpu):
    """Indices outside the grid are refused with TT_CUDA_ERR_INVALID_ARGUMENT
    (1); a cycle in drainagebasins' parents with TT_CUDA_ERR_CYCLE (5)."""
    from libtopotoolbox_gb300 import _native, api

    shape = (8, 8)
    for s, t in [([0, 1], [1, 64]), ([-1, 1], [1, 2])]:
        with pytest.raises(_native.TTCudaError) as e:
            api.flow_accumulation_edgelist(np.array(s), np.array(t), np.ones(2, np.float32), shape)
        assert e.value.status == 1
    with pytest.raises(_native.TTCudaError) as e:  # a two-cycle
        api.drainagebasins(np.array([0, 1]), np.array([1, 0]), shape)
    assert e.value.status == 5


def test_accumulation_edgelist_general(gpu, port):
    """Fractional, multi-target, shuffled and degenerate edge lists through
    the list-order sweep (src/flow_accumulation.c:10-30,
    src/streamquad.c:171-180): within 1e-5 relative of the FP64 sweep in the
    same list order (|a - b| / |b| per cell, all values positive) and
    identical from run to run; the oracle is pinned to the reference on
    these lists (tests/test_oracle_pins.py)."""
    from conftest import edge_list_cases

    from libtopotoolbox_gb300 import api

    rng = np.random.default_rng(5)
    for name, s, t, f, shape in edge_list_cases(port):
        w = np.asfortranarray(rng.uniform(0.5, 2.0, shape).astype(np.float32))
        for weights in (None, w):
            got = api.flow_accumulation_edgelist(s, t, f, shape, weights)
            exp = port.flow_accumulation_edgelist(s, t, f, shape, weights, f64=True)
            assert rel_err(got, exp, tau=1e-30) <= REL_TOL, name
            again = api.flow_accumulation_edgelist(s, t, f, shape, weights)
            assert np.array_equal(got, again), name
        start = w.ravel(order="F")
        got = api.traverse_down_f32_add_mul(start, f, s, t)
        exp = port.traverse_down_f32_add_mul(start, f, s, t, f64=True)
        n = int(max(s.max(initial=-1), t.max(initial=-1))) + 1
        assert rel_err(got[:n], exp[:n], tau=1e-30) <= REL_TOL, name
        assert np.array_equal(got[n:], start[n:]), name  # nodes no edge names


def test_or_and_sweeps(gpu, port):
    """traverse_down_u32_or_and and traverse_up_u32_or_and
    (src/streamquad.c:37-60) equal the oracle bit for bit on every list
    (fractional and multi-target topologies, shuffled, repeated edges and
    self-loops, a wide fan, empty)."""
    from conftest import edge_list_cases

    from libtopotoolbox_gb300 import api

    rng = np.random.default_rng(6)
    for name, s, t, _, shape in edge_list_cases(port):
        n = int(np.prod(shape))
        start = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
        start[rng.random(n) < 0.5] = 0
        w = rng.integers(0, 2**32, len(s), dtype=np.uint64).astype(np.uint32)
        assert np.array_equal(api.traverse_down_u32_or_and(start, w, s, t),
                              port.traverse_u32_or_and(start, w, s, t)), name
        assert np.array_equal(api.traverse_up_u32_or_and(start, w, s, t),
                              port.traverse_u32_or_and(start, w, s, t, up=True)), name


@pytest.mark.parametrize("idx", range(0, len(CASES), 3))
def test_basins_by_upward_sweep(gpu, port, idx):
    """drainagebasins equals the upward or/and sweep started from each
    outlet's own label with all-ones weights (test/random_dem.cpp:549-580)."""
    from libtopotoolbox_gb300 import api

    name, dem, bc = CASES[idx]
    node, direction = _flow(CASES[idx], 0)
    s, t = api.flow_routing_d8_edgelist(node, direction, 0)
    basins = api.drainagebasins(s, t, dem.shape).ravel(order="F")
    n = basins.size
    indeg = np.bincount(t, minlength=n)
    outdeg = np.bincount(s, minlength=n)
    start = np.zeros(n, np.uint32)
    outlet = (indeg > 0) & (outdeg == 0)
    start[outlet] = basins[outlet].astype(np.uint32)
    got = api.traverse_up_u32_or_and(start, np.full(len(s), 0xFFFFFFFF, np.uint32), s, t)
    assert np.array_equal(got, basins.astype(np.uint32)), name


def test_or_and_dev_mfd_1024(gpu, port):
    """Device forms of the or/and sweeps on a 1024 x 1024 multiple-flow-
    direction edge list (about 3.5 million edges), bit for bit."""
    from conftest import mfd_edges

    from libtopotoolbox_gb300 import dems
    from libtopotoolbox_gb300.api import dev

    torch = gpu
    z = dems.plain_512(seed=7, size=1024)[0]
    s, t, _ = mfd_edges(z)
    rng = np.random.default_rng(8)
    start = rng.integers(0, 2**32, z.size, dtype=np.uint64).astype(np.uint32)
    w = rng.integers(0, 2**32, len(s), dtype=np.uint64).astype(np.uint32)
    t_s, t_t = torch.from_numpy(s).cuda(), torch.from_numpy(t).cuda()
    t_w = torch.from_numpy(w.view(np.int32)).cuda()
    for up in (False, True):
        out = torch.from_numpy(start.view(np.int32).copy()).cuda()
        dev.traverse_u32_or_and(out, t_w, t_s, t_t, up=up)
        got = out.cpu().numpy().view(np.uint32)
        assert np.array_equal(got, port.traverse_u32_or_and(start, w, s, t, up=up)), up


def test_traverse_dev_and_mfd_1024(gpu, port):
    """Device form on a 1024 x 1024 multiple-flow-direction edge list
    (about 3.5 million edges, sources listed from the highest pixel down),
    against the FP64 sweep."""
    from conftest import mfd_edges

    from libtopotoolbox_gb300 import dems
    from libtopotoolbox_gb300.api import dev

    torch = gpu
    z = dems.plain_512(seed=6, size=1024)[0]
    s, t, f = mfd_edges(z)
    start = np.ones(z.size, np.float32)
    out = torch.from_numpy(start.copy()).cuda()
    dev.traverse_down_f32_add_mul(out, torch.from_numpy(f).cuda(), torch.from_numpy(s).cuda(),
                                  torch.from_numpy(t).cuda())
    got = out.cpu().numpy()
    exp = port.traverse_down_f32_add_mul(start, f, s, t, f64=True)
    assert rel_err(got, exp, tau=1e-30) <= REL_TOL


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
