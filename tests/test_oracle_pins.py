"""Pin the CPU oracle (oracle/tt_oracle.c) to the reference.

* Against the reference itself, compiled from its own sources by
  `make -C oracle ref` (skipped where the sources are absent): every output
  of the D8 path is compared bit for bit, including the node order, the
  conncomps labels and the gwdt back-links.
* Against the committed golden fixtures in tests/golden/ (produced by the
  compiled reference with tests/golden/make_golden.py), which travel with the
  repository and pin the oracle on hosts without the reference.
* Against the reference's own property tests (test/random_dem.cpp:37-425),
  restated here on the oracle's outputs.
"""
from pathlib import Path

import numpy as np
import pytest

from conftest import edge_list_cases, reconstruct_cases, same_float, topo_positions_ok

GOLDEN = Path(__file__).resolve().parent / "golden"


def _dems():
    from libtopotoolbox_gb300 import dems

    out = []
    for s in range(12):  # random_dem.cpp style: 100 x 200 pcg4d DEMs
        d = dems.pcg4d_dem((100, 200), s)
        out.append((f"pcg4d_{s}", d, dems.border_bc(d.shape)))
    d, bc, _ = dems.plain_512(size=256)
    out.append(("plain_256", d, bc))
    d, bc, _ = dems.plain_4096(size=256)
    out.append(("rounded_256", d, bc))
    d, bc, _ = dems.plain_16384(size=320)
    d2, bc2, _ = dems.nan_to_outlets(d, bc)
    out.append(("nodata_ninf_320", d2, bc2))
    out.append(("nodata_nan_320", d, bc))
    for shp in [(1, 1), (2, 3), (3, 3), (17, 5)]:
        rng = np.random.default_rng(shp[0] * 7 + shp[1])
        out.append((f"rand_{shp}", np.asfortranarray(rng.uniform(0, 5, shp).astype(np.float32)),
                    dems.border_bc(shp)))
    return out


DEMS = _dems()


@pytest.mark.parametrize("idx", range(len(DEMS)))
@pytest.mark.parametrize("hybrid", [False, True])
def test_port_equals_reference(port, ref, idx, hybrid):
    name, dem, bc = DEMS[idx]
    rp = port.pipeline(dem, bc, hybrid=hybrid)
    rr = ref.pipeline(dem, bc, hybrid=hybrid)
    for k in rp:
        a, b = rp[k], rr[k]
        if a.dtype.kind == "f":
            assert same_float(a, b), (name, k)
        else:
            assert np.array_equal(a, b), (name, k)
    _, pp = port.gwdt(rp["costs"], rp["flats"], want_prev=True)
    _, pr = ref.gwdt(rr["costs"], rr["flats"], want_prev=True)
    assert np.array_equal(pp, pr), name


@pytest.mark.parametrize("idx", range(len(DEMS)))
def test_port_hillshade_equals_reference(port, ref, idx):
    name, dem, bc = DEMS[idx]
    if min(dem.shape) < 3:
        pytest.skip("the reference reads out of bounds below 3 x 3")
    d = np.where(np.isfinite(dem), dem, np.float32(0)).astype(np.float32)
    for az, alt in [(3.9269908, 1.0471976), (0.3, 0.5)]:
        assert same_float(port.hillshade_fused(d, az, alt, 30.0), ref.hillshade_fused(d, az, alt, 30.0))
        for a, b in zip(port.hillshade(d, az, alt, 30.0), ref.hillshade(d, az, alt, 30.0)):
            assert same_float(a, b)


def test_port_order1_equals_reference(port, ref):
    name, dem, bc = DEMS[0]
    rp = port.pipeline(dem, bc)
    for order in (0, 1):
        a = port.flow_routing_d8_carve(rp["filled"], rp["dist"], rp["flats"], order)
        b = ref.flow_routing_d8_carve(rp["filled"], rp["dist"], rp["flats"], order)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_golden_fixtures(port):
    files = sorted(GOLDEN.glob("*.npz"))
    assert files, "golden fixtures missing"
    for f in files:
        z = np.load(f)
        dem, bc = z["dem"], z["bc"]
        r = port.pipeline(dem, bc, hybrid=bool(z["hybrid"]))
        for k in ("filled", "flats", "costs", "conncomps", "dist", "node", "direction", "acc"):
            if r[k].dtype.kind == "f":
                assert same_float(r[k], z[k]), (f.name, k)
            else:
                assert np.array_equal(r[k], z[k]), (f.name, k)
        if "hillshade" in z:
            assert same_float(port.hillshade_fused(np.nan_to_num(dem), float(z["az"]),
                                                   float(z["alt"]), float(z["cs"])), z["hillshade"])


@pytest.mark.parametrize("idx", range(12))
def test_reference_properties(port, idx):
    """The hot-path property tests of test/random_dem.cpp on oracle outputs."""
    name, dem, bc = DEMS[idx]
    r = port.pipeline(dem, bc)
    filled, flats, dist, costs = r["filled"], r["flats"], r["dist"], r["costs"]
    m, n = dem.shape
    assert np.all(filled >= dem)  # :37-42
    inner = filled[1:-1, 1:-1]
    higher = np.zeros(inner.shape, dtype=int)
    for di in (-1, 0, 1):
        for dj in (-1, 0, 1):
            if di or dj:
                higher += filled[1 + di:m - 1 + di, 1 + dj:n - 1 + dj] > inner
    assert not np.any(higher == 8)  # :48-53
    assert np.all(dist >= 0)
    assert np.all(dist[(flats & 4) > 0] == 1.0)  # :266-296
    other = ((flats & 1) > 0) & ((flats & 4) == 0)
    assert np.all(dist[other] > 1.0)
    assert np.all((costs > 0) == ((flats & 1) > 0))  # :203-214
    assert topo_positions_ok(r["node"], r["direction"])
    assert np.all(r["acc"] <= dem.size)  # :417-425


@pytest.mark.parametrize("idx", range(len(DEMS)))
@pytest.mark.parametrize("order", [0, 1])
def test_port_edgelists_equal_reference(port, ref, idx, order):
    """Edge lists, edge-list accumulation, drainage basins and degrees
    (src/flow_routing.c:258-312, src/flow_accumulation.c:10-30,
    src/drainagebasins.c:6-27, src/streamquad.c:209-224)."""
    name, dem, bc = DEMS[idx]
    r = port.pipeline(dem, bc)
    node, direction = port.flow_routing_d8_carve(r["filled"], r["dist"], r["flats"], order)
    sp, tp = port.flow_routing_d8_edgelist(node, direction, order)
    sr, tr = ref.flow_routing_d8_edgelist(node, direction, order)
    assert np.array_equal(sp, sr) and np.array_equal(tp, tr), name
    fr = np.ones(len(sp), np.float32)
    rng = np.random.default_rng(idx)
    w = np.asfortranarray(rng.uniform(0.5, 1.5, dem.shape).astype(np.float32))
    for weights in (None, w):
        a = port.flow_accumulation_edgelist(sp, tp, fr, dem.shape, weights)
        b = ref.flow_accumulation_edgelist(sp, tp, fr, dem.shape, weights)
        assert same_float(a, b), name
    fr2 = rng.uniform(0.0, 1.0, len(sp)).astype(np.float32)
    assert same_float(port.flow_accumulation_edgelist(sp, tp, fr2, dem.shape),
                      ref.flow_accumulation_edgelist(sp, tp, fr2, dem.shape)), name
    assert np.array_equal(port.drainagebasins(sp, tp, dem.shape),
                          ref.drainagebasins(sp, tp, dem.shape)), name
    for a, b in zip(port.edgelist_degree(sp, tp, dem.size), ref.edgelist_degree(sp, tp, dem.size)):
        assert np.array_equal(a, b), name
    # the edge list is the D8 forest in topological order: every source
    # appears once, before any edge whose source is its target
    assert len(np.unique(sp)) == len(sp)
    pos = np.full(dem.size, -1)
    pos[sp] = np.arange(len(sp))
    later = pos[tp]
    assert np.all((later == -1) | (later > np.arange(len(sp))))


def graphflood_cases():
    """Row-major DEMs with graphflood boundary codes: 1 inside, 3 (can leave
    the grid) on the border, 0 (nodata) where the DEM is NaN, a few 4/8/9."""
    out = []
    for name, dem, bc in DEMS:
        topo = np.ascontiguousarray(np.asarray(dem, dtype=np.float64).T)  # rows x cols
        if topo.size < 4:
            continue
        bcs = np.ones(topo.shape, np.uint8)
        bcs[0, :] = bcs[-1, :] = bcs[:, 0] = bcs[:, -1] = 3
        bcs[np.isnan(topo)] = 0
        rng = np.random.default_rng(topo.size)
        pick = rng.random(topo.shape)
        bcs[(pick < 0.01) & (bcs == 1)] = 4
        bcs[(pick > 0.995) & (bcs == 1)] = 8
        bcs[(pick > 0.5) & (pick < 0.505) & (bcs == 1)] = 9
        out.append((name, np.nan_to_num(topo, nan=0.0), bcs))
    return out


GF = graphflood_cases()


@pytest.mark.parametrize("idx", range(len(GF)))
@pytest.mark.parametrize("d8", [True, False])
def test_port_sfgraph_equals_reference(port, ref, idx, d8):
    """compute_sfgraph and the drainage areas (src/graphflood/sfgraph.c:27-113,
    src/graphflood/gf_flowacc.c:19-57)."""
    name, topo, bcs = GF[idx]
    a = port.compute_sfgraph(topo, bcs, 30.0, d8)
    b = ref.compute_sfgraph(topo, bcs, 30.0, d8)
    rcv, dist, don, ndon, stack = a
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), name
    assert np.array_equal(a[3], b[3]) and np.array_equal(a[4], b[4]), name
    for v in range(len(ndon)):
        assert np.array_equal(a[2][v, :ndon[v]], b[2][v, :ndon[v]]), (name, v)
    w = np.random.default_rng(idx).uniform(0.5, 2.0, topo.shape)
    for weights in (None, w):
        assert np.array_equal(port.compute_drainage_area_single_flow(rcv, stack, topo.shape, 30.0,
                                                                     weights),
                              ref.compute_drainage_area_single_flow(rcv, stack, topo.shape, 30.0,
                                                                    weights)), name


RECON = reconstruct_cases()


@pytest.mark.parametrize("idx", range(len(RECON)))
def test_port_reconstruct_equals_reference(port, ref, idx):
    """Grayscale reconstruction with arbitrary markers (src/reconstruct.c:270-312)."""
    name, marker, mask = RECON[idx]
    assert same_float(port.reconstruct(marker, mask), ref.reconstruct(marker, mask)), name
    a, fa = port.reconstruct_hybrid(marker, mask)
    b, fb = ref.reconstruct_hybrid(marker, mask)
    assert same_float(a, b), name
    assert fa == fb == 0, name
    # both forms reach the same fixpoint
    assert same_float(a, port.reconstruct(marker, mask)), name


def test_port_edge_sweeps_equal_reference(port, ref):
    """flow_accumulation_edgelist (src/flow_accumulation.c:10-30) and
    traverse_down_f32_add_mul (src/streamquad.c:171-180) on fractional,
    multi-target, shuffled and degenerate edge lists."""
    rng = np.random.default_rng(3)
    for name, s, t, f, shape in edge_list_cases(port):
        w = rng.uniform(0.5, 2.0, shape).astype(np.float32)
        for weights in (None, w):
            a = port.flow_accumulation_edgelist(s, t, f, shape, weights)
            b = ref.flow_accumulation_edgelist(s, t, f, shape, weights)
            assert same_float(a, b), name
        start = w.ravel(order="F")
        assert same_float(port.traverse_down_f32_add_mul(start, f, s, t),
                          ref.traverse_down_f32_add_mul(start, f, s, t)), name


def test_port_or_and_sweeps_equal_reference(port, ref):
    """traverse_down_u32_or_and and traverse_up_u32_or_and
    (src/streamquad.c:37-60) on the same edge lists, random bit patterns."""
    rng = np.random.default_rng(4)
    for name, s, t, _, shape in edge_list_cases(port):
        n = int(np.prod(shape))
        start = rng.integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)
        start[rng.random(n) < 0.5] = 0
        w = rng.integers(0, 2**32, len(s), dtype=np.uint64).astype(np.uint32)
        for up in (False, True):
            a = port.traverse_u32_or_and(start, w, s, t, up=up)
            b = ref.traverse_u32_or_and(start, w, s, t, up=up)
            assert np.array_equal(a, b), (name, up)
