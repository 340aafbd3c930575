"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Bit-exact: filled DEM, flat/sill/presill flags, costs, gwdt distances,
directions; node must be a topological order; unit accumulation exact;
weighted accumulation, hillshade and the adjoints within the stated
tolerances of the FP64 oracle.
"""
import numpy as np
import pytest

from conftest import same_float, topo_positions_ok

pytestmark = pytest.mark.gpu

HS_AZ, HS_ALT = 3.9269908, 1.0471976  # 315 deg / 60 deg in grid convention
# Relative error with floor: max |a - b| / max(|b|, TAU)
TAU = 1e-2
REL_TOL = 1e-5


def rel_err(a, b, tau=TAU):
    """max |a - b| / max(|b|, tau) over finite b; NaN and +-INF must match."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    assert np.array_equal(np.isnan(a), np.isnan(b)), "NaN pattern differs"
    inf = np.isinf(b)
    assert np.array_equal(a[inf], b[inf]), "infinite values differ"
    ok = np.isfinite(b)
    if not ok.any():
        return 0.0
    return float(np.max(np.abs(a[ok] - b[ok]) / np.maximum(np.abs(b[ok]), tau)))


def norm_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    ok = np.isfinite(b)
    den = np.linalg.norm(b[ok])
    return float(np.linalg.norm(a[ok] - b[ok]) / (den if den > 0 else 1.0))


def _cases():
    from libtopotoolbox_gb300 import dems

    cases = []
    for s in range(4):
        d = dems.pcg4d_dem((100, 200), s)
        cases.append((f"pcg4d_{s}", d, dems.border_bc(d.shape)))
    d, bc, _ = dems.plain_512()
    cases.append(("plain_512", d, bc))
    d, bc, _ = dems.plain_4096(size=512)
    cases.append(("rounded_pits_512", d, bc))
    d, bc, _ = dems.plain_16384(size=640)
    d2, bc2, _ = dems.nan_to_outlets(d, bc)
    cases.append(("nodata_ninf_640", d2, bc2))
    cases.append(("nodata_nan_640", d, bc))
    for shp in [(37, 53), (33, 33), (65, 31), (31, 97), (64, 64), (3, 3), (5, 2), (1, 1)]:
        rng = np.random.default_rng(shp[0] * 1000 + shp[1])
        d = np.asfortranarray(np.round(rng.uniform(0, 20, size=shp)).astype(np.float32))
        cases.append((f"rand_{shp[0]}x{shp[1]}", d, dems.border_bc(shp)))
    z = np.zeros((48, 40), dtype=np.float32, order="F")
    cases.append(("flat_zero", z, dems.border_bc(z.shape)))
    return cases


CASES = None


def cases():
    global CASES
    if CASES is None:
        CASES = _cases()
    return CASES


@pytest.fixture(scope="module", params=range(17))
def case(request):
    cs = cases()
    if request.param >= len(cs):
        pytest.skip("no case")
    return cs[request.param]


def test_fillsinks(gpu, port, case):
    from libtopotoolbox_gb300 import api

    name, dem, bc = case
    exp = port.fillsinks(dem, bc)
    got = api.fillsinks(dem, bc)
    assert same_float(got, exp), name
    # hybrid and reconstruct forms agree
    assert same_float(api.fillsinks_hybrid(dem, bc), exp)


def test_identifyflats(gpu, port, case):
    from libtopotoolbox_gb300 import api

    name, dem, bc = case
    filled = port.fillsinks(dem, bc)
    ef, en = port.identifyflats(filled)
    gf, gn = api.identifyflats(filled)
    assert np.array_equal(gf, ef), name
    assert gn == en


def test_costs(gpu, port, case):
    from libtopotoolbox_gb300 import api

    name, dem, bc = case
    filled = port.fillsinks(dem, bc)
    flats, _ = port.identifyflats(filled)
    ec, ecc = port.gwdt_computecosts(flats, dem, filled)
    gc, gcc = api.gwdt_computecosts(flats, dem, filled)
    assert same_float(gc, ec), name
    isflat = (flats & 1) > 0
    assert np.all(gcc[~isflat] == 0)
    # same partition of the flats into components
    a, b = ecc[isflat], gcc[isflat]
    if a.size:
        pairs = np.unique(np.stack([a, b], 1), axis=0)
        assert len(np.unique(pairs[:, 0])) == len(pairs) == len(np.unique(pairs[:, 1]))
        # the label is a pixel of maximal depth inside the component
        with np.errstate(invalid="ignore"):  # -INF nodata: -INF - -INF is NaN, never flat
            depth = (filled - dem).ravel(order="F")
        lab = gcc.ravel(order="F")
        fl = isflat.ravel(order="F")
        for L in np.unique(lab[fl])[:200]:
            members = np.nonzero(fl & (lab == L))[0]
            assert L in members
            dm = depth[members]
            if np.isnan(dm).all():
                continue  # -INF nodata flats: every depth is NaN
            assert depth[L] == np.nanmax(dm)


def test_gwdt(gpu, port, case):
    from libtopotoolbox_gb300 import api

    name, dem, bc = case
    filled = port.fillsinks(dem, bc)
    flats, _ = port.identifyflats(filled)
    costs, _ = port.gwdt_computecosts(flats, dem, filled)
    ed = port.gwdt(costs, flats, want_prev=False)
    gd, gp = api.gwdt(costs, flats, want_prev=True)
    assert same_float(gd, ed), name
    # prev identity of test/random_dem.cpp:266-296
    m = dem.shape[0]
    d = gd.ravel(order="F")
    c = costs.ravel(order="F")
    f = flats.ravel(order="F")
    pv = gp.ravel(order="F")
    sel = np.nonzero(((f & 1) > 0) & ((f & 4) == 0) & np.isfinite(d))[0]
    par = pv[sel]
    assert np.all(par != sel)
    diag = ((par % m) != (sel % m)) & ((par // m) != (sel // m))
    ch = np.where(diag, np.float32(1.41421356237309504880), np.float32(1.0)).astype(np.float32)
    prop = d[par] + (ch * (c[sel] + c[par])) / np.float32(2)
    assert np.array_equal(prop.astype(np.float32), d[sel])


@pytest.mark.parametrize("order", [0, 1])
def test_carve(gpu, port, case, order):
    from libtopotoolbox_gb300 import api

    name, dem, bc = case
    filled = port.fillsinks(dem, bc)
    flats, _ = port.identifyflats(filled)
    costs, _ = port.gwdt_computecosts(flats, dem, filled)
    dist = port.gwdt(costs, flats, want_prev=False)
    en, ed = port.flow_routing_d8_carve(filled, dist, flats, order)
    gn, gd = api.flow_routing_d8_carve(filled, dist, flats, order)
    assert np.array_equal(gd, ed), name
    assert not np.any(gd == 0xFF)
    assert topo_positions_ok(gn, gd, order), name


def test_accumulation(gpu, port, case):
    from libtopotoolbox_gb300 import api

    name, dem, bc = case
    r = port.pipeline(dem, bc)
    got = api.flow_accumulation(r["direction"])
    assert np.array_equal(got, r["acc"]), name  # exact counts below 2^24
    rng = np.random.default_rng(7)
    w = np.asfortranarray(rng.lognormal(0.0, 0.5, size=dem.shape).astype(np.float32))
    got_w = api.flow_accumulation(r["direction"], w)
    exp64 = port.flow_accumulation_f64(r["node"], r["direction"], w)
    assert rel_err(got_w, exp64, tau=1e-30) <= REL_TOL, name


def test_accumulation_backward(gpu, port, case):
    from libtopotoolbox_gb300 import api

    name, dem, bc = case
    r = port.pipeline(dem, bc)
    rng = np.random.default_rng(11)
    g = np.asfortranarray(rng.uniform(-1, 1, size=dem.shape).astype(np.float32))
    got = api.flow_accumulation_backward(r["direction"], g)
    exp = port.flow_accumulation_backward_f64(r["node"], r["direction"], g)
    assert norm_err(got, exp) <= REL_TOL, name
    scale = max(float(np.max(np.abs(exp))), 1e-30)
    assert float(np.max(np.abs(got - exp))) / scale <= REL_TOL, name


def test_hillshade(gpu, port, case):
    from libtopotoolbox_gb300 import api

    name, dem, bc = case
    if min(dem.shape) < 3:
        pytest.skip("hillshade needs at least 3 x 3")
    got = api.hillshade_fused(dem, HS_AZ, HS_ALT, 30.0)
    exp = port.hillshade_f64(dem, HS_AZ, HS_ALT, 30.0)
    assert rel_err(got, exp) <= REL_TOL, name
    out, dx, dy = api.hillshade(dem, HS_AZ, HS_ALT, 30.0)
    assert rel_err(out, exp) <= REL_TOL
    # Gradients against FP64: normwise 1e-5, and pointwise within 2^-20 of
    # the DEM's magnitude over 2h (the float32 cancellation floor of a
    # difference of two elevations).
    z = np.asarray(dem, np.float64)
    for got_g, axis in ((dx, 0), (dy, 1)):
        exp_g = _gradient_f64(z, 30.0, axis)
        assert norm_err(got_g, exp_g) <= REL_TOL
        fin = np.isfinite(exp_g)
        scale = np.nanmax(np.abs(z[np.isfinite(z)]), initial=1.0) / 60.0
        assert np.max(np.abs(got_g[fin] - exp_g[fin]), initial=0.0) <= 2.0 ** -20 * scale * 8
    # the reference's own float32 output is within its snapshot tolerance
    ref32 = port.hillshade_fused(dem, HS_AZ, HS_ALT, 30.0)
    ok = ~np.isnan(ref32)
    assert np.max(np.abs(got[ok] - ref32[ok]), initial=0.0) <= 1e-4


def _gradient_f64(z, cs, axis):
    """src/hillshade.c:23-76 in float64 along `axis` (0 = first dimension)."""
    z = np.moveaxis(z, axis, 0)
    g = np.empty_like(z)
    with np.errstate(invalid="ignore"):
        g[0] = (-z[2] + 4 * z[1] - 3 * z[0]) / (2 * cs)
        g[-1] = (z[-3] - 4 * z[-2] + 3 * z[-1]) / (2 * cs)
        g[1:-1] = np.where(np.isnan(z[1:-1]), np.nan, (z[2:] - z[:-2]) / (2 * cs))
    return np.moveaxis(g, 0, axis)


def test_hillshade_backward(gpu, port, case):
    from libtopotoolbox_gb300 import api

    name, dem, bc = case
    if min(dem.shape) < 3:
        pytest.skip("hillshade needs at least 3 x 3")
    rng = np.random.default_rng(5)
    g = np.asfortranarray(rng.uniform(-1, 1, size=dem.shape).astype(np.float32))
    got = api.hillshade_backward(dem, g, HS_AZ, HS_ALT, 30.0)
    exp = port.hillshade_backward_f64(dem, g, HS_AZ, HS_ALT, 30.0)
    # NaN and -INF DEMs included: cells whose shade is NaN contribute
    # nothing, so the gradient is finite everywhere (zero where no finite
    # shade depends on the cell).
    assert np.all(np.isfinite(exp)), name
    assert np.all(np.isfinite(got)), name
    assert norm_err(got, exp) <= REL_TOL, name
    scale = max(float(np.max(np.abs(exp))), 1e-30)
    assert float(np.max(np.abs(got - exp))) / scale <= REL_TOL, name


def test_pipeline(gpu, port, case):
    from libtopotoolbox_gb300 import api

    name, dem, bc = case
    r = port.pipeline(dem, bc)
    got = api.d8_pipeline(dem, bc)
    assert same_float(got["filled"], r["filled"]), name
    assert np.array_equal(got["flats"], r["flats"])
    assert same_float(got["dist"], r["dist"])
    assert np.array_equal(got["direction"], r["direction"])
    assert topo_positions_ok(got["node"], got["direction"])
    assert np.array_equal(got["acc"], r["acc"])


@pytest.mark.parametrize("shape", [(300, 700), (257, 65), (1000, 33), (64, 2000), (37, 95)])
def test_pinned_host_paths(gpu, shape):
    """Host-pointer calls on page-locked buffers take the overlapped paths
    (column bands for hillshade, early output copies for the pipeline) and
    give the same bits as the pageable path."""
    import torch

    from libtopotoolbox_gb300 import _native as N
    from libtopotoolbox_gb300 import api, dems

    m, n = shape
    dem = dems.pcg4d_dem(shape, 7)
    bc = dems.border_bc(shape)

    def pinned(dtype):  # column-major (m, n) view of a page-locked buffer
        return torch.empty((n, m), dtype=dtype, pin_memory=True).numpy().T

    h_dem = pinned(torch.float32)
    h_dem[:] = dem
    h_bc = pinned(torch.uint8)
    h_bc[:] = bc
    ptr = lambda a: N.C.c_void_p(a.ctypes.data)  # noqa: E731
    dp, keep = N.dims_arg((m, n))
    lib = N.lib()

    hs = pinned(torch.float32)
    lib.tt_cuda_hillshade_fused(ptr(hs), ptr(h_dem), HS_AZ, HS_ALT, 30.0, dp)
    N.check(N.last_status(), "hillshade_fused")
    assert same_float(hs, api.hillshade_fused(dem, HS_AZ, HS_ALT, 30.0))

    out = {k: pinned(t) for k, t in [("filled", torch.float32), ("flats", torch.int32),
                                      ("dist", torch.float32), ("node", torch.int64),
                                      ("direction", torch.uint8), ("acc", torch.float32)]}
    lib.tt_cuda_d8_pipeline(ptr(out["filled"]), ptr(out["flats"]), ptr(out["dist"]),
                            ptr(out["node"]), ptr(out["direction"]), ptr(out["acc"]),
                            ptr(h_dem), ptr(h_bc), None, dp)
    N.check(N.last_status(), "d8_pipeline")
    ref = api.d8_pipeline(dem, bc)
    for k in ("filled", "dist", "acc"):
        assert same_float(out[k], ref[k]), k
    for k in ("flats", "direction"):
        assert np.array_equal(out[k], ref[k]), k
    assert topo_positions_ok(out["node"], out["direction"])
