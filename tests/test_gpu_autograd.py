"""Adjoints through torch.autograd against an FP64 adjoint and central finite
differences (h = 1e-3), on the differentiation workload's distributions
(fractal Hurst 0.7, 800 m relief; lognormal(0, 0.5) runoff weights; loss =
sum of squared (acc - target) at 64 seeded outlets with targets U[0.5, 1.5] x
forward; hillshade upstream gradient U[-1, 1]) at a reduced size.

Tolerance: 1e-5 relative, normwise ||g - g_ref|| / ||g_ref|| and pointwise
max |g - g_ref| / max|g_ref|."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL = 1e-5


def _workload(size=384, seed=5):
    from libtopotoolbox_gb300 import dems

    dem, bc, w, cs = dems.grad_8192(seed=seed, size=size)
    return dem, bc, w, cs


def _col(t_np, torch, dev):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(t_np).T)).to(dev)


def test_flow_accumulation_adjoint(gpu, port):
    torch = gpu
    from libtopotoolbox_gb300 import api, autograd

    dem, bc, w, cs = _workload()
    r = port.pipeline(dem, bc)
    direction, node = r["direction"], r["node"]
    dv = torch.device("cuda", 0)
    wt = _col(w, torch, dv).requires_grad_(True)
    dt = _col(direction, torch, dv)
    acc = autograd.flow_accumulation(wt, dt)
    acc64 = port.flow_accumulation_f64(node, direction, w)
    assert np.max(np.abs(acc.detach().cpu().numpy().T - acc64) / np.abs(acc64)) <= REL

    rng = np.random.default_rng(64)
    outl = np.nonzero((direction.ravel(order="F") == 0) &
                      (acc64.ravel(order="F") > np.median(acc64)))[0]
    sel = rng.choice(outl, size=min(64, outl.size), replace=False)
    target = acc64.ravel(order="F")[sel] * rng.uniform(0.5, 1.5, size=sel.size)
    idx = torch.from_numpy(sel).to(dv)
    tgt = torch.from_numpy(target.astype(np.float32)).to(dv)
    # column-major flat index p = j*m + i  ==  row-major index of the (n, m) tensor
    loss = ((acc.reshape(-1)[idx] - tgt) ** 2).sum()
    loss.backward()
    g = wt.grad.cpu().numpy().T

    # FP64 adjoint
    gacc = np.zeros(dem.size)
    a_sel = acc64.ravel(order="F")[sel]
    gacc[sel] = 2.0 * (a_sel - target)
    gacc = gacc.reshape(dem.shape, order="F")
    g64 = port.flow_accumulation_backward_f64(node, direction, gacc)
    scale = np.max(np.abs(g64))
    assert np.linalg.norm(g - g64) / np.linalg.norm(g64) <= REL
    assert np.max(np.abs(g - g64)) / scale <= REL

    # central finite differences in FP64 on sampled weights
    def L(wv):
        a = port.flow_accumulation_f64w(node, direction, wv).ravel(order="F")
        return float(np.sum((a[sel] - target) ** 2))

    h = 1e-3
    w64 = w.astype(np.float64)
    cand = np.nonzero(np.abs(g64.ravel(order="F")) > 0)[0]
    picks = rng.choice(cand, size=min(24, cand.size), replace=False)
    for p in picks:
        wp = w64.copy(order="F")
        wm = w64.copy(order="F")
        wp.ravel(order="F")[p] += h
        wm.ravel(order="F")[p] -= h
        fd = (L(wp) - L(wm)) / (2 * h)
        gv = g.ravel(order="F")[p]
        assert abs(gv - fd) <= 1e-5 * max(abs(fd), scale * 1e-3), (p, gv, fd)


def test_hillshade_adjoint(gpu, port):
    torch = gpu
    from libtopotoolbox_gb300 import autograd

    dem, bc, w, cs = _workload(size=256)
    az, alt = 3.9269908, 1.0471976
    dv = torch.device("cuda", 0)
    zt = _col(dem, torch, dv).requires_grad_(True)
    out = autograd.hillshade(zt, az, alt, cs)
    rng = np.random.default_rng(3)
    gbar = rng.uniform(-1, 1, size=dem.shape)
    gb_t = _col(gbar.astype(np.float32), torch, dv)
    (out * gb_t).sum().backward()
    g = zt.grad.cpu().numpy().T
    g64 = port.hillshade_backward_f64(dem, gbar.astype(np.float32), az, alt, cs)
    assert np.linalg.norm(g - g64) / np.linalg.norm(g64) <= REL
    assert np.max(np.abs(g - g64)) / np.max(np.abs(g64)) <= REL

    z64 = dem.astype(np.float64)
    gb32 = gbar.astype(np.float32).astype(np.float64)

    def L(z):
        return float(np.sum(port.hillshade_f64(z, az, alt, cs) * gb32))

    h = 1e-3
    picks = rng.choice(dem.size, size=24, replace=False)
    scale = np.max(np.abs(g64))
    for p in picks:
        zp = z64.copy(order="F")
        zm = z64.copy(order="F")
        zp.ravel(order="F")[p] += h
        zm.ravel(order="F")[p] -= h
        fd = (L(zp) - L(zm)) / (2 * h)
        gv = g.ravel(order="F")[p]
        assert abs(gv - fd) <= 1e-5 * max(abs(fd), scale), (p, gv, fd)
