"""Deferred status of the device-pointer calls (tt_cuda_defer_begin /
tt_cuda_defer_end).

Inside a deferral the calls of the D8 path only enqueue their work: they
must give the same bits as the synchronous calls (each is checked against
the synchronous call on the same inputs, which the parity tests check
against the oracle), return without waiting for the GPU, and report the
iteration cap, a cycle or an invalid direction once, at the end.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _t(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a.T)).cuda()


def _weights(shape, seed):
    # 10^U(-8, 0) with 20 % zeros: the weighted sums need several scales
    rng = np.random.default_rng(seed)
    w = 10.0 ** rng.uniform(-8.0, 0.0, size=shape)
    w[rng.random(shape) < 0.2] = 0.0
    return np.asfortranarray(w.astype(np.float32))


def _stages(torch, dev, d_dem, d_bc, d_w):
    out = {}
    out["filled"] = dev.fillsinks(d_dem, d_bc)
    out["flats"] = dev.identifyflats(out["filled"])
    out["costs"], out["cc"] = dev.gwdt_computecosts(out["flats"], d_dem, out["filled"])
    out["dist"] = dev.gwdt(out["costs"], out["flats"])
    out["node"], out["direction"] = dev.flow_routing_d8_carve(out["filled"], out["dist"],
                                                              out["flats"])
    out["acc"] = dev.flow_accumulation(out["direction"])
    out["acc_w"] = dev.flow_accumulation(out["direction"], d_w)
    out["acc_1"] = dev.flow_accumulation(out["direction"], torch.full_like(d_w, 0.5))
    out["hill"] = dev.hillshade_fused(d_dem, 5.5, 0.7, 1.0)
    o = dev.d8_pipeline(d_dem, d_bc, weights=d_w)
    for k in ("filled", "flats", "dist", "node", "direction", "acc"):
        out["pipe_" + k] = o[k]
    return out


def _topological(node_t, dir_t):
    """node is a permutation of the pixels with every donor before its
    receiver (node orders are not unique, and the counting sort's order
    within one height is not fixed from run to run)."""
    m = node_t.shape[1]
    node = node_t.cpu().numpy().ravel()
    d = dir_t.cpu().numpy().ravel()
    pos = np.empty_like(node)
    pos[node] = np.arange(node.size)
    assert np.array_equal(np.sort(node), np.arange(node.size))
    di = np.array([0, 1, 1, 1, 0, -1, -1, -1])
    dj = np.array([1, 1, 0, -1, -1, -1, 0, 1])
    src = np.nonzero(d)[0]
    k = np.floor(np.log2(d[src])).astype(int)
    tgt = (src // m + dj[k]) * m + (src % m + di[k])
    return bool(np.all(pos[src] < pos[tgt]))


@pytest.mark.parametrize("shape", [(700, 523), (1500, 1500)])
def test_deferred_same_bits(gpu, shape):
    torch = gpu
    from libtopotoolbox_gb300 import dems
    from libtopotoolbox_gb300.api import dev

    dem = dems.pcg4d_dem(shape, 11)
    bc = dems.border_bc(shape)
    d_dem, d_bc = _t(torch, dem), _t(torch, bc)
    d_w = _t(torch, _weights(shape, 3))
    ref = _stages(torch, dev, d_dem, d_bc, d_w)
    torch.cuda.synchronize()
    with dev.deferred():
        got = _stages(torch, dev, d_dem, d_bc, d_w)
    for k, v in ref.items():
        if k.endswith("node"):
            assert _topological(v, ref[k.replace("node", "direction")]), k
            assert _topological(got[k], got[k.replace("node", "direction")]), k
            continue
        assert torch.equal(torch.nan_to_num(got[k], 7.0) if v.is_floating_point() else got[k],
                           torch.nan_to_num(v, 7.0) if v.is_floating_point() else v), k


def test_deferred_calls_do_not_wait(gpu):
    """With the stream held busy by a spin of about 0.2 s queued first, the
    deferred calls return and the work after them is still pending: no call
    synchronised the stream."""
    torch = gpu
    import time

    from libtopotoolbox_gb300 import dems
    from libtopotoolbox_gb300.api import dev

    shape = (1024, 1024)
    dem = dems.pcg4d_dem(shape, 12)
    d_dem, d_bc = _t(torch, dem), _t(torch, dems.border_bc(shape))
    d_w = _t(torch, _weights(shape, 4))
    dev.d8_pipeline(d_dem, d_bc, weights=d_w)  # sizes the workspaces outside the check
    done = torch.cuda.Event()
    with dev.deferred():
        dev.d8_pipeline(d_dem, d_bc, weights=d_w)  # and the deferral's own
    torch.cuda.synchronize()
    with dev.deferred():
        torch.cuda._sleep(400_000_000)
        t0 = time.perf_counter()
        dev.d8_pipeline(d_dem, d_bc, weights=d_w)
        enq = time.perf_counter() - t0
        done.record()
        pending = not done.query()
    assert pending, "a deferred call waited for the stream"
    assert enq < 0.15, f"enqueueing took {enq:.3f} s"


def test_deferred_not_converged_reported_at_end(gpu):
    torch = gpu
    from libtopotoolbox_gb300 import _native, dems
    from libtopotoolbox_gb300.api import dev

    dem, bc, _ = dems.plain_512(seed=3, size=256)
    d_dem, d_bc = _t(torch, dem), _t(torch, bc)
    lib = _native.lib()
    exact = dev.fillsinks(d_dem, d_bc)
    lib.tt_cuda_set_max_rounds(2)
    try:
        with pytest.raises(_native.TTCudaError) as e:
            with dev.deferred():
                out = dev.fillsinks(d_dem, d_bc)  # returns success: nothing was read back
                assert _native.last_status() == 0
        assert e.value.status == 4
    finally:
        lib.tt_cuda_set_max_rounds(0)
    torch.cuda.synchronize()
    assert bool((torch.nan_to_num(out, 0.0) >= torch.nan_to_num(exact, 0.0)).all())
    # usable afterwards, and exact again
    with dev.deferred():
        again = dev.fillsinks(d_dem, d_bc)
    assert torch.equal(torch.nan_to_num(again, 7.0), torch.nan_to_num(exact, 7.0))


@pytest.mark.parametrize("weighted", [False, True])
def test_deferred_cycle_reported_at_end(gpu, weighted):
    torch = gpu
    from libtopotoolbox_gb300 import _native
    from libtopotoolbox_gb300.api import dev

    d = np.full((70, 70), 4, dtype=np.uint8, order="F")  # every pixel flows to (i+1, j)
    d[-1, :] = 0
    d[31, 10] = 4   # (31,10) -> (32,10): across the tile edge at i = 32
    d[32, 10] = 64  # (32,10) -> (31,10)
    d_dir = _t(torch, d)
    w = _t(torch, _weights(d.shape, 5)) if weighted else None
    with pytest.raises(_native.TTCudaError) as e:
        with dev.deferred():
            dev.flow_accumulation(d_dir, w)
    assert e.value.status == 5
    ok = np.full((70, 70), 4, dtype=np.uint8, order="F")
    ok[-1, :] = 0
    with dev.deferred():
        acc = dev.flow_accumulation(_t(torch, ok))
    assert float(acc[0, -1]) == 70.0


def test_deferral_rules(gpu):
    torch = gpu
    from libtopotoolbox_gb300 import _native, dems
    from libtopotoolbox_gb300.api import dev

    lib = _native.lib()
    assert lib.tt_cuda_defer_end() == 1  # not deferring
    shape = (100, 90)
    d_dem = _t(torch, dems.pcg4d_dem(shape, 13))
    d_bc = _t(torch, dems.border_bc(shape))
    side = torch.cuda.Stream()
    with dev.deferred():
        assert lib.tt_cuda_defer_begin(dev._stream()) == 1  # already deferring
        with torch.cuda.stream(side):  # another stream inside the deferral
            with pytest.raises(_native.TTCudaError) as e:
                dev.fillsinks(d_dem, d_bc)
            assert e.value.status == 1
        dev.fillsinks(d_dem, d_bc)
