"""Batched form: every DEM of a batch gets exactly what a separate call gives,
and exactly what the oracle gives on DEMs of the batched workload itself.

Uneven tiles (sides 37-300, aspect 0.5-2, quantised to 0.1 m, as in the
batched workload but smaller), run through one mosaic with NaN gutters and a
captured CUDA graph; compared bit for bit with per-DEM device calls, on the
first (captured) run and on a graph replay.
"""
import numpy as np
import pytest

from conftest import same_float

pytestmark = pytest.mark.gpu


def _tiles(count=12, seed=9):
    from libtopotoolbox_gb300 import dems

    return dems.batch_tiles(seed=seed, count=count, side_range=(37, 300))


def _t(a, torch):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a).T)).to("cuda")


def test_batch_matches_single_calls(gpu, tmp_path, monkeypatch):
    torch = gpu
    monkeypatch.setenv("TT_CUDA_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    from libtopotoolbox_gb300.api import dev
    from libtopotoolbox_gb300.batch import Batch, tune

    tiles = _tiles()
    shapes = [d.shape for d, _ in tiles]
    dems = [_t(d, torch) for d, _ in tiles]
    bcs = [_t(b, torch) for _, b in tiles]
    best, results = tune(shapes, dems, bcs, reps=1, scales=(0.9, 1.3))
    assert len(results) == 2 + 5  # two widths, then the other five schedules
    bt = Batch(shapes)  # picks the tuned width and schedule from the cache
    assert bt.info()["canvas_cols"] == best["canvas_cols"]
    assert bt.schedule == best["schedule"]
    first = bt.run(dems, bcs)
    torch.cuda.synchronize()
    snap = {k: [t.clone() for t in v] for k, v in first.items()}
    again = bt.run(dems, bcs, outputs=first)  # graph replay
    torch.cuda.synchronize()
    assert bt.info()["graph_nodes"] > 0
    for k, (d, b) in enumerate(zip(dems, bcs)):
        filled = dev.fillsinks(d, b)
        flats = dev.identifyflats(filled)
        costs, _ = dev.gwdt_computecosts(flats, d, filled)
        dist = dev.gwdt(costs, flats)
        _, direction = dev.flow_routing_d8_carve(filled, dist, flats, want_node=False)
        acc = dev.flow_accumulation(direction)
        ref = {"filled": filled, "flats": flats, "dist": dist, "direction": direction,
               "acc": acc}
        for name, r in ref.items():
            r = r.cpu().numpy()
            for src in (snap, again):
                got = src[name][k].cpu().numpy()
                if r.dtype.kind == "f":
                    assert same_float(got, r), (k, name)
                else:
                    assert np.array_equal(got, r), (k, name)
    bt.close()


def test_batch_workload_sample_vs_oracle(gpu, port, tmp_path, monkeypatch):
    """DEMs drawn from the batched workload itself (512 DEMs, sides
    log-uniform 128-2048, aspect 0.5-2, fractal, quantised to 0.1 m): its
    three largest and five others at random, run as one batch; every output
    of every DEM against the oracle's pipeline on that DEM (which is pinned
    to the reference): filled, flats, dist and directions bit-exact, unit
    accumulation exact."""
    torch = gpu
    monkeypatch.setenv("TT_CUDA_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    from libtopotoolbox_gb300 import dems
    from libtopotoolbox_gb300.batch import Batch

    shapes = dems.batch_tile_shapes()
    area = np.array([a * b for a, b in shapes])
    big = list(np.argsort(-area)[:3])
    rng = np.random.default_rng(4)
    rest = [k for k in rng.permutation(len(shapes)) if k not in big][:5]
    pick = sorted(int(k) for k in big + rest)
    tiles = dems.batch_tiles(only=set(pick))
    assert max(max(d.shape) for d, _ in tiles) >= 1800
    bt = Batch([d.shape for d, _ in tiles])
    out = bt.run([_t(d, torch) for d, _ in tiles], [_t(b, torch) for _, b in tiles])
    torch.cuda.synchronize()
    for k, (dem, bc) in enumerate(tiles):
        r = port.pipeline(dem, bc)
        assert same_float(out["filled"][k].cpu().numpy().T, r["filled"]), (pick[k], "filled")
        assert np.array_equal(out["flats"][k].cpu().numpy().T, r["flats"]), (pick[k], "flats")
        assert same_float(out["dist"][k].cpu().numpy().T, r["dist"]), (pick[k], "dist")
        assert np.array_equal(out["direction"][k].cpu().numpy().T, r["direction"]), (pick[k], "dir")
        assert np.array_equal(out["acc"][k].cpu().numpy().T, r["acc"]), (pick[k], "acc")
    bt.close()


def test_batch_every_schedule_same_bits(gpu, tmp_path, monkeypatch):
    """The sweep schedules the tuner chooses between change only the time:
    every schedule gives the same outputs, bit for bit."""
    torch = gpu
    monkeypatch.setenv("TT_CUDA_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    from libtopotoolbox_gb300.batch import Batch

    tiles = _tiles(count=10, seed=21)
    shapes = [d.shape for d, _ in tiles]
    dems = [_t(d, torch) for d, _ in tiles]
    bcs = [_t(b, torch) for _, b in tiles]
    ref = None
    for sched in range(6):
        bt = Batch(shapes, schedule=sched)
        out = bt.run(dems, bcs)
        torch.cuda.synchronize()
        got = {k: [t.cpu().numpy() for t in v] for k, v in out.items()}
        bt.close()
        if ref is None:
            ref = got
            continue
        for k in ref:
            for a, b in zip(ref[k], got[k]):
                if a.dtype.kind == "f":
                    assert same_float(a, b), (sched, k)
                else:
                    assert np.array_equal(a, b), (sched, k)
