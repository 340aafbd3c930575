"""Sharding independent DEMs across ranks (libtopotoolbox_gb300.shard), on
CPU: the assignment rule, and a world_size-2 gloo run in which each rank
fills its own DEMs (with the oracle standing in for its GPU) and rank 0
gathers the results on the host.  The data path has no collective; the
only messages are the host gather of results."""
import os
import socket
import sys
import tempfile
from pathlib import Path

import numpy as np
import pytest

from libtopotoolbox_gb300 import shard

ROOT = Path(__file__).resolve().parent.parent


def _shapes(n, seed):
    rng = np.random.default_rng(seed)
    side = np.exp(rng.uniform(np.log(16), np.log(200), size=n))
    asp = rng.uniform(0.5, 2.0, size=n)
    return [(max(3, int(s * np.sqrt(a))), max(3, int(s / np.sqrt(a)))) for s, a in zip(side, asp)]


@pytest.mark.parametrize("world", [1, 2, 3, 4, 8])
def test_assign_cover_and_balance(world):
    shapes = _shapes(257, 4)
    owner = shard.assign(shapes, world)
    assert len(owner) == len(shapes) and set(owner) <= set(range(world))
    assert owner == shard.assign(shapes, world)  # every rank computes the same
    parts = [shard.local_indices(shapes, r, world) for r in range(world)]
    assert sorted(i for p in parts for i in p) == list(range(len(shapes)))
    pix = [a * b for a, b in shapes]
    ld = shard.loads(shapes, world)
    assert sum(ld) == sum(pix)
    # any greedy list assignment stays within total / world + largest DEM
    assert max(ld) <= sum(pix) / world + max(pix)
    # largest-first greedy is far tighter on many mid-sized DEMs
    assert max(ld) <= 1.02 * sum(pix) / world + 1


def test_assign_edge_cases():
    assert shard.assign([], 3) == []
    assert shard.assign([(10, 10)], 4) == [0]
    # equal sizes go round-robin in index order
    assert shard.assign([(5, 5)] * 6, 3) == [0, 1, 2, 0, 1, 2]
    # one huge DEM sits alone on its rank
    owner = shard.assign([(1000, 1000), (10, 10), (10, 10), (10, 10)], 2)
    assert owner[0] == 0 and owner[1:] == [1, 1, 1]
    with pytest.raises(ValueError):
        shard.assign([(3, 3)], 0)
    with pytest.raises(ValueError):
        shard.local_indices([(3, 3)], 2, 2)


def test_batch_workload_balance():
    from libtopotoolbox_gb300 import dems

    shapes = dems.batch_tile_shapes()
    pix = sum(a * b for a, b in shapes)
    for world in (2, 4, 8):
        ld = shard.loads(shapes, world)
        assert max(ld) / (pix / world) < 1.01, (world, max(ld) / (pix / world))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, outdir):
    sys.path.insert(0, str(ROOT))
    sys.path.insert(0, str(ROOT / "oracle"))
    import torch.distributed as dist

    import pyoracle
    from libtopotoolbox_gb300 import dems, shard

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        shapes = _shapes(24, 9)
        mine = shard.local_indices(shapes, rank, world)
        port_ = pyoracle.Oracle("port")
        local = {}
        for i in mine:  # this rank's DEMs only: no exchange while computing
            d = dems.pcg4d_dem(shapes[i], 100 + i)
            local[i] = {"filled": port_.fillsinks(d, dems.border_bc(shapes[i])), "rank": rank}
        merged = shard.gather_results(local, dst=0)
        if rank == 0:
            np.savez(os.path.join(outdir, "merged.npz"),
                     **{f"f{i}": v["filled"] for i, v in merged.items()},
                     **{f"r{i}": np.int64(v["rank"]) for i, v in merged.items()})
        else:
            assert merged is None
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks_gather(port):
    import multiprocessing as mp

    pytest.importorskip("torch.distributed")
    world = 2
    shapes = _shapes(24, 9)
    with tempfile.TemporaryDirectory() as outdir:
        ctx = mp.get_context("spawn")
        p_port = _free_port()
        procs = [ctx.Process(target=_rank_main, args=(r, world, p_port, outdir))
                 for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=120)
        for p in procs:
            if p.is_alive():
                p.kill()
        assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
        got = np.load(os.path.join(outdir, "merged.npz"))
        owner = shard.assign(shapes, world)
        from libtopotoolbox_gb300 import dems

        for i, shp in enumerate(shapes):
            d = dems.pcg4d_dem(shp, 100 + i)
            exp = port.fillsinks(d, dems.border_bc(shp))
            assert np.array_equal(got[f"f{i}"], exp), i
            assert int(got[f"r{i}"]) == owner[i], i
