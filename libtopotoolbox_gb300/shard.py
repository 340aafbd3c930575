"""Independent DEMs across ranks: one process per GPU, no data-path collective.

The batched workload's DEMs share nothing, so each rank runs the DEMs
assigned to it through its own `Batch` on its own GPU.  A single DEM does
not shard (fill, gwdt and accumulation propagate across the whole grid);
for one DEM every rank is a replica.

    owner = assign(shapes, world)                  # rank of every DEM
    mine = local_indices(shapes, rank, world)      # this rank's DEMs
    out = run_batch_sharded(dems, bcs, rank, world)  # this rank's results
    full = gather_results(out, dst=0)              # host gather on rank 0

Assignment is the longest-processing-time rule on pixel counts: DEMs in
decreasing size (ties by index) each go to the rank with the fewest pixels
so far (ties to the lowest rank).  Its largest per-rank load is within
4/3 - 1/(3 world) of the best possible, and every rank computes the same
assignment locally, so ranks agree without exchanging anything.
"""
from __future__ import annotations

import heapq


def _pixels(shape):
    return int(shape[0]) * int(shape[1])


def assign(shapes, world: int):
    """Rank (0 .. world-1) of every DEM, by the longest-processing-time rule
    on pixel counts."""
    if world < 1:
        raise ValueError("world must be at least 1")
    order = sorted(range(len(shapes)), key=lambda i: (-_pixels(shapes[i]), i))
    heap = [(0, r) for r in range(world)]  # (pixels so far, rank)
    owner = [0] * len(shapes)
    for i in order:
        load, r = heapq.heappop(heap)
        owner[i] = r
        heapq.heappush(heap, (load + _pixels(shapes[i]), r))
    return owner


def local_indices(shapes, rank: int, world: int):
    """Indices of the DEMs rank `rank` runs, in increasing order."""
    if not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside 0..{world - 1}")
    return [i for i, r in enumerate(assign(shapes, world)) if r == rank]


def loads(shapes, world: int):
    """Pixels per rank under `assign`."""
    out = [0] * world
    for i, r in enumerate(assign(shapes, world)):
        out[r] += _pixels(shapes[i])
    return out


def run_batch_sharded(dems, bcs, rank: int, world: int, canvas_cols=None):
    """Runs this rank's DEMs (CUDA tensors of shape (ncols, nrows)) through
    one `Batch` on the current device.  Returns {DEM index: output dict of
    this rank's DEMs}; nothing is exchanged with other ranks."""
    from .batch import Batch

    shapes = [(int(d.shape[1]), int(d.shape[0])) for d in dems]
    mine = local_indices(shapes, rank, world)
    if not mine:
        return {}
    bt = Batch([shapes[i] for i in mine], canvas_cols=canvas_cols)
    try:
        out = bt.run([dems[i] for i in mine], [bcs[i] for i in mine])
    finally:
        bt.close()
    return {i: {k: v[n] for k, v in out.items()} for n, i in enumerate(mine)}


def gather_results(local: dict, dst: int = 0, group=None, to_host: bool = True):
    """Host gather of per-DEM results onto rank `dst` over torch.distributed
    (any backend that carries Python objects, gloo included).  Returns the
    merged {DEM index: result} on `dst` and None elsewhere.  Tensors are
    moved to host memory first when `to_host` is set."""
    import torch
    import torch.distributed as dist

    def host(v):
        if isinstance(v, torch.Tensor):
            return v.detach().cpu()
        if isinstance(v, dict):
            return {k: host(x) for k, x in v.items()}
        return v

    payload = {i: host(v) for i, v in local.items()} if to_host else local
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    parts = [None] * world if rank == dst else None
    dist.gather_object(payload, parts, dst=dst, group=group)
    if rank != dst:
        return None
    merged = {}
    for p in parts:
        overlap = merged.keys() & p.keys()
        if overlap:
            raise RuntimeError(f"DEMs {sorted(overlap)[:5]} returned by two ranks")
        merged.update(p)
    return merged
