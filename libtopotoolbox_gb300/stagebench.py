"""Per-stage timing of the D8 pipeline (also the target for ncu captures).

    python -m libtopotoolbox_gb300.stagebench --workload plain_4096 \
        --stage flow_accumulation --reps 5

Runs the stages before `--stage` once to build its inputs, then times the
chosen stage `--reps` times with CUDA events on the current stream and prints
one JSON line (ms per call, Gcells/s, algorithmic GB/s).  `--stage pipeline`
times the whole sequence.  Inputs stay resident in device memory.
"""
from __future__ import annotations

import argparse
import json
import sys

import numpy as np

BYTES = {
    "fillsinks": 9, "identifyflats": 8, "gwdt_computecosts": 24, "gwdt": 12,
    "flow_routing_d8_carve": 21, "flow_accumulation": 13,
    "flow_accumulation_weighted": 17, "flow_accumulation_backward": 9,
    "hillshade_fused": 8, "hillshade_backward": 12, "pipeline": 87,
    "flow_routing_d8_edgelist": 25, "drainagebasins": 24, "flow_accumulation_edgelist": 24,
}
STAGES = ["fillsinks", "identifyflats", "gwdt_computecosts", "gwdt",
          "flow_routing_d8_carve", "flow_accumulation", "flow_accumulation_weighted",
          "flow_accumulation_backward", "hillshade_fused", "hillshade_backward", "pipeline",
          "flow_routing_d8_edgelist", "drainagebasins", "flow_accumulation_edgelist", "batch"]


def load(workload, size):
    from . import dems

    kw = {} if size is None else {"size": size}
    if workload == "grad_8192":
        dem, bc, w, cs = dems.grad_8192(**kw)
        return dem, bc, w, cs
    dem, bc, cs = getattr(dems, workload)(**kw)
    if np.isnan(dem).any():
        dem, bc, _ = dems.nan_to_outlets(dem, bc)
    rng = np.random.default_rng(0)
    w = np.asfortranarray(rng.lognormal(0.0, 0.5, size=dem.shape).astype(np.float32))
    return dem, bc, w, cs


def batch_main(args):
    """Batched workload: `--tiles` DEMs (sides log-uniform 128..2048, aspect
    0.5..2, quantised to 0.1 m) through one tuned mosaic and a CUDA graph,
    against the same DEMs through per-DEM device calls."""
    import time

    import torch

    from . import dems as D
    from .api import dev
    from .batch import Batch, tune

    t0 = time.perf_counter()
    tiles = D.batch_tiles(count=args.tiles)
    gen_s = time.perf_counter() - t0
    dv = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a.T)).to(dv)  # noqa: E731
    dems = [t(d) for d, _ in tiles]
    bcs = [t(b) for _, b in tiles]
    shapes = [d.shape for d, _ in tiles]
    cells = sum(a * b for a, b in shapes)
    best, cands = tune(shapes, dems, bcs, reps=2)
    bt = Batch(shapes)
    out = bt.run(dems, bcs)
    torch.cuda.synchronize()
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731

    def timed(fn, reps):
        ts = []
        for _ in range(reps):
            a, b = ev(), ev()
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.median(ts))

    batched_ms = timed(lambda: bt.run(dems, bcs, outputs=out), args.reps)

    def per_dem():
        for d, b in zip(dems, bcs):
            filled = dev.fillsinks(d, b)
            flats = dev.identifyflats(filled)
            costs, _ = dev.gwdt_computecosts(flats, d, filled)
            dist = dev.gwdt(costs, flats)
            _, direction = dev.flow_routing_d8_carve(filled, dist, flats, want_node=False)
            dev.flow_accumulation(direction)

    per_dem()
    torch.cuda.synchronize()
    per_ms = timed(per_dem, max(1, args.reps // 2))
    info = bt.info()
    print(json.dumps({"stage": "batch", "tiles": len(tiles), "pixels": cells,
                      "canvas": [info["canvas_rows"], info["canvas_cols"]],
                      "graph_nodes": info["graph_nodes"], "batched_ms": batched_ms,
                      "per_dem_ms": per_ms, "speedup": per_ms / batched_ms,
                      "batched_gcells_s": cells / (batched_ms * 1e-3) / 1e9,
                      "per_dem_gcells_s": cells / (per_ms * 1e-3) / 1e9,
                      "tuning": cands, "generate_s": gen_s}))
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="plain_4096",
                    choices=["plain_512", "plain_4096", "plain_16384", "grad_8192"])
    ap.add_argument("--size", type=int, default=None)
    ap.add_argument("--stage", default="pipeline", choices=STAGES)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--tiles", type=int, default=512, help="DEMs for --stage batch")
    args = ap.parse_args(argv)
    if args.stage == "batch":
        return batch_main(args)

    import torch

    from . import _native as N
    from .api import dev

    N.lib()
    dv = torch.device("cuda", 0)
    dem, bc, w, cs = load(args.workload, args.size)
    m, n = dem.shape
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a.T)).to(dv)  # noqa: E731
    d_dem, d_bc, d_w = t(dem), t(bc), t(w)
    st = args.stage

    ctx = {}
    if st != "pipeline":
        filled = dev.fillsinks(d_dem, d_bc)
        flats = dev.identifyflats(filled)
        costs, _ = dev.gwdt_computecosts(flats, d_dem, filled)
        dist = dev.gwdt(costs, flats)
        edges = st in ("flow_routing_d8_edgelist", "drainagebasins", "flow_accumulation_edgelist")
        node, direction = dev.flow_routing_d8_carve(filled, dist, flats, want_node=edges)
        g = torch.rand_like(d_dem) * 2 - 1
        src = tgt = fr = None
        if edges:
            src, tgt = dev.flow_routing_d8_edgelist(node, direction)
            fr = torch.ones(src.numel(), dtype=torch.float32, device=dv)
        ctx = dict(filled=filled, flats=flats, costs=costs, dist=dist, direction=direction, g=g,
                   node=node, src=src, tgt=tgt, fr=fr)
    torch.cuda.synchronize()

    def call():
        c = ctx
        if st == "fillsinks":
            dev.fillsinks(d_dem, d_bc, out=c["filled"])
        elif st == "identifyflats":
            dev.identifyflats(c["filled"], out=c["flats"])
        elif st == "gwdt_computecosts":
            dev.gwdt_computecosts(c["flats"], d_dem, c["filled"])
        elif st == "gwdt":
            dev.gwdt(c["costs"], c["flats"])
        elif st == "flow_routing_d8_carve":
            dev.flow_routing_d8_carve(c["filled"], c["dist"], c["flats"])
        elif st == "flow_accumulation":
            dev.flow_accumulation(c["direction"])
        elif st == "flow_accumulation_weighted":
            dev.flow_accumulation(c["direction"], d_w)
        elif st == "flow_accumulation_backward":
            dev.flow_accumulation_backward(c["direction"], c["g"])
        elif st == "hillshade_fused":
            dev.hillshade_fused(d_dem, 3.9269908, 1.0471976, cs)
        elif st == "hillshade_backward":
            dev.hillshade_backward(d_dem, c["g"], 3.9269908, 1.0471976, cs)
        elif st == "flow_routing_d8_edgelist":
            dev.flow_routing_d8_edgelist(c["node"], c["direction"])
        elif st == "drainagebasins":
            dev.drainagebasins(c["src"], c["tgt"], d_dem)
        elif st == "flow_accumulation_edgelist":
            dev.flow_accumulation_edgelist(c["src"], c["tgt"], c["fr"], d_dem)
        else:
            dev.d8_pipeline(d_dem, d_bc)

    call()
    torch.cuda.synchronize()
    times = []
    stream = torch.cuda.current_stream()
    for _ in range(args.reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        call()
        b.record(stream)
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b))
    ms = float(np.median(times))
    cells = m * n
    print(json.dumps({"stage": st, "workload": args.workload, "dims": [m, n], "ms": ms,
                      "ms_all": times, "gcells_s": cells / (ms * 1e-3) / 1e9,
                      "alg_gbs": BYTES[st] * cells / (ms * 1e-3) / 1e9,
                      "last_rounds": int(N.lib().tt_cuda_last_rounds())}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
