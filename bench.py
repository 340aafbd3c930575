#!/usr/bin/env python
"""Benchmark of the D8 flow pipeline on GB300.

One step = the plain pipeline (fillsinks -> identifyflats ->
gwdt_computecosts -> gwdt -> flow_routing_d8_carve -> flow_accumulation, unit
weights) plus hillshade on one synthetic DEM, through the library's device
entry points with the DEM already in HBM.  The default workload is the
4096 x 4096 fractal with 200 inverted Gaussian pits rounded to 1 m.

Prints one JSON line (rank 0).  `--impl reference` times the CPU
implementation of the same path (the oracle's C restatement of the
reference) on the host cores instead.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Gcells/s fill+D8+acc on 1 GB300 vs CPU; adjoint/fwd time at 1e-5 rel err"
UNIT = "Gcells/s"
# Algorithmic bytes per cell: every API input read once, every output written
# once, scratch excluded (unit weights, prev = NULL).
BYTES = {
    "fillsinks": 9, "identifyflats": 8, "gwdt_computecosts": 24, "gwdt": 12,
    "flow_routing_d8_carve": 21, "flow_accumulation": 13, "hillshade_fused": 8,
}
PIPELINE_BYTES = sum(v for k, v in BYTES.items() if k != "hillshade_fused")  # 87
HS_AZ, HS_ALT = 3.9269908, 1.0471976

WORKLOADS = {
    "plain_4096_hillshade": ("plain_4096", {}),
    "plain_16384": ("plain_16384", {}),
    "plain_512": ("plain_512", {}),
}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def make_workload(name):
    from libtopotoolbox_gb300 import dems

    gen, kw = WORKLOADS[name]
    dem, bc, cs = getattr(dems, gen)(**kw)
    if np.isnan(dem).any():
        dem, bc, _ = dems.nan_to_outlets(dem, bc)
    return dem, bc, cs


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        self.start = 0
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # nvidia-smi takes a moment to start: wait for its first sample,
            # so that the samples kept are all taken during the timed region
            t0 = time.time()
            while not self.lines and time.time() - t0 < 5.0:
                time.sleep(0.01)
            self.start = len(self.lines)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines[self.start:]:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def load_traffic():
    p = ROOT / "profiles" / "roofline_traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            return {}
    return {}


def cpu_baseline_sample(dem, bc, seconds_target=20.0):
    """The oracle port on a bounded crop of the workload, one host core."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle

    orc = pyoracle.Oracle("port")
    side = min(dem.shape[0], 1024)
    crop = np.asfortranarray(dem[:side, :side])
    cb = np.zeros(crop.shape, np.uint8, order="F")
    cb[0, :] = cb[-1, :] = cb[:, 0] = cb[:, -1] = 1
    cb |= np.asfortranarray(bc[:side, :side])
    t0 = time.perf_counter()
    reps = 0
    while True:
        orc.pipeline(crop, cb, hybrid=True)
        reps += 1
        el = time.perf_counter() - t0
        if el > seconds_target or reps >= 50:
            break
    gcps = crop.size * reps / el / 1e9
    return {"value": gcps, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{reps} x plain pipeline (hybrid fill) on a {side}x{side} crop of the "
                      f"workload DEM, oracle C restatement of the reference, 1 thread, "
                      f"{el:.1f} s"}


def adjoint_leg(dev, reps=5):
    """Forward vs forward + adjoint of weighted accumulation (and hillshade) on
    the 8192 x 8192 differentiation workload, with the gradient's relative
    error against the FP64 adjoint oracle."""
    import torch

    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle
    from libtopotoolbox_gb300 import dems
    from libtopotoolbox_gb300.api import dev as D

    dem, bc, w, cs = dems.grad_8192()
    m, n = dem.shape
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a.T)).to(dev)  # noqa: E731
    d_dem, d_bc, d_w = t(dem), t(bc), t(w)
    o = D.d8_pipeline(d_dem, d_bc)
    direction, node = o["direction"], o["node"]
    acc = D.flow_accumulation(direction, d_w)
    torch.cuda.synchronize()
    acc_h = acc.cpu().numpy().T
    dir_h = direction.cpu().numpy().T
    rng = np.random.default_rng(64)
    outl = np.nonzero((dir_h.ravel(order="F") == 0) &
                      (acc_h.ravel(order="F") > np.median(acc_h)))[0]
    sel = rng.choice(outl, size=min(64, outl.size), replace=False)
    target = acc_h.ravel(order="F")[sel].astype(np.float64) * rng.uniform(0.5, 1.5, sel.size)
    g = np.zeros(m * n, np.float32)
    g[sel] = (2.0 * (acc_h.ravel(order="F")[sel] - target)).astype(np.float32)
    d_g = torch.from_numpy(g.reshape(n, m)).to(dev)
    gbar = torch.rand_like(d_dem) * 2 - 1

    def timed(fn):
        ts = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.median(ts))

    fwd = timed(lambda: D.flow_accumulation(direction, d_w, out=acc))
    gw = torch.empty_like(acc)
    adj = timed(lambda: D.flow_accumulation_backward(direction, d_g, out=gw))
    hs = torch.empty_like(d_dem)
    hfwd = timed(lambda: D.hillshade_fused(d_dem, HS_AZ, HS_ALT, cs, out=hs))
    hg = torch.empty_like(d_dem)
    hadj = timed(lambda: D.hillshade_backward(d_dem, gbar, HS_AZ, HS_ALT, cs, out=hg))
    # FP64 adjoint oracle along the same receivers
    orc = pyoracle.Oracle("port")
    node_h = node.cpu().numpy().T
    g64 = orc.flow_accumulation_backward_f64(node_h, dir_h, g.reshape(m, n, order="F"))
    got = gw.cpu().numpy().T
    nrm = float(np.linalg.norm(got - g64) / max(np.linalg.norm(g64), 1e-300))
    mx = float(np.max(np.abs(got - g64)) / max(np.max(np.abs(g64)), 1e-300))
    a64 = orc.flow_accumulation_f64(node_h, dir_h, w)
    fwd_err = float(np.max(np.abs(acc_h - a64) / np.abs(a64)))
    return {"workload": f"grad_8192 ({m}x{n}, lognormal(0,0.5) weights, 64 outlets)",
            "acc_fwd_ms": fwd, "acc_adj_ms": adj, "acc_ratio": (fwd + adj) / fwd,
            "acc_grad_rel_err_norm": nrm, "acc_grad_rel_err_max": mx,
            "acc_fwd_rel_err_max": fwd_err,
            "hillshade_fwd_ms": hfwd, "hillshade_adj_ms": hadj,
            "hillshade_ratio": (hfwd + hadj) / hfwd}


def batch_leg(dev, reps=3, rank=0, world=1, dist=None):
    """512 uneven DEMs: one tuned mosaic replayed from a CUDA graph against
    per-DEM device calls.  With several ranks the DEMs are sharded by pixel
    count (largest first to the least loaded rank); each rank runs its share
    with no collective, and the times are the maximum over ranks."""
    import torch

    from libtopotoolbox_gb300 import dems, shard
    from libtopotoolbox_gb300.api import dev as D
    from libtopotoolbox_gb300.batch import Batch, tune

    all_shapes = dems.batch_tile_shapes()
    cells = sum(a * b for a, b in all_shapes)
    mine = shard.local_indices(all_shapes, rank, world)
    tiles = dems.batch_tiles(only=set(mine))
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a.T)).to(dev)  # noqa: E731
    dm = [t(d) for d, _ in tiles]
    bc = [t(b) for _, b in tiles]
    shapes = [d.shape for d, _ in tiles]
    best, cands = tune(shapes, dm, bc, reps=1)
    bt = Batch(shapes)
    out = bt.run(dm, bc)
    torch.cuda.synchronize()

    def timed(fn, k):
        ts = []
        for _ in range(k):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.median(ts))

    def max_over_ranks(v):
        if dist is None:
            return v
        x = torch.tensor([v], device=dev)
        dist.all_reduce(x, op=dist.ReduceOp.MAX)
        return float(x.item())

    batched = max_over_ranks(timed(lambda: bt.run(dm, bc, outputs=out), reps))

    def per_dem():
        for d, b in zip(dm, bc):
            f = D.fillsinks(d, b)
            fl = D.identifyflats(f)
            c, _ = D.gwdt_computecosts(fl, d, f)
            ds = D.gwdt(c, fl)
            _, dr = D.flow_routing_d8_carve(f, ds, fl, want_node=False)
            D.flow_accumulation(dr)

    per_dem()
    per = max_over_ranks(timed(per_dem, 1))
    info = bt.info()
    bt.close()
    res = {"workload": f"{len(all_shapes)} DEMs, sides log-uniform 128..2048, {cells} pixels",
           "batched_ms": batched, "per_dem_ms": per, "speedup": per / batched,
           "batched_gcells_s": cells / (batched * 1e-3) / 1e9,
           "canvas": [info["canvas_rows"], info["canvas_cols"]],
           "graph_nodes": info["graph_nodes"], "tuned_canvas_cols": best["canvas_cols"]}
    if world > 1:
        res["sharding"] = {"ranks": world, "rule": "largest first to least loaded rank",
                           "pixels_per_rank": shard.loads(all_shapes, world),
                           "canvas_of_rank0": res.pop("canvas")}
    return res


def edges_leg(dev, node, direction, reps=5):
    """The edge-list rows on the workload's own node order and directions:
    flow_routing_d8_edgelist, drainagebasins and flow_accumulation_edgelist
    (device pointers, CUDA events), beside the oracle's C restatement of the
    reference on one host core."""
    import torch

    from libtopotoolbox_gb300.api import dev as D

    cells = direction.numel()
    src, tgt = D.flow_routing_d8_edgelist(node, direction)
    fr = torch.ones(src.numel(), dtype=torch.float32, device=dev)
    like = torch.empty(direction.shape, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()

    def timed(fn):
        ts = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.median(ts))

    ms = {
        "flow_routing_d8_edgelist": timed(lambda: D.flow_routing_d8_edgelist(node, direction)),
        "drainagebasins": timed(lambda: D.drainagebasins(src, tgt, like)),
        "flow_accumulation_edgelist": timed(lambda: D.flow_accumulation_edgelist(src, tgt, fr,
                                                                                   like)),
    }
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle

    orc = pyoracle.Oracle("port")
    nd = node.cpu().numpy().T.copy(order="F")
    dr = direction.cpu().numpy().T.copy(order="F")
    cpu = {}
    t0 = time.perf_counter()
    hs, ht = orc.flow_routing_d8_edgelist(nd, dr)
    cpu["flow_routing_d8_edgelist"] = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    orc.drainagebasins(hs, ht, dr.shape)
    cpu["drainagebasins"] = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    orc.flow_accumulation_edgelist(hs, ht, np.ones(len(hs), np.float32), dr.shape)
    cpu["flow_accumulation_edgelist"] = (time.perf_counter() - t0) * 1e3
    return {"workload": f"edge list of the {dr.shape[0]}x{dr.shape[1]} workload "
                        f"({int(src.numel())} edges)",
            "gpu_ms": ms, "gcells_s": {k: cells / (v * 1e-3) / 1e9 for k, v in ms.items()},
            "cpu_port_ms_1core": cpu,
            "speedup_vs_cpu": {k: cpu[k] / ms[k] for k in ms}}


def graphflood_leg(dem, cs, reps=5):
    """Graphflood's single-flow graph and drainage area on the workload DEM
    (float64, row-major, border BC 3) through the device API, beside the
    oracle's C restatement of the reference on one host core."""
    import ctypes as C

    import torch

    from libtopotoolbox_gb300 import _native as N

    topo = np.ascontiguousarray(np.asarray(dem, np.float64).T)
    bcs = np.ones(topo.shape, np.uint8)
    bcs[0, :] = bcs[-1, :] = bcs[:, 0] = bcs[:, -1] = 3
    n = topo.size
    dv = torch.device("cuda", torch.cuda.current_device())
    d_topo = torch.from_numpy(topo).to(dv)
    d_bcs = torch.from_numpy(bcs).to(dv)
    rcv = torch.empty(n, dtype=torch.int64, device=dv)
    stack = torch.empty(n, dtype=torch.int64, device=dv)
    dist = torch.empty(n, dtype=torch.float64, device=dv)
    don = torch.empty(n * 8, dtype=torch.int64, device=dv)
    ndon = torch.empty(n, dtype=torch.uint8, device=dv)
    area = torch.empty(n, dtype=torch.float64, device=dv)
    dim = (C.c_size_t * 2)(*topo.shape)
    lib = N.lib()
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    p = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731

    def graph():
        N.check(lib.tt_cuda_compute_sfgraph_dev(p(d_topo), p(rcv), p(dist), p(don), p(ndon),
                                                p(stack), p(d_bcs), C.cast(dim, C.c_void_p),
                                                float(cs), True, st), "compute_sfgraph_dev")

    def drain():
        N.check(lib.tt_cuda_compute_drainage_area_single_flow_dev(
            p(area), p(rcv), C.cast(dim, C.c_void_p), float(cs), st),
            "compute_drainage_area_single_flow_dev")

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        return float(np.median(ts))

    ms = {"compute_sfgraph": timed(graph), "compute_drainage_area_single_flow": timed(drain)}
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle

    orc = pyoracle.Oracle("port")
    t0 = time.perf_counter()
    r = orc.compute_sfgraph(topo, bcs, float(cs), True)
    cpu = {"compute_sfgraph": (time.perf_counter() - t0) * 1e3}
    t0 = time.perf_counter()
    orc.compute_drainage_area_single_flow(r[0], r[4], topo.shape, float(cs))
    cpu["compute_drainage_area_single_flow"] = (time.perf_counter() - t0) * 1e3
    return {"workload": f"graphflood single-flow graph, D8, {topo.shape[0]}x{topo.shape[1]} "
                        f"float64 workload DEM",
            "gpu_ms": ms, "gcells_s": {k: n / (v * 1e-3) / 1e9 for k, v in ms.items()},
            "cpu_port_ms_1core": cpu, "speedup_vs_cpu": {k: cpu[k] / ms[k] for k in ms}}


def io_leg(dem, reps=5):
    """The I/O step before the path: the workload DEM as a Fortran-order
    .npy streamed into device memory by the native loader (two pinned
    buffers, reads overlapping copies), against numpy.load + a pageable
    torch upload.  The file sits in the page cache (it was just written), so
    this measures the host-memory-to-device path, not the disk."""
    import tempfile

    import torch

    from libtopotoolbox_gb300 import rasterio

    d = tempfile.mkdtemp(prefix="tt_io_")
    path = os.path.join(d, "dem.npy")
    np.save(path, np.asfortranarray(dem))
    nbytes = dem.size * 4

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        return float(np.median(ts)) * 1e3

    native = timed(lambda: rasterio.read_npy(path))
    base = timed(lambda: torch.from_numpy(np.ascontiguousarray(np.load(path).T)).cuda())
    t = rasterio.read_npy(path)
    out = os.path.join(d, "back.npy")
    wr = timed(lambda: rasterio.write_npy(out, t))
    ok = bool(np.array_equal(np.load(out), dem))
    os.remove(path)
    os.remove(out)
    os.rmdir(d)
    return {"workload": f"{dem.shape[0]}x{dem.shape[1]} float32 .npy ({nbytes} bytes), page cache",
            "read_ms": native, "read_gbs": nbytes / native / 1e6,
            "numpy_load_upload_ms": base, "write_ms": wr, "write_gbs": nbytes / wr / 1e6,
            "roundtrip_exact": ok}


def run_reference(args):
    """--impl reference: the CPU implementation on the host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle
    from concurrent.futures import ThreadPoolExecutor

    orc = pyoracle.Oracle("port")
    dem, bc, cs = make_workload(args.workload)
    cores = os.cpu_count() or 1
    side = min(dem.shape[0], 1024)
    crops = []
    for k in range(cores):
        i0 = (k * 613) % max(1, dem.shape[0] - side + 1)
        j0 = (k * 389) % max(1, dem.shape[1] - side + 1)
        c = np.asfortranarray(dem[i0:i0 + side, j0:j0 + side])
        b = np.zeros(c.shape, np.uint8, order="F")
        b[0, :] = b[-1, :] = b[:, 0] = b[:, -1] = 1
        b |= np.asfortranarray(bc[i0:i0 + side, j0:j0 + side])
        crops.append((c, b))

    def one(cb):
        orc.pipeline(cb[0], cb[1], hybrid=True)
        orc.hillshade_fused(cb[0], HS_AZ, HS_ALT, cs)

    with ThreadPoolExecutor(max_workers=cores) as ex:
        for _ in range(args.warmup):
            list(ex.map(one, crops))
        times = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            list(ex.map(one, crops))
            times.append(time.perf_counter() - t0)
    cells = side * side * cores
    ms = 1e3 * float(np.mean(times))
    value = cells / (ms * 1e-3) / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": args.workload, "sample": f"{cores} concurrent {side}x{side} crops"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"per step: plain pipeline + hillshade on {cores} crops of "
                                   f"{side}x{side}, one per host thread (oracle C restatement; "
                                   f"the reference sources are not on this host)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--workload", default="plain_4096_hillshade", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-edges", action="store_true")
    ap.add_argument("--no-graphflood", action="store_true")
    ap.add_argument("--no-io", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from libtopotoolbox_gb300 import api
    from libtopotoolbox_gb300 import _native as N

    lib = N.lib()
    dem, bc, cs = make_workload(args.workload)
    m, n = dem.shape
    cells = m * n
    # Device-resident inputs: column-major grid == (ncols, nrows) tensor.
    d_dem = torch.from_numpy(np.ascontiguousarray(dem.T)).to(dev)
    d_bc = torch.from_numpy(np.ascontiguousarray(bc.T)).to(dev)
    o = {
        "filled": torch.empty((n, m), dtype=torch.float32, device=dev),
        "flats": torch.empty((n, m), dtype=torch.int32, device=dev),
        "costs": torch.empty((n, m), dtype=torch.float32, device=dev),
        "conncomps": torch.empty((n, m), dtype=torch.int64, device=dev),
        "dist": torch.empty((n, m), dtype=torch.float32, device=dev),
        "node": torch.empty((n, m), dtype=torch.int64, device=dev),
        "direction": torch.empty((n, m), dtype=torch.uint8, device=dev),
        "acc": torch.empty((n, m), dtype=torch.float32, device=dev),
        "hillshade": torch.empty((n, m), dtype=torch.float32, device=dev),
    }
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > L2
    stream = torch.cuda.current_stream(dev)
    sp = N.C.c_void_p(stream.cuda_stream)
    dp, keep = N.dims_arg((m, n))
    P = lambda t: N.C.c_void_p(t.data_ptr())  # noqa: E731

    stages = ["fillsinks", "identifyflats", "gwdt_computecosts", "gwdt",
              "flow_routing_d8_carve", "flow_accumulation", "hillshade_fused"]

    def step(events=None):
        calls = [
            lambda: lib.tt_cuda_fillsinks_dev(P(o["filled"]), P(d_dem), P(d_bc), dp, sp),
            lambda: lib.tt_cuda_identifyflats_dev(P(o["flats"]), P(o["filled"]), dp, None, sp),
            lambda: lib.tt_cuda_gwdt_computecosts_dev(P(o["costs"]), P(o["conncomps"]),
                                                      P(o["flats"]), P(d_dem), P(o["filled"]),
                                                      dp, sp),
            lambda: lib.tt_cuda_gwdt_dev(P(o["dist"]), None, P(o["costs"]), P(o["flats"]), dp, sp),
            lambda: lib.tt_cuda_flow_routing_d8_carve_dev(P(o["node"]), P(o["direction"]),
                                                          P(o["filled"]), P(o["dist"]),
                                                          P(o["flats"]), dp, 0, sp),
            lambda: lib.tt_cuda_flow_accumulation_dev(P(o["acc"]), P(o["direction"]), None, dp, sp),
            lambda: lib.tt_cuda_hillshade_fused_dev(P(o["hillshade"]), P(d_dem), HS_AZ, HS_ALT,
                                                    cs, dp, sp),
        ]
        for k, c in enumerate(calls):
            if events is not None:
                events[k].record(stream)
            N.check(c(), stages[k])
            if stages[k] in ("fillsinks", "gwdt"):
                rounds[stages[k]] = int(lib.tt_cuda_last_rounds())
        if events is not None:
            events[-1].record(stream)

    rounds = {}
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # The headline step: the whole path through its fused entry point
    # (tt_cuda_d8_pipeline_dev, hillshade included), which contracts the
    # receiver forest once for both the node order and the accumulation.
    def pipe_step():
        N.check(lib.tt_cuda_d8_pipeline_dev(
            P(o["filled"]), P(o["flats"]), P(o["dist"]), P(o["node"]), P(o["direction"]),
            P(o["acc"]), P(o["hillshade"]), P(d_dem), P(d_bc), None, HS_AZ, HS_ALT, cs,
            dp, sp), "d8_pipeline_dev")

    for _ in range(args.warmup):
        pipe_step()
    torch.cuda.synchronize()

    stage_ms = {s: [] for s in stages}
    step_ms, fn_ms = [], []
    with ClockSampler(local) as clk:
        barrier()
        lib.tt_cuda_launch_count(1)
        for _ in range(args.steps):
            flush.fill_(1.0)  # L2 flush outside the timed events
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            pipe_step()
            e1.record(stream)
            torch.cuda.synchronize()
            step_ms.append(e0.elapsed_time(e1))
        launches = int(lib.tt_cuda_launch_count(1)) / args.steps
        barrier()
        # The same work as one call per reference function, timed per stage.
        for _ in range(args.steps):
            flush.fill_(1.0)
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(len(stages) + 1)]
            step(ev)
            torch.cuda.synchronize()
            for k, s in enumerate(stages):
                stage_ms[s].append(ev[k].elapsed_time(ev[k + 1]))
            fn_ms.append(ev[0].elapsed_time(ev[-1]))
        barrier()
    ms = float(np.mean(step_ms))
    if dist is not None:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = cells * world / (ms * 1e-3) / 1e9

    # End-to-end through the host-pointer C ABI: pinned host buffers, copies
    # inside the timed region.
    def pinned(shape, dtype):
        t = torch.empty(shape, dtype=dtype, pin_memory=True)
        return t.numpy()

    h_dem = pinned((n, m), torch.float32)
    h_dem[:] = dem.T
    h_bc = pinned((n, m), torch.uint8)
    h_bc[:] = bc.T
    h_out = {k: pinned((n, m), t.dtype) for k, t in o.items()
             if k in ("filled", "flats", "dist", "node", "direction", "acc", "hillshade")}
    hp = lambda a: N.C.c_void_p(a.ctypes.data)  # noqa: E731

    def e2e_step():
        lib.tt_cuda_d8_pipeline(hp(h_out["filled"]), hp(h_out["flats"]), hp(h_out["dist"]),
                                hp(h_out["node"]), hp(h_out["direction"]), hp(h_out["acc"]),
                                hp(h_dem), hp(h_bc), None, dp)
        N.check(N.last_status(), "d8_pipeline")
        lib.tt_cuda_hillshade_fused(hp(h_out["hillshade"]), hp(h_dem), HS_AZ, HS_ALT, cs, dp)
        N.check(N.last_status(), "hillshade_fused")

    e2e_step()
    e2e_ms = []
    for _ in range(max(2, min(args.steps, 5))):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    h2d = cells * (4 + 1) + cells * 4  # dem + bc for the pipeline, dem for hillshade
    d2h = cells * (4 + 4 + 4 + 8 + 1 + 4 + 4)
    e2e_val = cells * world / (float(np.mean(e2e_ms)) * 1e-3) / 1e9

    # The batched leg runs on every rank (each on its share of the DEMs).
    batched = None if args.no_batch else batch_leg(dev, rank=rank, world=world, dist=dist)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0

    hbm, peak_kind = peaks()
    # Dominant stage by time.
    mean_stage = {s: float(np.mean(v)) for s, v in stage_ms.items()}
    dom = max(mean_stage, key=mean_stage.get)
    dom_bytes = BYTES[dom] * cells
    achieved = dom_bytes / (mean_stage[dom] * 1e-3) / 1e9
    traffic = load_traffic().get(f"{args.workload}:{dom}")
    pipe_bytes = PIPELINE_BYTES + BYTES["hillshade_fused"]
    pipe_gbs = pipe_bytes * cells / (ms * 1e-3) / 1e9
    per_fn_ms = float(np.mean(fn_ms))
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": args.workload, "dem": f"{m}x{n} float32 column-major",
                   "weights": "unit", "hillshade": "azimuth 315, altitude 60",
                   "l2": "flushed (512 MiB write) between timed steps",
                   "parallelism": "replicas" if world > 1 else "single"},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm,
                     "unit": "GB/s", "frac": achieved / hbm, "traffic": traffic,
                     "peak_source": peak_kind,
                     "algorithmic_bytes_per_cell": BYTES[dom]},
        "step": "tt_cuda_d8_pipeline_dev (fill, flats, costs, gwdt, carve, "
                "accumulation, hillshade) on device-resident inputs",
        "pipeline_roofline": {"bytes_per_cell": pipe_bytes, "ms": ms,
                              "achieved_gbs": pipe_gbs, "frac": pipe_gbs / hbm},
        "per_function": {"ms_per_step": per_fn_ms,
                         "value": cells * world / (per_fn_ms * 1e-3) / 1e9,
                         "calls": "one tt_cuda_<name>_dev call per reference function"},
        "stages_ms": mean_stage,
        "device_rounds": rounds,
        "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": float(np.mean(e2e_ms)),
                "path": "tt_cuda_d8_pipeline + tt_cuda_hillshade_fused (host pointers)"},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if not args.no_adjoint:
        line["adjoint"] = adjoint_leg(dev)
    if batched is not None:
        line["batched"] = batched
    if not args.no_edges:
        line["edges"] = edges_leg(dev, o["node"], o["direction"])
    if not args.no_graphflood:
        line["graphflood"] = graphflood_leg(dem, cs)
    if not args.no_io:
        line["io"] = io_leg(dem)
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_sample(dem, bc)
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
