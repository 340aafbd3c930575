#!/usr/bin/env python
"""Benchmark of the D8 flow pipeline on GB300.

One step = the plain pipeline (fillsinks -> identifyflats ->
gwdt_computecosts -> gwdt -> flow_routing_d8_carve -> flow_accumulation, unit
weights) on one synthetic DEM, through the library's fused device entry point
with the DEM already in HBM.  The default workload is the whole-chip
16384 x 16384 fractal (5 % nodata disks as -INF outlets, 1000 closed
depressions); the 4096 x 4096 workload with hillshade is measured beside it.

Prints one JSON line (rank 0).  `--impl reference` times the CPU
implementation of the same path (the oracle's C restatement of the
reference, pinned bit for bit to the compiled reference) on whole workload
DEMs on the host cores instead.

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
# Host memory one whole-DEM oracle pipeline holds at its peak (gwdt: DEM, bc,
# filled, flats, costs, dist, heap, back), bytes per pixel, with headroom.
CPU_BYTES_PER_PIXEL = 40
# One whole 16384 x 16384 step of the oracle pipeline on one Grace core:
# 179 s measured (the reference arm's single-step median), per pixel.
CPU_SECONDS_PER_PIXEL = 179.0 / 2**28

# name -> (generator in libtopotoolbox_gb300.dems, hillshade in the step)
WORKLOADS = {
    "plain_16384": ("plain_16384", False),
    "plain_4096_hillshade": ("plain_4096", True),
    "plain_512": ("plain_512", False),
}
SECONDARY = "plain_4096_hillshade"


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def make_workload(name):
    """(dem, bc, cellsize, hillshade) of a workload; NaN nodata becomes -INF
    with bc = 1, the reference callers' convention (test/grid.c:505-515)."""
    from libtopotoolbox_gb300 import dems

    gen, hs = WORKLOADS[name]
    dem, bc, cs = getattr(dems, gen)()
    if np.isnan(dem).any():
        dem, bc, _ = dems.nan_to_outlets(dem, bc)
    return dem, bc, cs, hs


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index, off=False):
        self.index = index
        self.off = off
        self.proc = None
        self.lines = []

    def __enter__(self):
        self.start = 0
        if self.off:
            return self
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


class CpuPipeline(threading.Thread):
    """The oracle's C restatement of the reference pipeline on one whole
    workload DEM, one host thread (the reference's pipeline is serial), run
    beside the GPU legs: its ctypes calls release the GIL."""

    def __init__(self, dem, bc, cs, hillshade):
        super().__init__(daemon=True)
        self.args = (dem, bc, (HS_AZ, HS_ALT, cs) if hillshade else None)
        self.seconds = None
        self.error = None

    def run(self):
        try:
            sys.path.insert(0, str(ROOT / "oracle"))
            import pyoracle

            orc = pyoracle.Oracle("port")
            dem, bc, hs = self.args
            t0 = time.perf_counter()
            orc.run_pipeline(dem, bc, hillshade=hs)
            self.seconds = time.perf_counter() - t0
        except Exception as e:  # reported in the JSON line
            self.error = repr(e)

    def result(self, what):
        self.join()
        m, n = self.args[0].shape
        if self.seconds is None:
            return {"value": None, "unit": UNIT, "cores": 1, "kind": "port",
                    "sample": what, "error": self.error}
        return {"value": m * n / self.seconds / 1e9, "unit": UNIT, "cores": 1, "kind": "port",
                "seconds": self.seconds,
                "sample": f"{what}: one whole {m}x{n} workload DEM through fillsinks_hybrid, "
                          f"identifyflats, gwdt_computecosts, gwdt, flow_routing_d8_carve, "
                          f"flow_accumulation (oracle C restatement of the reference, pinned bit "
                          f"for bit to it), 1 thread, {self.seconds:.1f} s"}


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

    def per_dem_deferred():  # the same calls without a host round trip each
        with D.deferred():
            per_dem()

    per_dem_deferred()
    per_def = max_over_ranks(timed(per_dem_deferred, 1))
    info = bt.info()
    bt.close()
    res = {"workload": f"{len(all_shapes)} DEMs, sides log-uniform 128..2048, {cells} pixels",
           "batched_ms": batched, "per_dem_ms": per, "speedup": per / batched,
           "per_dem_deferred_ms": per_def, "speedup_vs_deferred": per_def / batched,
           "batched_gcells_s": cells / (batched * 1e-3) / 1e9,
           "canvas": [info["canvas_rows"], info["canvas_cols"]],
           "graph_nodes": info["graph_nodes"], "tuned_canvas_cols": best["canvas_cols"],
           "tuned_schedule": best["schedule"], "tuning": cands}
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


def mem_available():
    try:
        for ln in open("/proc/meminfo"):
            if ln.startswith("MemAvailable:"):
                return int(ln.split()[1]) * 1024
    except OSError:
        pass
    return 0


def run_reference(args):
    """--impl reference: the CPU implementation on whole workload DEMs.

    Every timed step is one whole DEM of the workload (the same DEM, config
    and metric as the GPU arm) through the oracle's C restatement of the
    reference, which is serial per DEM; steps run concurrently on the host
    cores, as many at once as the cores and the host memory allow.  A crop
    is not the same workload (the CPU cost per pixel grows with the DEM), so
    the warm-up steps, which only warm the code path (there is no compiler
    or cache state to prepare across whole-DEM runs), run on the workload's
    top-left 1024 x 1024 corner.  value = K * pixels / wall time of the K
    timed steps.  When K whole DEMs at that concurrency would take longer
    than --ref-budget-s, the arm prints its `unavailable` line instead, with
    the single-step time it is projected from."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle
    from concurrent.futures import ThreadPoolExecutor

    orc = pyoracle.Oracle("port")
    dem, bc, cs, hs = make_workload(args.workload)
    cells = dem.size
    cores = os.cpu_count() or 1
    per = cells * CPU_BYTES_PER_PIXEL
    avail = mem_available()
    mem_conc = int(0.7 * avail / per) if avail else 1
    conc = max(1, min(cores, args.steps, mem_conc))
    hsarg = (HS_AZ, HS_ALT, cs) if hs else None
    rounds = -(-args.steps // conc)
    projected = rounds * CPU_SECONDS_PER_PIXEL * cells
    if projected > args.ref_budget_s:
        m, n = dem.shape
        print(json.dumps({
            "impl": "reference",
            "unavailable": f"{args.steps} whole {m}x{n} DEM steps, {conc} at a time (host "
                           f"memory), need ~{projected / 60:.0f} min at the measured "
                           f"{CPU_SECONDS_PER_PIXEL * 2**28:.0f} s per 16384x16384 step on one "
                           f"Grace core, beyond the {args.ref_budget_s / 60:.0f} min budget of "
                           f"this arm; a crop is not the same workload"}), flush=True)
        return 0
    c0 = min(1024, dem.shape[0]), min(1024, dem.shape[1])
    wdem = np.asfortranarray(dem[:c0[0], :c0[1]])
    wbc = np.asfortranarray(bc[:c0[0], :c0[1]]).copy()
    wbc[0, :] = wbc[-1, :] = 1
    wbc[:, 0] = wbc[:, -1] = 1

    def one(whole):
        t0 = time.perf_counter()
        if whole:
            orc.run_pipeline(dem, bc, hillshade=hsarg)
        else:
            orc.run_pipeline(wdem, wbc, hillshade=hsarg)
        return time.perf_counter() - t0

    with ThreadPoolExecutor(max_workers=conc) as ex:
        warm = list(ex.map(one, [False] * args.warmup))
        t0 = time.perf_counter()
        per_step = list(ex.map(one, [True] * args.steps))
        wall = time.perf_counter() - t0
    ms = 1e3 * wall / args.steps
    value = cells * args.steps / wall / 1e9
    m, n = dem.shape
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": workload_config(args.workload, dem.shape, hs, 1),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": conc, "kind": "port",
                         "sample": f"per step one whole {m}x{n} workload DEM through the "
                                   f"pipeline{' + hillshade' if hs else ''} (oracle C "
                                   f"restatement of the reference, pinned bit for bit to it; "
                                   f"the reference's sources are not on this host); {conc} "
                                   f"steps at a time, one per core (the fewest of K, the "
                                   f"{cores} host cores and the {max(mem_conc, 1)} that "
                                   f"{avail / 2**30:.0f} GiB of host memory hold)",
                         "single_step_s": {"median": float(np.median(per_step)),
                                           "min": float(np.min(per_step)),
                                           "max": float(np.max(per_step))},
                         "warmup": f"{args.warmup} untimed steps on the top-left "
                                   f"{c0[0]}x{c0[1]} corner ({float(np.sum(warm)):.1f} s)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def workload_config(name, shape, hillshade, world):
    m, n = shape
    cfg = {"workload": name, "dem": f"{m}x{n} float32 column-major", "weights": "unit",
           "l2": "inputs larger than L2, and L2 flushed (512 MiB write) between timed steps",
           "parallelism": "replicas" if world > 1 else "single"}
    if name == "plain_16384":
        cfg["nodata"] = "5 % NaN disks, as -INF outlets with bc = 1"
    if hillshade:
        cfg["hillshade"] = "azimuth 315, altitude 60"
    return cfg


def gpu_pipeline_leg(N, dev, name, steps, warmup, world=1, dist=None, clocks=None):
    """Times one workload on the GPU.  Returns the measurements and the
    device outputs (node, direction) for the legs that reuse them.

    * fused: tt_cuda_d8_pipeline_dev on device-resident inputs (the
      headline), CUDA events on the launching stream, L2 flushed between
      steps;
    * per function: one tt_cuda_<name>_dev call per reference function,
      timed stage by stage;
    * e2e: the host-pointer C ABI (tt_cuda_d8_pipeline, and
      tt_cuda_hillshade_fused where the workload has hillshade) from pinned
      host buffers, copies inside the timed region."""
    import torch

    lib = N.lib()
    dem, bc, cs, hs = make_workload(name)
    m, n = dem.shape
    cells = m * n
    d_dem = torch.from_numpy(np.ascontiguousarray(dem.T)).to(dev)
    d_bc = torch.from_numpy(np.ascontiguousarray(bc.T)).to(dev)
    mk = lambda dt: torch.empty((n, m), dtype=dt, device=dev)  # noqa: E731
    o = {"filled": mk(torch.float32), "flats": mk(torch.int32), "costs": mk(torch.float32),
         "conncomps": mk(torch.int64), "dist": mk(torch.float32), "node": mk(torch.int64),
         "direction": mk(torch.uint8), "acc": mk(torch.float32)}
    if hs:
        o["hillshade"] = mk(torch.float32)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > L2
    stream = torch.cuda.current_stream(dev)
    sp = N.C.c_void_p(stream.cuda_stream)
    dp, keep = N.dims_arg((m, n))
    P = lambda t: N.C.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731

    stages = ["fillsinks", "identifyflats", "gwdt_computecosts", "gwdt",
              "flow_routing_d8_carve", "flow_accumulation"] + (["hillshade_fused"] if hs else [])
    rounds = {}

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
            lambda: lib.tt_cuda_hillshade_fused_dev(P(o.get("hillshade")), P(d_dem), HS_AZ, HS_ALT,
                                                    cs, dp, sp),
        ]
        for k, st in enumerate(stages):
            if events is not None:
                events[k].record(stream)
            N.check(calls[k](), st)
            if st in ("fillsinks", "gwdt"):
                rounds[st] = int(lib.tt_cuda_last_rounds())
        if events is not None:
            events[-1].record(stream)

    def pipe_step():
        N.check(lib.tt_cuda_d8_pipeline_dev(
            P(o["filled"]), P(o["flats"]), P(o["dist"]), P(o["node"]), P(o["direction"]),
            P(o["acc"]), P(o.get("hillshade")), P(d_dem), P(d_bc), None, HS_AZ, HS_ALT, cs,
            dp, sp), "d8_pipeline_dev")

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(warmup):
        step()
    for _ in range(warmup):
        pipe_step()
    torch.cuda.synchronize()

    stage_ms = {s: [] for s in stages}
    step_ms, fn_ms = [], []
    with (clocks if clocks is not None else ClockSampler(None, off=True)) as clk:
        barrier()
        lib.tt_cuda_launch_count(1)
        for _ in range(steps):
            flush.fill_(1.0)  # L2 flush outside the timed events
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            pipe_step()
            e1.record(stream)
            torch.cuda.synchronize()
            step_ms.append(e0.elapsed_time(e1))
        launches = int(lib.tt_cuda_launch_count(1)) / steps
        barrier()
    # The same work as one call per reference function, timed per stage.
    for _ in range(steps):
        flush.fill_(1.0)
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(len(stages) + 1)]
        step(ev)
        torch.cuda.synchronize()
        for k, st in enumerate(stages):
            stage_ms[st].append(ev[k].elapsed_time(ev[k + 1]))
        fn_ms.append(ev[0].elapsed_time(ev[-1]))
    barrier()
    ms = float(np.mean(step_ms))
    if dist is not None:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())

    # End to end through the host-pointer C ABI: pinned host buffers, copies
    # inside the timed region.
    def pinned(dtype):
        return torch.empty((n, m), dtype=dtype, pin_memory=True).numpy()

    h_dem = pinned(torch.float32)
    h_dem[:] = dem.T
    h_bc = pinned(torch.uint8)
    h_bc[:] = bc.T
    outs = ["filled", "flats", "dist", "node", "direction", "acc"] + (["hillshade"] if hs else [])
    h_out = {k: pinned(o[k].dtype) for k in outs}
    hp = lambda a: N.C.c_void_p(a.ctypes.data)  # noqa: E731

    def e2e_step():
        lib.tt_cuda_d8_pipeline(hp(h_out["filled"]), hp(h_out["flats"]), hp(h_out["dist"]),
                                hp(h_out["node"]), hp(h_out["direction"]), hp(h_out["acc"]),
                                hp(h_dem), hp(h_bc), None, dp)
        N.check(N.last_status(), "d8_pipeline")
        if hs:
            lib.tt_cuda_hillshade_fused(hp(h_out["hillshade"]), hp(h_dem), HS_AZ, HS_ALT, cs, dp)
            N.check(N.last_status(), "hillshade_fused")

    e2e_step()
    e2e_ms = []
    for _ in range(max(2, min(steps, 5))):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    h2d = cells * (4 + 1) + (cells * 4 if hs else 0)  # dem + bc (+ dem for hillshade)
    d2h = sum(o[k].element_size() for k in outs) * cells
    mean_stage = {st: float(np.mean(v)) for st, v in stage_ms.items()}
    per_fn_ms = float(np.mean(fn_ms))
    res = {
        "workload": name, "config": workload_config(name, (m, n), hs, world),
        "cells": cells, "ms": ms, "value": cells * world / (ms * 1e-3) / 1e9,
        "launches": launches, "stages_ms": mean_stage, "device_rounds": rounds,
        "per_function": {"ms_per_step": per_fn_ms,
                         "value": cells * world / (per_fn_ms * 1e-3) / 1e9,
                         "calls": "one tt_cuda_<name>_dev call per reference function"},
        "e2e": {"value": cells * world / (float(np.mean(e2e_ms)) * 1e-3) / 1e9, "unit": UNIT,
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": float(np.mean(e2e_ms)),
                "path": "tt_cuda_d8_pipeline" + (" + tt_cuda_hillshade_fused" if hs else "")
                        + " (host pointers, pinned buffers)"},
        "hillshade": hs,
    }
    keep_out = {"node": o["node"], "direction": o["direction"], "dem": dem, "bc": bc, "cs": cs}
    return res, keep_out


def roofline_of(res, name):
    hbm, peak_kind = peaks()
    st = res["stages_ms"]
    dom = max(st, key=st.get)
    achieved = BYTES[dom] * res["cells"] / (st[dom] * 1e-3) / 1e9
    pipe_bytes = PIPELINE_BYTES + (BYTES["hillshade_fused"] if res["hillshade"] else 0)
    pipe_gbs = pipe_bytes * res["cells"] / (res["ms"] * 1e-3) / 1e9
    return ({"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
             "frac": achieved / hbm, "traffic": load_traffic().get(f"{name}:{dom}"),
             "peak_source": peak_kind, "algorithmic_bytes_per_cell": BYTES[dom]},
            {"bytes_per_cell": pipe_bytes, "ms": res["ms"], "achieved_gbs": pipe_gbs,
             "frac": pipe_gbs / hbm, "peak_source": peak_kind})


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--workload", default="plain_16384", choices=sorted(WORKLOADS))
    ap.add_argument("--ref-budget-s", type=float, default=1800.0,
                    help="reference arm: longest projected run of the timed whole-DEM steps")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true")
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

    from libtopotoolbox_gb300 import _native as N

    N.lib()
    clk = ClockSampler(local)
    head, out = gpu_pipeline_leg(N, dev, args.workload, args.steps, args.warmup, world, dist,
                                 clocks=clk)
    torch.cuda.empty_cache()
    cpu_threads = {}
    if rank == 0 and not args.no_cpu_baseline:
        # Whole-DEM CPU runs of the headline (and secondary) workload, one
        # host thread each, beside the remaining GPU legs.
        cpu_threads["head"] = CpuPipeline(out["dem"], out["bc"], out["cs"], head["hillshade"])
        cpu_threads["head"].start()
    secondary = None
    sec_out = None
    if not args.no_secondary and args.workload != SECONDARY:
        secondary, sec_out = gpu_pipeline_leg(N, dev, SECONDARY, args.steps, args.warmup,
                                              world, dist)
        if rank == 0 and not args.no_cpu_baseline:
            cpu_threads["secondary"] = CpuPipeline(sec_out["dem"], sec_out["bc"], sec_out["cs"],
                                                   secondary["hillshade"])
            cpu_threads["secondary"].start()
    # The batched leg runs on every rank (each on its share of the DEMs).
    batched = None if args.no_batch else batch_leg(dev, rank=rank, world=world, dist=dist)

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return 0

    roof, pipe_roof = roofline_of(head, args.workload)
    line = {
        "metric": METRIC, "value": head["value"], "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["ms"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": head["config"], "roofline": roof,
        "step": "tt_cuda_d8_pipeline_dev (fill, flats, costs, gwdt, carve, accumulation"
                + (", hillshade" if head["hillshade"] else "") + ") on device-resident inputs",
        "pipeline_roofline": pipe_roof, "per_function": head["per_function"],
        "stages_ms": head["stages_ms"], "device_rounds": head["device_rounds"],
        "e2e": head["e2e"], "gpu_launches": head["launches"], "clocks": clk.summary(),
    }
    small = sec_out if sec_out is not None else out
    if not args.no_adjoint:
        line["adjoint"] = adjoint_leg(dev)
    if batched is not None:
        line["batched"] = batched
    if not args.no_edges:
        line["edges"] = edges_leg(dev, small["node"], small["direction"])
    if not args.no_graphflood:
        line["graphflood"] = graphflood_leg(small["dem"], small["cs"])
    if not args.no_io:
        line["io"] = io_leg(small["dem"])
    if secondary is not None:
        sroof, spipe = roofline_of(secondary, SECONDARY)
        secondary.update({"roofline": sroof, "pipeline_roofline": spipe})
        if "secondary" in cpu_threads:
            secondary["cpu_same_config"] = cpu_threads["secondary"].result(
                "same workload and config as this leg")
            cv = secondary["cpu_same_config"]["value"]
            if cv:
                secondary["speedup_vs_cpu"] = {"device_resident": secondary["value"] / cv,
                                               "e2e": secondary["e2e"]["value"] / cv}
        line["secondary"] = secondary
    if "head" in cpu_threads:
        line["cpu_baseline"] = cpu_threads["head"].result(
            "same workload and config as the headline")
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
