"""Batched D8 pipeline over many independent DEMs (tt_cuda_batch_*).

    runner = Batch([dem.shape for dem in dems])      # tuned mosaic width
    out = runner.run(dem_tensors, bc_tensors)         # dict of lists

Each DEM is a column-major grid held as a contiguous CUDA tensor of shape
(ncols, nrows).  All DEMs go through fill -> flats -> costs -> gwdt ->
directions -> unit accumulation with one launch per stage for the whole
batch; the first run with a set of tensors is captured into a CUDA graph
that later runs with the same tensors replay.

The tuning parameters are the mosaic width (the shape of the canvas the
DEMs are packed into) and the sweep schedule of the tile relaxations (fill
and gwdt: column or row sweeps first, visits run to local convergence or
capped at 8 sweeps, or visits ordered by value in bands; see
tt_cuda_set_relax_schedule).  `tune()` times
candidate widths on the actual batch, then every schedule at the best
width, and stores the fastest pair, keyed by the batch's shapes, in a JSON
cache (``TT_CUDA_AUTOTUNE_CACHE`` or
``~/.cache/libtopotoolbox_gb300/autotune.json``).
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import math
import os
from pathlib import Path

from . import _native as N

CANDIDATE_SCALES = (0.8, 1.0, 1.25, 1.6)
SCHEDULES = (0, 1, 2, 3, 4, 5)


def cache_path() -> Path:
    p = os.environ.get("TT_CUDA_AUTOTUNE_CACHE")
    if p:
        return Path(p)
    return Path.home() / ".cache" / "libtopotoolbox_gb300" / "autotune.json"


def signature(shapes) -> str:
    h = hashlib.sha1(json.dumps([list(map(int, s)) for s in shapes]).encode()).hexdigest()
    return f"batch:{len(shapes)}:{h[:16]}"


def _load_cache():
    try:
        return json.loads(cache_path().read_text())
    except Exception:
        return {}


def _store_cache(key, value):
    d = _load_cache()
    d[key] = value
    p = cache_path()
    try:
        p.parent.mkdir(parents=True, exist_ok=True)
        p.write_text(json.dumps(d, indent=1))
    except OSError:
        pass


class Batch:
    """A planned batch.  `shapes` are (nrows, ncols) per DEM."""

    def __init__(self, shapes, canvas_cols: int | None = None, schedule: int | None = None):
        self.shapes = [(int(a), int(b)) for a, b in shapes]
        tuned = _load_cache().get(signature(self.shapes), {})
        if canvas_cols is None:
            canvas_cols = tuned.get("canvas_cols", 0)
        if schedule is None:
            schedule = tuned.get("schedule", 0)
        self.canvas_cols = int(canvas_cols)
        self.schedule = int(schedule)
        lib = N.lib()
        dims = (C.c_int64 * (2 * len(self.shapes)))(*[v for s in self.shapes for v in s])
        h = C.c_void_p()
        N.check(lib.tt_cuda_batch_create(len(self.shapes), C.cast(dims, N.PD),
                                         self.canvas_cols, C.byref(h)), "batch_create")
        self._h = h

    def info(self):
        arr = (C.c_int64 * 4)()
        N.check(N.lib().tt_cuda_batch_info(self._h, arr), "batch_info")
        return {"canvas_rows": arr[0], "canvas_cols": arr[1], "pixels": arr[2],
                "graph_nodes": arr[3]}

    def close(self):
        if getattr(self, "_h", None):
            N.lib().tt_cuda_batch_destroy(self._h)
            self._h = None

    __del__ = close

    def run(self, dems, bcs, outputs=None, stream=None):
        """dems / bcs: lists of CUDA tensors (ncols, nrows).  Returns a dict
        of output lists (filled, flats, dist, direction, acc)."""
        import torch

        B = len(self.shapes)
        if outputs is None:
            outputs = {
                "filled": [torch.empty_like(d) for d in dems],
                "flats": [torch.empty(d.shape, dtype=torch.int32, device=d.device) for d in dems],
                "dist": [torch.empty_like(d) for d in dems],
                "direction": [torch.empty(d.shape, dtype=torch.uint8, device=d.device)
                              for d in dems],
                "acc": [torch.empty_like(d) for d in dems],
            }

        def arr(ts):
            if ts is None:
                return None
            return (C.c_void_p * B)(*[t.data_ptr() for t in ts])

        keep = [arr(dems), arr(bcs)] + [arr(outputs.get(k)) for k in
                                        ("filled", "flats", "dist", "direction", "acc")]
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        lib = N.lib()
        lib.tt_cuda_set_relax_schedule(self.schedule)  # taken when the graph is captured
        try:
            N.check(lib.tt_cuda_batch_run(self._h, *[C.cast(a, C.c_void_p) if a is not None
                                                     else None for a in keep],
                                          C.c_void_p(st)), "batch_run")
        finally:
            lib.tt_cuda_set_relax_schedule(-1)
        return outputs


def tune(shapes, dems, bcs, reps: int = 2, scales=CANDIDATE_SCALES, schedules=SCHEDULES):
    """Time candidate mosaic widths (schedule 0), then every sweep schedule
    at the best width, on this batch; cache and return the fastest."""
    import torch

    area = sum((a + 1) * (b + 1) for a, b in shapes)
    base = math.sqrt(area * 1.15)
    results = []

    def measure(cols, sched):
        bt = Batch(shapes, canvas_cols=cols, schedule=sched)
        out = bt.run(dems, bcs)  # plain run + capture
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            bt.run(dems, bcs, outputs=out)
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        info = bt.info()
        bt.close()
        results.append({"canvas_cols": info["canvas_cols"], "schedule": sched, "ms": min(ts),
                        "canvas_pixels": info["canvas_rows"] * info["canvas_cols"]})
        return results[-1]

    best = None
    for sc in scales:
        r = measure(int(base * sc), 0)
        if best is None or r["ms"] < best["ms"]:
            best = r
    for sched in schedules:
        if sched == 0:
            continue
        r = measure(best["canvas_cols"], sched)
        if r["ms"] < best["ms"]:
            best = r
    _store_cache(signature(shapes), {"canvas_cols": best["canvas_cols"],
                                     "schedule": best["schedule"], "ms": best["ms"],
                                     "candidates": results})
    return best, results
