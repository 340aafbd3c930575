"""ctypes wrappers of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Two libraries share one interface:

* ``Oracle("port")`` loads ``oracle/liboracle.so`` -- the project-written C
  restatement of libtopotoolbox's D8 path (oracle/tt_oracle.c), buildable on
  any host with gcc;
* ``Oracle("ref")`` loads ``oracle/_ref/libtopotoolbox_ref.so`` -- the
  reference's own sources compiled by ``make -C oracle ref`` where they are
  available.

Only tests/, the smoke check and bench.py's CPU-baseline leg use this module,
and only as the checker or the timed CPU baseline.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_LIB = HERE / "liboracle.so"
REF_LIB = HERE / "_ref" / "libtopotoolbox_ref.so"

P = C.c_void_p
PD = C.POINTER(C.c_int64)
F = C.c_float
D = C.c_double


def build_port() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    return PORT_LIB


def reference_root(root=None) -> Path | None:
    """The reference checkout: `root`, else $TT_REFERENCE_ROOT; None when
    neither names a directory holding the reference's sources."""
    root = root or os.environ.get("TT_REFERENCE_ROOT")
    if not root or not (Path(root) / "src" / "fillsinks.c").exists():
        return None
    return Path(root)


def build_ref(root=None) -> Path | None:
    """Compile the reference's hot-path sources (in place, read-only) into
    oracle/_ref/; None when no reference checkout is given or present."""
    ref_root = reference_root(root)
    if ref_root is None:
        return REF_LIB if REF_LIB.exists() else None
    subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF_ROOT={ref_root}"], check=True)
    return REF_LIB


def _f32(a):
    return np.asfortranarray(a, dtype=np.float32)


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def _dims(shape):
    arr = (C.c_int64 * 2)(int(shape[0]), int(shape[1]))
    return C.cast(arr, PD), arr


class Oracle:
    """CPU implementation of the D8 path: kind "port" or "ref"."""

    def __init__(self, kind: str = "port"):
        self.kind = kind
        path = PORT_LIB if kind == "port" else REF_LIB
        if not path.exists():
            if kind == "port":
                build_port()
            else:
                build_ref()
        if not path.exists():
            raise FileNotFoundError(path)
        self.lib = C.CDLL(str(path))
        pre = "orc_" if kind == "port" else ""
        D = C.c_double
        self._pre = pre
        sig = {
            "fillsinks": (None, [P, P, P, PD]),
            "fillsinks_hybrid": (C.c_int if kind == "port" else None, [P, P, P, P, PD]),
            "reconstruct": (None, [P, P, PD]),
            "reconstruct_hybrid": (C.c_int, [P, P, P, PD]),
            "identifyflats": (C.c_int64, [P, P, PD]),
            "gwdt_computecosts": (None, [P, P, P, P, P, PD]),
            "gwdt": (None, [P, P, P, P, P, P, PD]),
            "flow_routing_d8_carve": (None, [P, P, P, P, P, PD, C.c_uint]),
            "flow_accumulation": (None, [P, P, P, P, PD]),
            "hillshade_fused": (None, [P, P, F, F, F, PD]),
            "hillshade": (None, [P, P, P, P, F, F, F, PD]),
            "flow_routing_d8_edgelist": (C.c_int64, [P, P, P, P, PD, C.c_uint]),
            "flow_accumulation_edgelist": (None, [P, P, P, P, P, C.c_int64, PD]),
            "drainagebasins": (None, [P, P, P, C.c_int64, PD]),
            "edgelist_degree": (None, [P, P, P, P, C.c_int64, C.c_int64]),
            "traverse_down_f32_add_mul": (None, [P, P, P, P, C.c_int64]),
            "traverse_down_u32_or_and": (None, [P, P, P, P, C.c_int64]),
            "traverse_up_u32_or_and": (None, [P, P, P, P, C.c_int64]),
            "compute_sfgraph": (None, [P, P, P, P, P, P, P, P, D,
                                       C.c_int if kind == "port" else C.c_bool]),
            "compute_drainage_area_single_flow": (None, [P, P, P, P, D]),
            "compute_weighted_drainage_area_single_flow": (None, [P, P, P, P, P, D]),
        }
        if kind == "port":
            sig.update({
                "flow_accumulation_f64": (None, [P, P, P, P, PD]),
                "flow_accumulation_backward_f64": (None, [P, P, P, P, PD]),
                "flow_accumulation_f64w": (None, [P, P, P, P, PD]),
                "hillshade_f64": (None, [P, P, D, D, D, PD]),
                "hillshade_backward_f64": (None, [P, P, P, D, D, D, PD]),
                "flow_accumulation_edgelist_f64": (None, [P, P, P, P, P, C.c_int64, PD]),
                "traverse_down_f64_from_f32": (None, [P, P, P, P, C.c_int64]),
            })
        self.fn = {}
        for name, (res, args) in sig.items():
            f = getattr(self.lib, pre + name)
            f.restype = res
            f.argtypes = args
            self.fn[name] = f

    # The reference's fillsinks negates `dem` in place while it runs; every
    # wrapper passes a private copy so callers' arrays are never touched.
    def fillsinks(self, dem, bc):
        dem = np.array(dem, dtype=np.float32, order="F", copy=True)
        bc = np.asfortranarray(bc, dtype=np.uint8)
        out = np.empty_like(dem, order="F")
        dp, k = _dims(dem.shape)
        self.fn["fillsinks"](_ptr(out), _ptr(dem), _ptr(bc), dp)
        return out

    def fillsinks_hybrid(self, dem, bc):
        dem = np.array(dem, dtype=np.float32, order="F", copy=True)
        bc = np.asfortranarray(bc, dtype=np.uint8)
        out = np.empty_like(dem, order="F")
        q = np.empty(dem.shape, dtype=np.int64, order="F")
        dp, k = _dims(dem.shape)
        self.fn["fillsinks_hybrid"](_ptr(out), _ptr(q), _ptr(dem), _ptr(bc), dp)
        return out

    def reconstruct(self, marker, mask):
        """Reconstructed marker (src/reconstruct.c:270-278); inputs untouched."""
        mk = np.array(marker, dtype=np.float32, order="F", copy=True)
        mask = np.array(mask, dtype=np.float32, order="F", copy=True)
        dp, k = _dims(mk.shape)
        self.fn["reconstruct"](_ptr(mk), _ptr(mask), dp)
        return mk

    def reconstruct_hybrid(self, marker, mask):
        """(reconstructed marker, flag) of src/reconstruct.c:291-312."""
        mk = np.array(marker, dtype=np.float32, order="F", copy=True)
        mask = np.array(mask, dtype=np.float32, order="F", copy=True)
        q = np.empty(mk.shape, dtype=np.int64, order="F")
        dp, k = _dims(mk.shape)
        flag = self.fn["reconstruct_hybrid"](_ptr(mk), _ptr(q), _ptr(mask), dp)
        return mk, int(flag)

    def identifyflats(self, dem):
        dem = _f32(dem)
        out = np.empty(dem.shape, dtype=np.int32, order="F")
        dp, k = _dims(dem.shape)
        n = self.fn["identifyflats"](_ptr(out), _ptr(dem), dp)
        return out, int(n)

    def gwdt_computecosts(self, flats, dem, filled):
        flats = np.asfortranarray(flats, dtype=np.int32)
        dem, filled = _f32(dem), _f32(filled)
        costs = np.empty(dem.shape, dtype=np.float32, order="F")
        cc = np.empty(dem.shape, dtype=np.int64, order="F")
        dp, k = _dims(dem.shape)
        self.fn["gwdt_computecosts"](_ptr(costs), _ptr(cc), _ptr(flats), _ptr(dem),
                                     _ptr(filled), dp)
        return costs, cc

    def gwdt(self, costs, flats, want_prev=True):
        costs = _f32(costs)
        flats = np.asfortranarray(flats, dtype=np.int32)
        dist = np.empty(costs.shape, dtype=np.float32, order="F")
        prev = np.empty(costs.shape, dtype=np.int64, order="F") if want_prev else None
        heap = np.empty(costs.shape, dtype=np.int64, order="F")
        back = np.empty(costs.shape, dtype=np.int64, order="F")
        dp, k = _dims(costs.shape)
        self.fn["gwdt"](_ptr(dist), _ptr(prev), _ptr(costs), _ptr(flats), _ptr(heap),
                        _ptr(back), dp)
        return (dist, prev) if want_prev else dist

    def flow_routing_d8_carve(self, dem, dist, flats, order=0):
        dem, dist = _f32(dem), _f32(dist)
        flats = np.asfortranarray(flats, dtype=np.int32)
        node = np.empty(dem.shape, dtype=np.int64, order="F")
        direction = np.empty(dem.shape, dtype=np.uint8, order="F")
        dp, k = _dims(dem.shape)
        self.fn["flow_routing_d8_carve"](_ptr(node), _ptr(direction), _ptr(dem), _ptr(dist),
                                         _ptr(flats), dp, int(order))
        return node, direction

    def flow_accumulation(self, node, direction, weights=None):
        node = np.asfortranarray(node, dtype=np.int64)
        direction = np.asfortranarray(direction, dtype=np.uint8)
        w = _f32(weights) if weights is not None else None
        acc = np.empty(direction.shape, dtype=np.float32, order="F")
        dp, k = _dims(direction.shape)
        self.fn["flow_accumulation"](_ptr(acc), _ptr(node), _ptr(direction), _ptr(w), dp)
        return acc

    def flow_accumulation_f64(self, node, direction, weights=None):
        node = np.asfortranarray(node, dtype=np.int64)
        direction = np.asfortranarray(direction, dtype=np.uint8)
        w = _f32(weights) if weights is not None else None
        acc = np.empty(direction.shape, dtype=np.float64, order="F")
        dp, k = _dims(direction.shape)
        self.fn["flow_accumulation_f64"](_ptr(acc), _ptr(node), _ptr(direction), _ptr(w), dp)
        return acc

    def flow_accumulation_f64w(self, node, direction, weights64):
        node = np.asfortranarray(node, dtype=np.int64)
        direction = np.asfortranarray(direction, dtype=np.uint8)
        w = np.asfortranarray(weights64, dtype=np.float64)
        acc = np.empty(direction.shape, dtype=np.float64, order="F")
        dp, k = _dims(direction.shape)
        self.fn["flow_accumulation_f64w"](_ptr(acc), _ptr(node), _ptr(direction), _ptr(w), dp)
        return acc

    def flow_accumulation_backward_f64(self, node, direction, grad_acc):
        node = np.asfortranarray(node, dtype=np.int64)
        direction = np.asfortranarray(direction, dtype=np.uint8)
        g = np.asfortranarray(grad_acc, dtype=np.float64)
        out = np.empty(direction.shape, dtype=np.float64, order="F")
        dp, k = _dims(direction.shape)
        self.fn["flow_accumulation_backward_f64"](_ptr(out), _ptr(node), _ptr(direction),
                                                  _ptr(g), dp)
        return out

    def hillshade_fused(self, dem, az, alt, cs):
        dem = _f32(dem)
        out = np.empty_like(dem, order="F")
        dp, k = _dims(dem.shape)
        self.fn["hillshade_fused"](_ptr(out), _ptr(dem), float(az), float(alt), float(cs), dp)
        return out

    def hillshade(self, dem, az, alt, cs):
        dem = _f32(dem)
        out, dx, dy = (np.empty_like(dem, order="F") for _ in range(3))
        dp, k = _dims(dem.shape)
        self.fn["hillshade"](_ptr(out), _ptr(dx), _ptr(dy), _ptr(dem), float(az), float(alt),
                             float(cs), dp)
        return out, dx, dy

    def hillshade_f64(self, dem, az, alt, cs):
        dem = np.asfortranarray(dem, dtype=np.float64)
        out = np.empty(dem.shape, dtype=np.float64, order="F")
        dp, k = _dims(dem.shape)
        self.fn["hillshade_f64"](_ptr(out), _ptr(dem), float(az), float(alt), float(cs), dp)
        return out

    def hillshade_backward_f64(self, dem, grad_out, az, alt, cs):
        dem = np.asfortranarray(dem, dtype=np.float64)
        g = np.asfortranarray(grad_out, dtype=np.float64)
        out = np.empty(dem.shape, dtype=np.float64, order="F")
        dp, k = _dims(dem.shape)
        self.fn["hillshade_backward_f64"](_ptr(out), _ptr(dem), _ptr(g), float(az), float(alt),
                                          float(cs), dp)
        return out

    # ---- edge-list forms -------------------------------------------------
    def flow_routing_d8_edgelist(self, node, direction, order=0):
        node = np.asfortranarray(node, dtype=np.int64)
        direction = np.asfortranarray(direction, dtype=np.uint8)
        n = direction.size
        src = np.empty(n, dtype=np.int64)
        tgt = np.empty(n, dtype=np.int64)
        dp, k = _dims(direction.shape)
        e = self.fn["flow_routing_d8_edgelist"](_ptr(src), _ptr(tgt), _ptr(node),
                                                _ptr(direction), dp, int(order))
        return src[:e].copy(), tgt[:e].copy()

    def flow_accumulation_edgelist(self, source, target, fraction, shape, weights=None,
                                   f64=False):
        src = np.ascontiguousarray(source, dtype=np.int64)
        tgt = np.ascontiguousarray(target, dtype=np.int64)
        fr = np.ascontiguousarray(fraction, dtype=np.float32)
        w = _f32(weights) if weights is not None else None
        acc = np.empty(shape, dtype=np.float64 if f64 else np.float32, order="F")
        dp, k = _dims(shape)
        name = "flow_accumulation_edgelist_f64" if f64 else "flow_accumulation_edgelist"
        self.fn[name](_ptr(acc), _ptr(src), _ptr(tgt), _ptr(fr), _ptr(w), len(src), dp)
        return acc

    def drainagebasins(self, source, target, shape):
        src = np.ascontiguousarray(source, dtype=np.int64)
        tgt = np.ascontiguousarray(target, dtype=np.int64)
        out = np.empty(shape, dtype=np.int64, order="F")
        dp, k = _dims(shape)
        self.fn["drainagebasins"](_ptr(out), _ptr(src), _ptr(tgt), len(src), dp)
        return out

    def traverse_down_f32_add_mul(self, output, input, source, target, f64=False):
        """Updated copy of `output` (src/streamquad.c:171-180); with f64 the
        same sweep in FP64 (port only)."""
        out = np.array(output, dtype=np.float64 if f64 else np.float32, copy=True)
        inp = np.ascontiguousarray(input, dtype=np.float32)
        src = np.ascontiguousarray(source, dtype=np.int64)
        tgt = np.ascontiguousarray(target, dtype=np.int64)
        name = "traverse_down_f64_from_f32" if f64 else "traverse_down_f32_add_mul"
        self.fn[name](_ptr(out), _ptr(inp), _ptr(src), _ptr(tgt), len(src))
        return out

    def traverse_u32_or_and(self, output, input, source, target, up=False):
        """Updated copy of `output` (src/streamquad.c:37-60): the or/and
        sweep down the list, or up it (reverse order, source and target
        exchanged) with `up`."""
        out = np.array(output, dtype=np.uint32, copy=True)
        inp = np.ascontiguousarray(input, dtype=np.uint32)
        src = np.ascontiguousarray(source, dtype=np.int64)
        tgt = np.ascontiguousarray(target, dtype=np.int64)
        name = "traverse_up_u32_or_and" if up else "traverse_down_u32_or_and"
        self.fn[name](_ptr(out), _ptr(inp), _ptr(src), _ptr(tgt), len(src))
        return out

    def edgelist_degree(self, source, target, node_count):
        src = np.ascontiguousarray(source, dtype=np.int64)
        tgt = np.ascontiguousarray(target, dtype=np.int64)
        indeg = np.empty(node_count, dtype=np.uint8)
        outdeg = np.empty(node_count, dtype=np.uint8)
        self.fn["edgelist_degree"](_ptr(indeg), _ptr(outdeg), _ptr(src), _ptr(tgt),
                                   int(node_count), len(src))
        return indeg, outdeg

    # ---- graphflood single-flow graph (row-major, C-ordered arrays) -------
    def compute_sfgraph(self, topo, bcs, dx, d8=True):
        topo = np.ascontiguousarray(topo, dtype=np.float64)
        bcs = np.ascontiguousarray(bcs, dtype=np.uint8)
        n = topo.size
        k = 8 if d8 else 4
        rcv = np.empty(n, dtype=np.uint64)
        dist = np.empty(n, dtype=np.float64)
        don = np.zeros(n * k, dtype=np.uint64)
        ndon = np.empty(n, dtype=np.uint8)
        stack = np.empty(n, dtype=np.uint64)
        dim = (C.c_size_t * 2)(*topo.shape)
        self.fn["compute_sfgraph"](_ptr(topo), _ptr(rcv), _ptr(dist), _ptr(don), _ptr(ndon),
                                   _ptr(stack), _ptr(bcs), C.cast(dim, P), float(dx),
                                   bool(d8))
        return rcv, dist, don.reshape(n, k), ndon, stack

    def compute_drainage_area_single_flow(self, rcv, stack, shape, dx, weights=None):
        rcv = np.ascontiguousarray(rcv, dtype=np.uint64)
        stack = np.ascontiguousarray(stack, dtype=np.uint64)
        out = np.empty(int(np.prod(shape)), dtype=np.float64)
        dim = (C.c_size_t * 2)(*shape)
        if weights is None:
            self.fn["compute_drainage_area_single_flow"](_ptr(out), _ptr(rcv), _ptr(stack),
                                                         C.cast(dim, P), float(dx))
        else:
            w = np.ascontiguousarray(weights, dtype=np.float64).ravel()
            self.fn["compute_weighted_drainage_area_single_flow"](
                _ptr(out), _ptr(w), _ptr(rcv), _ptr(stack), C.cast(dim, P), float(dx))
        return out.reshape(shape)

    def run_pipeline(self, dem, bc, hillshade=None):
        """The pipeline of `pipeline` (hybrid fill) for timing: every
        intermediate is dropped as soon as the next stage has read it, so a
        16384 x 16384 run peaks near 35 bytes per pixel.  `hillshade`
        (azimuth, altitude, cellsize) adds hillshade_fused of `dem`.
        Returns the accumulation."""
        filled = self.fillsinks_hybrid(dem, bc)
        flats, _ = self.identifyflats(filled)
        costs, cc = self.gwdt_computecosts(flats, dem, filled)
        del cc
        dist = self.gwdt(costs, flats, want_prev=False)
        del costs
        node, direction = self.flow_routing_d8_carve(filled, dist, flats, 0)
        del filled, dist, flats
        acc = self.flow_accumulation(node, direction)
        del node, direction
        if hillshade is not None:
            self.hillshade_fused(dem, *hillshade)
        return acc

    def pipeline(self, dem, bc, weights=None, hybrid=True):
        """fill -> flats -> costs -> gwdt -> carve -> accumulation, the call
        sequence of test/random_dem.cpp:682-724 (with flow_accumulation)."""
        filled = self.fillsinks_hybrid(dem, bc) if hybrid else self.fillsinks(dem, bc)
        flats, _ = self.identifyflats(filled)
        costs, cc = self.gwdt_computecosts(flats, dem, filled)
        dist = self.gwdt(costs, flats, want_prev=False)
        node, direction = self.flow_routing_d8_carve(filled, dist, flats, 0)
        acc = self.flow_accumulation(node, direction, weights)
        return dict(filled=filled, flats=flats, costs=costs, conncomps=cc, dist=dist,
                    node=node, direction=direction, acc=acc)
