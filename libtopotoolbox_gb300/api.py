"""Reference-named Python API over the native C ABI.

Host functions take numpy grids of shape (nrows, ncols); they are made
Fortran-contiguous (column-major, the layout of include/topotoolbox.h) and
passed through the drop-in host-pointer entry points ``tt_cuda_<name>``,
which have exactly the parameter lists of the reference functions.  Outputs
are allocated here and returned.  After every call the per-thread status is
checked and a ``TTCudaError`` is raised on failure.

``dev`` holds the device-pointer forms for torch CUDA tensors.  A grid with
dims (nrows, ncols) in column-major order is a contiguous torch tensor of
shape (ncols, nrows); ``dev`` functions take and return such tensors and run
on torch's current CUDA stream.
"""
from __future__ import annotations

import contextlib
import ctypes as C

import numpy as np

from . import _native as N


def _f32(a):
    return np.asfortranarray(a, dtype=np.float32)


def _u8(a):
    return np.asfortranarray(a, dtype=np.uint8)


def _i32(a):
    return np.asfortranarray(a, dtype=np.int32)


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def _dims(a):
    if a.ndim != 2:
        raise ValueError("grids are 2-D (nrows, ncols)")
    return (a.shape[0], a.shape[1])


def _after(where):
    s = N.last_status()
    N.check(s, where)


def has_gpu() -> bool:
    return bool(N.lib().tt_cuda_has_gpu())


def last_rounds() -> int:
    return int(N.lib().tt_cuda_last_rounds())


def launch_count(reset: bool = False) -> int:
    return int(N.lib().tt_cuda_launch_count(1 if reset else 0))


# ---------------------------------------------------------------------------
# Host-pointer (drop-in) functions
# ---------------------------------------------------------------------------

def fillsinks(dem, bc):
    """Filled DEM (include/topotoolbox.h:293, src/fillsinks.c:23-48)."""
    dem, bc = _f32(dem), _u8(bc)
    out = np.empty_like(dem, order="F")
    dp, keep = N.dims_arg(_dims(dem))
    N.lib().tt_cuda_fillsinks(_ptr(out), _ptr(dem), _ptr(bc), dp)
    _after("fillsinks")
    return out


def fillsinks_hybrid(dem, bc):
    """Same result as fillsinks (include/topotoolbox.h:351)."""
    dem, bc = _f32(dem), _u8(bc)
    out = np.empty_like(dem, order="F")
    dp, keep = N.dims_arg(_dims(dem))
    N.lib().tt_cuda_fillsinks_hybrid(_ptr(out), None, _ptr(dem), _ptr(bc), dp)
    _after("fillsinks_hybrid")
    return out


def reconstruct(marker, mask):
    """Grayscale reconstruction (include/topotoolbox.h:1056).  Returns the
    reconstructed marker (the input is not modified)."""
    mk = np.array(marker, dtype=np.float32, order="F", copy=True)
    mask = _f32(mask)
    dp, keep = N.dims_arg(_dims(mask))
    N.lib().tt_cuda_reconstruct(_ptr(mk), _ptr(mask), dp)
    _after("reconstruct")
    return mk


def reconstruct_hybrid(marker, mask):
    """(reconstructed marker, flag) of include/topotoolbox.h:1070; the flag
    is 1 when the reconstruction did not converge (the input is not
    modified)."""
    mk = np.array(marker, dtype=np.float32, order="F", copy=True)
    mask = _f32(mask)
    dp, keep = N.dims_arg(_dims(mask))
    flag = N.lib().tt_cuda_reconstruct_hybrid(_ptr(mk), None, _ptr(mask), dp)
    _after("reconstruct_hybrid")
    return mk, int(flag)


def identifyflats(dem):
    """(flags, count): bit 0 flat, bit 1 sill, bit 2 presill
    (include/topotoolbox.h:405, src/identifyflats.c:33-121)."""
    dem = _f32(dem)
    out = np.empty(dem.shape, dtype=np.int32, order="F")
    dp, keep = N.dims_arg(_dims(dem))
    cnt = N.lib().tt_cuda_identifyflats(_ptr(out), _ptr(dem), dp)
    _after("identifyflats")
    return out, int(cnt)


def gwdt_computecosts(flats, original_dem, filled_dem):
    """(costs, conncomps) (include/topotoolbox.h:464, src/gwdt.c:167-278)."""
    flats, orig, filled = _i32(flats), _f32(original_dem), _f32(filled_dem)
    costs = np.empty(orig.shape, dtype=np.float32, order="F")
    cc = np.empty(orig.shape, dtype=np.int64, order="F")
    dp, keep = N.dims_arg(_dims(orig))
    N.lib().tt_cuda_gwdt_computecosts(_ptr(costs), _ptr(cc), _ptr(flats), _ptr(orig),
                                      _ptr(filled), dp)
    _after("gwdt_computecosts")
    return costs, cc


def gwdt(costs, flats, want_prev=False):
    """dist (and prev) (include/topotoolbox.h:533, src/gwdt.c:290-351)."""
    costs, flats = _f32(costs), _i32(flats)
    dist = np.empty(costs.shape, dtype=np.float32, order="F")
    prev = np.empty(costs.shape, dtype=np.int64, order="F") if want_prev else None
    dp, keep = N.dims_arg(_dims(costs))
    N.lib().tt_cuda_gwdt(_ptr(dist), _ptr(prev), _ptr(costs), _ptr(flats), None, None, dp)
    _after("gwdt")
    return (dist, prev) if want_prev else dist


def flow_routing_d8_carve(dem, dist, flats, order=0):
    """(node, direction) (include/topotoolbox.h:860,
    src/flow_routing.c:135-256).  For order=1 the arrays are row-major with
    dims = (ncols, nrows): pass them transposed as C-ordered data."""
    dem, dist, flats = _f32(dem), _f32(dist), _i32(flats)
    node = np.empty(dem.shape, dtype=np.int64, order="F")
    direction = np.empty(dem.shape, dtype=np.uint8, order="F")
    dp, keep = N.dims_arg(_dims(dem))
    N.lib().tt_cuda_flow_routing_d8_carve(_ptr(node), _ptr(direction), _ptr(dem), _ptr(dist),
                                          _ptr(flats), dp, int(order))
    _after("flow_routing_d8_carve")
    return node, direction


def flow_accumulation(direction, weights=None, node=None):
    """acc (include/topotoolbox.h:962, src/flow_accumulation.c:32-80)."""
    direction = _u8(direction)
    w = _f32(weights) if weights is not None else None
    acc = np.empty(direction.shape, dtype=np.float32, order="F")
    nd = np.asfortranarray(node, dtype=np.int64) if node is not None else None
    dp, keep = N.dims_arg(_dims(direction))
    N.lib().tt_cuda_flow_accumulation(_ptr(acc), _ptr(nd), _ptr(direction), _ptr(w), dp)
    _after("flow_accumulation")
    return acc


def flow_accumulation_backward(direction, grad_acc):
    """grad_weights: sum of grad_acc along each pixel's path to its outlet."""
    direction, g = _u8(direction), _f32(grad_acc)
    out = np.empty(direction.shape, dtype=np.float32, order="F")
    dp, keep = N.dims_arg(_dims(direction))
    N.lib().tt_cuda_flow_accumulation_backward(_ptr(out), None, _ptr(direction), _ptr(g), dp)
    _after("flow_accumulation_backward")
    return out


def gradient_secondorder(dem, cellsize):
    """(p0, p1) (include/topotoolbox.h:2347, src/hillshade.c:23-76)."""
    dem = _f32(dem)
    p0 = np.empty_like(dem, order="F")
    p1 = np.empty_like(dem, order="F")
    dp, keep = N.dims_arg(_dims(dem))
    N.lib().tt_cuda_gradient_secondorder(_ptr(p0), _ptr(p1), _ptr(dem), float(cellsize), dp)
    _after("gradient_secondorder")
    return p0, p1


def hillshade(dem, azimuth, altitude, cellsize):
    """(output, dx, dy) (include/topotoolbox.h:2400, src/hillshade.c:79-97)."""
    dem = _f32(dem)
    out, dx, dy = (np.empty_like(dem, order="F") for _ in range(3))
    dp, keep = N.dims_arg(_dims(dem))
    N.lib().tt_cuda_hillshade(_ptr(out), _ptr(dx), _ptr(dy), _ptr(dem), float(azimuth),
                              float(altitude), float(cellsize), dp)
    _after("hillshade")
    return out, dx, dy


def hillshade_fused(dem, azimuth, altitude, cellsize):
    """output (include/topotoolbox.h:2449, src/hillshade.c:102-213)."""
    dem = _f32(dem)
    out = np.empty_like(dem, order="F")
    dp, keep = N.dims_arg(_dims(dem))
    N.lib().tt_cuda_hillshade_fused(_ptr(out), _ptr(dem), float(azimuth), float(altitude),
                                    float(cellsize), dp)
    _after("hillshade_fused")
    return out


def hillshade_backward(dem, grad_output, azimuth, altitude, cellsize):
    """grad_dem = J^T grad_output for hillshade_fused."""
    dem, g = _f32(dem), _f32(grad_output)
    out = np.empty_like(dem, order="F")
    dp, keep = N.dims_arg(_dims(dem))
    N.lib().tt_cuda_hillshade_backward(_ptr(out), _ptr(dem), _ptr(g), float(azimuth),
                                       float(altitude), float(cellsize), dp)
    _after("hillshade_backward")
    return out


def flow_routing_d8_edgelist(node, direction, order=0):
    """(source, target) (include/topotoolbox.h:912, src/flow_routing.c:258-312):
    one edge per pixel with a direction, in `node` order."""
    node = np.asfortranarray(node, dtype=np.int64)
    direction = _u8(direction)
    src = np.empty(direction.size, dtype=np.int64)
    tgt = np.empty(direction.size, dtype=np.int64)
    dp, keep = N.dims_arg(_dims(direction))
    e = N.lib().tt_cuda_flow_routing_d8_edgelist(_ptr(src), _ptr(tgt), _ptr(node),
                                                 _ptr(direction), dp, int(order))
    _after("flow_routing_d8_edgelist")
    return src[:e].copy(), tgt[:e].copy()


def flow_accumulation_edgelist(source, target, fraction, shape, weights=None):
    """acc (include/topotoolbox.h:1019, src/flow_accumulation.c:10-30) for any
    edge list: fractions, several edges out of a pixel, any order."""
    src = np.ascontiguousarray(source, dtype=np.int64)
    tgt = np.ascontiguousarray(target, dtype=np.int64)
    fr = np.ascontiguousarray(fraction, dtype=np.float32)
    w = _f32(weights) if weights is not None else None
    acc = np.empty(shape, dtype=np.float32, order="F")
    dp, keep = N.dims_arg(tuple(shape))
    N.lib().tt_cuda_flow_accumulation_edgelist(_ptr(acc), _ptr(src), _ptr(tgt), _ptr(fr),
                                               _ptr(w), len(src), dp)
    _after("flow_accumulation_edgelist")
    return acc


def traverse_down_f32_add_mul(output, input, source, target):
    """output[target] += output[source] * input[e] for every edge in list
    order (include/topotoolbox.h:1755, src/streamquad.c:171-180).  Returns
    the updated copy of `output` (float32 node attribute list)."""
    out = np.array(output, dtype=np.float32, copy=True)
    inp = np.ascontiguousarray(input, dtype=np.float32)
    src = np.ascontiguousarray(source, dtype=np.int64)
    tgt = np.ascontiguousarray(target, dtype=np.int64)
    N.lib().tt_cuda_traverse_down_f32_add_mul(_ptr(out), _ptr(inp), _ptr(src), _ptr(tgt),
                                              len(src))
    _after("traverse_down_f32_add_mul")
    return out


def traverse_down_u32_or_and(output, input, source, target):
    """output[target] |= output[source] & input[e] for every edge in list
    order (include/topotoolbox.h:1235, src/streamquad.c:49-60).  Returns the
    updated copy of `output` (uint32 node attribute list)."""
    return _traverse_u32("tt_cuda_traverse_down_u32_or_and", output, input, source, target)


def traverse_up_u32_or_and(output, weights, source, target):
    """output[source] |= output[target] & weights[e] for every edge in
    reverse list order (include/topotoolbox.h:1186, src/streamquad.c:37-47).
    Returns the updated copy of `output` (uint32 node attribute list)."""
    return _traverse_u32("tt_cuda_traverse_up_u32_or_and", output, weights, source, target)


def _traverse_u32(name, output, input, source, target):
    out = np.array(output, dtype=np.uint32, copy=True)
    inp = np.ascontiguousarray(input, dtype=np.uint32)
    src = np.ascontiguousarray(source, dtype=np.int64)
    tgt = np.ascontiguousarray(target, dtype=np.int64)
    getattr(N.lib(), name)(_ptr(out), _ptr(inp), _ptr(src), _ptr(tgt), len(src))
    _after(name[len("tt_cuda_"):])
    return out


def drainagebasins(source, target, shape):
    """basins (include/topotoolbox.h:2304, src/drainagebasins.c:6-27)."""
    src = np.ascontiguousarray(source, dtype=np.int64)
    tgt = np.ascontiguousarray(target, dtype=np.int64)
    out = np.empty(shape, dtype=np.int64, order="F")
    dp, keep = N.dims_arg(tuple(shape))
    N.lib().tt_cuda_drainagebasins(_ptr(out), _ptr(src), _ptr(tgt), len(src), dp)
    _after("drainagebasins")
    return out


def edgelist_degree(source, target, node_count):
    """(indegree, outdegree) (include/topotoolbox.h:1853, src/streamquad.c:209-224)."""
    src = np.ascontiguousarray(source, dtype=np.int64)
    tgt = np.ascontiguousarray(target, dtype=np.int64)
    indeg = np.empty(node_count, dtype=np.uint8)
    outdeg = np.empty(node_count, dtype=np.uint8)
    N.lib().tt_cuda_edgelist_degree(_ptr(indeg), _ptr(outdeg), _ptr(src), _ptr(tgt),
                                    int(node_count), len(src))
    _after("edgelist_degree")
    return indeg, outdeg


def compute_sfgraph(topo, bcs, dx, d8=True):
    """Graphflood single-flow graph (include/topotoolbox.h:2053,
    src/graphflood/sfgraph.c:27-113) of a row-major (rows, cols) float64
    grid: (receivers, distances, donors (N, 8|4), donor counts, stack)."""
    topo = np.ascontiguousarray(topo, dtype=np.float64)
    bcs = np.ascontiguousarray(bcs, dtype=np.uint8)
    n, k = topo.size, (8 if d8 else 4)
    rcv = np.empty(n, np.uint64)
    dist = np.empty(n, np.float64)
    don = np.zeros(n * k, np.uint64)
    ndon = np.empty(n, np.uint8)
    stack = np.empty(n, np.uint64)
    dim = (N.C.c_size_t * 2)(*topo.shape)
    N.lib().tt_cuda_compute_sfgraph(_ptr(topo), _ptr(rcv), _ptr(dist), _ptr(don), _ptr(ndon),
                                    _ptr(stack), _ptr(bcs), N.C.cast(dim, N.C.c_void_p),
                                    float(dx), bool(d8))
    _after("compute_sfgraph")
    return rcv, dist, don.reshape(n, k), ndon, stack


def compute_drainage_area_single_flow(receivers, shape, dx, stack=None):
    """Drainage area (include/topotoolbox.h:2122, src/graphflood/gf_flowacc.c:19-35)."""
    rcv = np.ascontiguousarray(receivers, dtype=np.uint64)
    out = np.empty(int(np.prod(shape)), np.float64)
    dim = (N.C.c_size_t * 2)(*shape)
    st = np.ascontiguousarray(stack, dtype=np.uint64) if stack is not None else None
    N.lib().tt_cuda_compute_drainage_area_single_flow(_ptr(out), _ptr(rcv), _ptr(st),
                                                      N.C.cast(dim, N.C.c_void_p), float(dx))
    _after("compute_drainage_area_single_flow")
    return out.reshape(shape)


def d8_pipeline(dem, bc, weights=None):
    """The reference call sequence fill -> flats -> costs -> gwdt -> carve ->
    accumulation in one call (host buffers).  Returns a dict."""
    dem, bc = _f32(dem), _u8(bc)
    shape = dem.shape
    w = _f32(weights) if weights is not None else None
    out = {
        "filled": np.empty(shape, np.float32, order="F"),
        "flats": np.empty(shape, np.int32, order="F"),
        "dist": np.empty(shape, np.float32, order="F"),
        "node": np.empty(shape, np.int64, order="F"),
        "direction": np.empty(shape, np.uint8, order="F"),
        "acc": np.empty(shape, np.float32, order="F"),
    }
    dp, keep = N.dims_arg(_dims(dem))
    N.lib().tt_cuda_d8_pipeline(_ptr(out["filled"]), _ptr(out["flats"]), _ptr(out["dist"]),
                                _ptr(out["node"]), _ptr(out["direction"]), _ptr(out["acc"]),
                                _ptr(dem), _ptr(bc), _ptr(w), dp)
    _after("d8_pipeline")
    return out


# ---------------------------------------------------------------------------
# Device-pointer functions on torch CUDA tensors
# ---------------------------------------------------------------------------

class dev:  # namespace
    """Device forms.  Tensors are column-major grids: shape (ncols, nrows)."""

    @staticmethod
    def _stream():
        import torch

        return C.c_void_p(torch.cuda.current_stream().cuda_stream)

    @staticmethod
    def _dims(t):
        return (t.shape[1], t.shape[0])

    @staticmethod
    @contextlib.contextmanager
    def deferred():
        """Defers the status checks of the D8 path's device calls in the block
        (tt_cuda_defer_begin / tt_cuda_defer_end): they only enqueue their
        work on torch's current stream, which must stay the same in the
        block.  Leaving the block synchronises the stream once and raises
        ``TTCudaError`` for the first failure any call recorded."""
        N.check(N.lib().tt_cuda_defer_begin(dev._stream()), "defer_begin")
        try:
            yield
        except BaseException:
            N.lib().tt_cuda_defer_end()
            raise
        N.check(N.lib().tt_cuda_defer_end(), "defer_end")

    @staticmethod
    def _p(t):
        if t is None:
            return None
        if not t.is_cuda or not t.is_contiguous():
            raise ValueError("device functions take contiguous CUDA tensors")
        return C.c_void_p(t.data_ptr())

    @staticmethod
    def fillsinks(dem, bc, out=None):
        import torch

        out = torch.empty_like(dem) if out is None else out
        dp, keep = N.dims_arg(dev._dims(dem))
        N.check(N.lib().tt_cuda_fillsinks_dev(dev._p(out), dev._p(dem), dev._p(bc), dp,
                                              dev._stream()), "fillsinks_dev")
        return out

    @staticmethod
    def reconstruct(marker, mask):
        """Reconstructs `marker` under `mask` in place and returns it."""
        dp, keep = N.dims_arg(dev._dims(mask))
        N.check(N.lib().tt_cuda_reconstruct_dev(dev._p(marker), dev._p(mask), dp,
                                                dev._stream()), "reconstruct_dev")
        return marker

    @staticmethod
    def identifyflats(dem, out=None):
        import torch

        out = torch.empty(dem.shape, dtype=torch.int32, device=dem.device) if out is None else out
        dp, keep = N.dims_arg(dev._dims(dem))
        N.check(N.lib().tt_cuda_identifyflats_dev(dev._p(out), dev._p(dem), dp, None,
                                                  dev._stream()), "identifyflats_dev")
        return out

    @staticmethod
    def gwdt_computecosts(flats, dem, filled):
        import torch

        costs = torch.empty(dem.shape, dtype=torch.float32, device=dem.device)
        cc = torch.empty(dem.shape, dtype=torch.int64, device=dem.device)
        dp, keep = N.dims_arg(dev._dims(dem))
        N.check(N.lib().tt_cuda_gwdt_computecosts_dev(dev._p(costs), dev._p(cc), dev._p(flats),
                                                      dev._p(dem), dev._p(filled), dp,
                                                      dev._stream()), "gwdt_computecosts_dev")
        return costs, cc

    @staticmethod
    def gwdt(costs, flats, prev=None):
        import torch

        dist = torch.empty_like(costs)
        dp, keep = N.dims_arg(dev._dims(costs))
        N.check(N.lib().tt_cuda_gwdt_dev(dev._p(dist), dev._p(prev), dev._p(costs), dev._p(flats),
                                         dp, dev._stream()), "gwdt_dev")
        return dist

    @staticmethod
    def flow_routing_d8_carve(dem, dist, flats, order=0, want_node=True):
        import torch

        direction = torch.empty(dem.shape, dtype=torch.uint8, device=dem.device)
        node = torch.empty(dem.shape, dtype=torch.int64, device=dem.device) if want_node else None
        dp, keep = N.dims_arg(dev._dims(dem))
        N.check(N.lib().tt_cuda_flow_routing_d8_carve_dev(dev._p(node), dev._p(direction),
                                                          dev._p(dem), dev._p(dist),
                                                          dev._p(flats), dp, int(order),
                                                          dev._stream()),
                "flow_routing_d8_carve_dev")
        return node, direction

    @staticmethod
    def flow_accumulation(direction, weights=None, out=None):
        import torch

        out = torch.empty(direction.shape, dtype=torch.float32,
                          device=direction.device) if out is None else out
        dp, keep = N.dims_arg(dev._dims(direction))
        N.check(N.lib().tt_cuda_flow_accumulation_dev(dev._p(out), dev._p(direction),
                                                      dev._p(weights), dp, dev._stream()),
                "flow_accumulation_dev")
        return out

    @staticmethod
    def flow_routing_d8_edgelist(node, direction, order=0):
        """Returns (source, target) CUDA tensors trimmed to the edge count."""
        import torch

        n = direction.numel()
        src = torch.empty(n, dtype=torch.int64, device=direction.device)
        tgt = torch.empty(n, dtype=torch.int64, device=direction.device)
        cnt = N.C.c_int64(0)
        dp, keep = N.dims_arg(dev._dims(direction))
        N.check(N.lib().tt_cuda_flow_routing_d8_edgelist_dev(
            dev._p(src), dev._p(tgt), N.C.byref(cnt), dev._p(node), dev._p(direction), dp,
            int(order), dev._stream()), "flow_routing_d8_edgelist_dev")
        return src[:cnt.value], tgt[:cnt.value]

    @staticmethod
    def flow_accumulation_edgelist(source, target, fraction, like, weights=None, out=None):
        import torch

        out = torch.empty(like.shape, dtype=torch.float32, device=like.device) \
            if out is None else out
        dp, keep = N.dims_arg(dev._dims(like))
        N.check(N.lib().tt_cuda_flow_accumulation_edgelist_dev(
            dev._p(out), dev._p(source), dev._p(target), dev._p(fraction), dev._p(weights),
            int(source.numel()), dp, dev._stream()), "flow_accumulation_edgelist_dev")
        return out

    @staticmethod
    def traverse_down_f32_add_mul(output, input, source, target):
        """In place on the 1-D float32 tensor `output`; returns it."""
        N.check(N.lib().tt_cuda_traverse_down_f32_add_mul_dev(
            dev._p(output), dev._p(input), dev._p(source), dev._p(target),
            int(source.numel()), int(output.numel()), dev._stream()),
            "traverse_down_f32_add_mul_dev")
        return output

    @staticmethod
    def traverse_u32_or_and(output, input, source, target, up=False):
        """traverse_down_u32_or_and, or traverse_up_u32_or_and with `up`, in
        place on the 1-D 32-bit tensor `output` (int32 tensors carry the
        uint32 words bit for bit); returns it."""
        name = "tt_cuda_traverse_up_u32_or_and_dev" if up else \
            "tt_cuda_traverse_down_u32_or_and_dev"
        N.check(getattr(N.lib(), name)(
            dev._p(output), dev._p(input), dev._p(source), dev._p(target),
            int(source.numel()), int(output.numel()), dev._stream()), name[len("tt_cuda_"):])
        return output

    @staticmethod
    def drainagebasins(source, target, like, out=None):
        import torch

        out = torch.empty(like.shape, dtype=torch.int64, device=like.device) \
            if out is None else out
        dp, keep = N.dims_arg(dev._dims(like))
        N.check(N.lib().tt_cuda_drainagebasins_dev(dev._p(out), dev._p(source), dev._p(target),
                                                   int(source.numel()), dp, dev._stream()),
                "drainagebasins_dev")
        return out

    @staticmethod
    def flow_accumulation_backward(direction, grad_acc, out=None):
        import torch

        out = torch.empty(direction.shape, dtype=torch.float32,
                          device=direction.device) if out is None else out
        dp, keep = N.dims_arg(dev._dims(direction))
        N.check(N.lib().tt_cuda_flow_accumulation_backward_dev(dev._p(out), dev._p(direction),
                                                               dev._p(grad_acc), dp,
                                                               dev._stream()),
                "flow_accumulation_backward_dev")
        return out

    @staticmethod
    def hillshade_fused(dem, azimuth, altitude, cellsize, out=None):
        import torch

        out = torch.empty_like(dem) if out is None else out
        dp, keep = N.dims_arg(dev._dims(dem))
        N.check(N.lib().tt_cuda_hillshade_fused_dev(dev._p(out), dev._p(dem), float(azimuth),
                                                    float(altitude), float(cellsize), dp,
                                                    dev._stream()), "hillshade_fused_dev")
        return out

    @staticmethod
    def hillshade_backward(dem, grad_output, azimuth, altitude, cellsize, out=None):
        import torch

        out = torch.empty_like(dem) if out is None else out
        dp, keep = N.dims_arg(dev._dims(dem))
        N.check(N.lib().tt_cuda_hillshade_backward_dev(dev._p(out), dev._p(dem),
                                                       dev._p(grad_output), float(azimuth),
                                                       float(altitude), float(cellsize), dp,
                                                       dev._stream()), "hillshade_backward_dev")
        return out

    @staticmethod
    def d8_pipeline(dem, bc, weights=None, outputs=None, hillshade_angles=None, cellsize=1.0):
        """Whole pipeline on device tensors.  `outputs` is a dict of
        preallocated tensors (filled, flats, dist, node, direction, acc,
        hillshade); missing entries are allocated."""
        import torch

        o = dict(outputs or {})
        shp, d = dem.shape, dem.device
        o.setdefault("filled", torch.empty(shp, dtype=torch.float32, device=d))
        o.setdefault("flats", torch.empty(shp, dtype=torch.int32, device=d))
        o.setdefault("dist", torch.empty(shp, dtype=torch.float32, device=d))
        o.setdefault("node", torch.empty(shp, dtype=torch.int64, device=d))
        o.setdefault("direction", torch.empty(shp, dtype=torch.uint8, device=d))
        o.setdefault("acc", torch.empty(shp, dtype=torch.float32, device=d))
        az, alt = (hillshade_angles or (0.0, 0.0))
        if hillshade_angles is not None:
            o.setdefault("hillshade", torch.empty(shp, dtype=torch.float32, device=d))
        hs = o.get("hillshade") if hillshade_angles is not None else None
        dp, keep = N.dims_arg(dev._dims(dem))
        N.check(N.lib().tt_cuda_d8_pipeline_dev(dev._p(o["filled"]), dev._p(o["flats"]),
                                                dev._p(o["dist"]), dev._p(o["node"]),
                                                dev._p(o["direction"]), dev._p(o["acc"]),
                                                dev._p(hs), dev._p(dem), dev._p(bc),
                                                dev._p(weights), float(az), float(alt),
                                                float(cellsize), dp, dev._stream()),
                "d8_pipeline_dev")
        return o
