"""ctypes binding of the native library ``libtt_cuda.so`` (include/tt_cuda.h).

The library is loaded from this package directory.  There is no fallback:
if it is missing or cannot be loaded, ``lib()`` raises, so every compute
entry point of this package fails loudly instead of running elsewhere.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libtt_cuda.so"

P = C.c_void_p
F = C.c_float
I64 = C.c_int64
PD = C.POINTER(C.c_int64)  # ptrdiff_t dims[2]
U = C.c_uint
ST = C.c_int  # tt_cuda_status

# name -> (restype, argtypes), mirroring include/tt_cuda.h
SIGNATURES = {
    "tt_cuda_has_gpu": (C.c_int, []),
    "tt_cuda_last_error": (ST, []),
    "tt_cuda_status_string": (C.c_char_p, [ST]),
    "tt_cuda_set_max_rounds": (None, [I64]),
    "tt_cuda_release_workspace": (None, []),
    "tt_cuda_launch_count": (I64, [C.c_int]),
    "tt_cuda_last_rounds": (I64, []),
    "tt_cuda_set_relax_schedule": (None, [C.c_int]),
    "tt_cuda_defer_begin": (ST, [P]),
    "tt_cuda_defer_end": (ST, []),
    # drop-in host-pointer forms
    "tt_cuda_fillsinks": (None, [P, P, P, PD]),
    "tt_cuda_fillsinks_hybrid": (None, [P, P, P, P, PD]),
    "tt_cuda_reconstruct": (None, [P, P, PD]),
    "tt_cuda_reconstruct_hybrid": (C.c_int, [P, P, P, PD]),
    "tt_cuda_identifyflats": (C.c_int64, [P, P, PD]),
    "tt_cuda_gwdt_computecosts": (None, [P, P, P, P, P, PD]),
    "tt_cuda_gwdt": (None, [P, P, P, P, P, P, PD]),
    "tt_cuda_flow_routing_d8_carve": (None, [P, P, P, P, P, PD, U]),
    "tt_cuda_flow_accumulation": (None, [P, P, P, P, PD]),
    "tt_cuda_gradient_secondorder": (None, [P, P, P, F, PD]),
    "tt_cuda_hillshade": (None, [P, P, P, P, F, F, F, PD]),
    "tt_cuda_hillshade_fused": (None, [P, P, F, F, F, PD]),
    "tt_cuda_flow_accumulation_backward": (None, [P, P, P, P, PD]),
    "tt_cuda_hillshade_backward": (None, [P, P, P, F, F, F, PD]),
    "tt_cuda_d8_pipeline": (None, [P, P, P, P, P, P, P, P, P, PD]),
    "tt_cuda_flow_routing_d8_edgelist": (I64, [P, P, P, P, PD, U]),
    "tt_cuda_flow_accumulation_edgelist": (None, [P, P, P, P, P, I64, PD]),
    "tt_cuda_drainagebasins": (None, [P, P, P, I64, PD]),
    "tt_cuda_traverse_down_f32_add_mul": (None, [P, P, P, P, I64]),
    "tt_cuda_traverse_down_u32_or_and": (None, [P, P, P, P, I64]),
    "tt_cuda_traverse_up_u32_or_and": (None, [P, P, P, P, I64]),
    "tt_cuda_edgelist_degree": (None, [P, P, P, P, I64, I64]),
    "tt_cuda_compute_sfgraph": (None, [P, P, P, P, P, P, P, P, C.c_double, C.c_bool]),
    "tt_cuda_compute_drainage_area_single_flow": (None, [P, P, P, P, C.c_double]),
    # device-pointer forms
    "tt_cuda_fillsinks_dev": (ST, [P, P, P, PD, P]),
    "tt_cuda_fillsinks_noalloc_dev": (ST, [P, P, P, PD, P]),
    "tt_cuda_reconstruct_dev": (ST, [P, P, PD, P]),
    "tt_cuda_identifyflats_dev": (ST, [P, P, PD, P, P]),
    "tt_cuda_gwdt_computecosts_dev": (ST, [P, P, P, P, P, PD, P]),
    "tt_cuda_gwdt_dev": (ST, [P, P, P, P, PD, P]),
    "tt_cuda_flow_routing_d8_carve_dev": (ST, [P, P, P, P, P, PD, U, P]),
    "tt_cuda_flow_accumulation_dev": (ST, [P, P, P, PD, P]),
    "tt_cuda_flow_accumulation_backward_dev": (ST, [P, P, P, PD, P]),
    "tt_cuda_gradient_secondorder_dev": (ST, [P, P, P, F, PD, P]),
    "tt_cuda_hillshade_fused_dev": (ST, [P, P, F, F, F, PD, P]),
    "tt_cuda_hillshade_backward_dev": (ST, [P, P, P, F, F, F, PD, P]),
    "tt_cuda_d8_pipeline_dev": (ST, [P, P, P, P, P, P, P, P, P, P, F, F, F, PD, P]),
    "tt_cuda_flow_routing_d8_edgelist_dev": (ST, [P, P, C.POINTER(I64), P, P, PD, U, P]),
    "tt_cuda_flow_accumulation_edgelist_dev": (ST, [P, P, P, P, P, I64, PD, P]),
    "tt_cuda_drainagebasins_dev": (ST, [P, P, P, I64, PD, P]),
    "tt_cuda_traverse_down_f32_add_mul_dev": (ST, [P, P, P, P, I64, I64, P]),
    "tt_cuda_traverse_down_u32_or_and_dev": (ST, [P, P, P, P, I64, I64, P]),
    "tt_cuda_traverse_up_u32_or_and_dev": (ST, [P, P, P, P, I64, I64, P]),
    "tt_cuda_edgelist_degree_dev": (ST, [P, P, P, P, I64, I64, P]),
    "tt_cuda_compute_sfgraph_dev": (ST, [P, P, P, P, P, P, P, P, C.c_double, C.c_bool, P]),
    "tt_cuda_compute_drainage_area_single_flow_dev": (ST, [P, P, P, C.c_double, P]),
    "tt_cuda_read_file_dev": (ST, [P, C.c_char_p, I64, I64, P]),
    "tt_cuda_write_file_dev": (ST, [C.c_char_p, I64, P, I64, P]),
    # batched form
    "tt_cuda_batch_create": (ST, [C.c_int, PD, I64, C.POINTER(P)]),
    "tt_cuda_batch_info": (ST, [P, C.POINTER(I64)]),
    "tt_cuda_batch_run": (ST, [P, P, P, P, P, P, P, P, P]),
    "tt_cuda_batch_destroy": (None, [P]),
}

STATUS = {
    0: "success",
    1: "invalid argument",
    2: "allocation failed",
    3: "CUDA runtime error",
    4: "iteration cap reached",
    5: "direction grid contains a cycle",
    6: "no CUDA device",
}

_LIB = None


class TTCudaError(RuntimeError):
    def __init__(self, status: int, where: str):
        super().__init__(f"{where}: {STATUS.get(status, status)} (status {status})")
        self.status = status


def lib() -> C.CDLL:
    """Load libtt_cuda.so (once).  Raises if it is absent: no CPU fallback."""
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is missing; build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'`")
        h = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(h, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = h
    return _LIB


def dims_arg(dims):
    arr = (C.c_int64 * 2)(int(dims[0]), int(dims[1]))
    return C.cast(arr, PD), arr  # keep `arr` alive alongside the pointer


def check(status: int, where: str) -> None:
    if status != 0:
        raise TTCudaError(status, where)


def last_status() -> int:
    return int(lib().tt_cuda_last_error())
