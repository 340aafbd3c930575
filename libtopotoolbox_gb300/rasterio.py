"""Raster files straight to and from device memory (tt_cuda_read_file_dev /
tt_cuda_write_file_dev): the GPU-side step before and after the D8 path.

    dem = read_npy("dem.npy")            # torch CUDA tensor, (ncols, nrows)
    write_npy("filled.npy", filled)       # column-major (Fortran-order) .npy

The reference's callers read DEMs with GDAL (test/grid.c:41-134); here a
`.npy` file (or any raw little-endian grid at a known byte offset, through
`read_raw`) is streamed by the native loader through two pinned buffers, so
disk reads overlap the host-to-device copies and no pageable host copy of the
grid is made.  Grids follow the library's convention: a column-major
(nrows, ncols) grid is a contiguous tensor of shape (ncols, nrows).
"""
from __future__ import annotations

import ast
import os
import struct

import numpy as np

from . import _native as N

_TORCH = {"<f4": "float32", "<f8": "float64", "|u1": "uint8", "<i4": "int32",
          "<i8": "int64", "<u8": "uint64"}


def _torch_dtype(descr):
    import torch

    if descr not in _TORCH:
        raise ValueError(f"unsupported .npy dtype {descr!r}")
    return getattr(torch, _TORCH[descr])


def npy_header(path):
    """(descr, fortran_order, shape, data_offset) of a .npy file."""
    with open(path, "rb") as f:
        magic = f.read(8)
        if magic[:6] != b"\x93NUMPY":
            raise ValueError(f"{path}: not a .npy file")
        major = magic[6]
        if major == 1:
            hlen = struct.unpack("<H", f.read(2))[0]
            off = 10
        else:
            hlen = struct.unpack("<I", f.read(4))[0]
            off = 12
        hdr = ast.literal_eval(f.read(hlen).decode("latin1"))
    return hdr["descr"], bool(hdr["fortran_order"]), tuple(hdr["shape"]), off + hlen


def read_raw(path, offset, shape, dtype, device=None):
    """A raw grid of `shape` (torch order) and torch `dtype` at byte
    `offset` of `path`, as a CUDA tensor."""
    import torch

    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else device
    t = torch.empty(shape, dtype=dtype, device=dev)
    nbytes = t.numel() * t.element_size()
    st = torch.cuda.current_stream(dev).cuda_stream
    N.check(N.lib().tt_cuda_read_file_dev(N.C.c_void_p(t.data_ptr()), os.fsencode(path),
                                          int(offset), int(nbytes), N.C.c_void_p(st)),
            "read_file_dev")
    return t


def read_npy(path, device=None):
    """A 2-D .npy grid as a column-major CUDA tensor of shape (ncols, nrows).
    Fortran-order files are streamed as they are; C-order files are
    streamed and then transposed on the device."""
    descr, fortran, shape, off = npy_header(path)
    if len(shape) != 2:
        raise ValueError(f"{path}: expected a 2-D grid, got shape {shape}")
    dt = _torch_dtype(descr)
    nrows, ncols = shape
    if fortran:
        return read_raw(path, off, (ncols, nrows), dt, device)
    return read_raw(path, off, (nrows, ncols), dt, device).t().contiguous()


def write_npy(path, grid):
    """Writes a column-major CUDA tensor of shape (ncols, nrows) as a
    Fortran-order (nrows, ncols) .npy file."""
    import torch

    grid = grid.contiguous()
    descr = {v: k for k, v in _TORCH.items()}[str(grid.dtype).replace("torch.", "")]
    ncols, nrows = grid.shape
    hdr = repr({"descr": descr, "fortran_order": True, "shape": (nrows, ncols)})
    pad = 64 - (10 + len(hdr) + 1) % 64
    text = (hdr + " " * pad + "\n").encode("latin1")
    with open(path, "wb") as f:
        f.write(b"\x93NUMPY\x01\x00" + struct.pack("<H", len(text)) + text)
    st = torch.cuda.current_stream(grid.device).cuda_stream
    N.check(N.lib().tt_cuda_write_file_dev(os.fsencode(path), 10 + len(text),
                                           N.C.c_void_p(grid.data_ptr()),
                                           int(grid.numel() * grid.element_size()),
                                           N.C.c_void_p(st)),
            "write_file_dev")
