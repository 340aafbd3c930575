"""PyTorch autograd wrappers of the hand-written adjoints.

``flow_accumulation(weights, direction)``
    Weighted flow accumulation (src/flow_accumulation.c:32-80) with the
    receivers held fixed.  Backward is tt_cuda_flow_accumulation_backward:
    grad_w(u) = sum of grad_acc over the flow path from u to its outlet.
    The forward keeps only the 1-byte direction grid for the backward; the
    adjoint rebuilds its tile contraction from it, so no level boundaries
    have to be checkpointed.

``hillshade(dem, azimuth, altitude, cellsize)``
    hillshade_fused (src/hillshade.c:102-213) with the DEM as the
    differentiable input.  Backward is tt_cuda_hillshade_backward
    (grad_dem = J^T grad_output); cells whose shade is NaN contribute nothing.

Grids are column-major: a (nrows, ncols) grid is a contiguous CUDA tensor of
shape (ncols, nrows), float32.
"""
from __future__ import annotations

import torch

from .api import dev


class _FlowAccumulation(torch.autograd.Function):
    @staticmethod
    def forward(ctx, weights, direction):
        acc = dev.flow_accumulation(direction, weights.contiguous())
        ctx.save_for_backward(direction)
        return acc

    @staticmethod
    def backward(ctx, grad_acc):
        (direction,) = ctx.saved_tensors
        gw = dev.flow_accumulation_backward(direction, grad_acc.contiguous().float())
        return gw, None


class _Hillshade(torch.autograd.Function):
    @staticmethod
    def forward(ctx, dem, azimuth, altitude, cellsize):
        dem = dem.contiguous()
        out = dev.hillshade_fused(dem, azimuth, altitude, cellsize)
        ctx.save_for_backward(dem)
        ctx.angles = (float(azimuth), float(altitude), float(cellsize))
        return out

    @staticmethod
    def backward(ctx, grad_out):
        (dem,) = ctx.saved_tensors
        az, alt, cs = ctx.angles
        g = dev.hillshade_backward(dem, grad_out.contiguous().float(), az, alt, cs)
        return g, None, None, None


def flow_accumulation(weights: torch.Tensor, direction: torch.Tensor) -> torch.Tensor:
    return _FlowAccumulation.apply(weights, direction)


def hillshade(dem: torch.Tensor, azimuth: float, altitude: float, cellsize: float) -> torch.Tensor:
    return _Hillshade.apply(dem, azimuth, altitude, cellsize)
