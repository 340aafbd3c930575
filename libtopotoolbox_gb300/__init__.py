"""libtopotoolbox_gb300: libtopotoolbox's D8 flow pipeline on one GB300.

fillsinks -> identifyflats -> gwdt_computecosts -> gwdt ->
flow_routing_d8_carve -> flow_accumulation, plus hillshade, as hand-written
sm_103a CUDA kernels behind the C ABI of include/tt_cuda.h
(``libtt_cuda.so``).  ``api`` mirrors the reference's function names over
that ABI; ``autograd`` wraps the adjoints for PyTorch; ``batch`` runs many
DEMs through one captured CUDA graph.
"""
from . import api  # noqa: F401
from .api import (  # noqa: F401
    d8_pipeline,
    fillsinks,
    fillsinks_hybrid,
    flow_accumulation,
    flow_accumulation_backward,
    flow_routing_d8_carve,
    gradient_secondorder,
    gwdt,
    gwdt_computecosts,
    has_gpu,
    hillshade,
    hillshade_backward,
    hillshade_fused,
    identifyflats,
    reconstruct,
)

__all__ = [
    "api",
    "fillsinks",
    "fillsinks_hybrid",
    "reconstruct",
    "identifyflats",
    "gwdt_computecosts",
    "gwdt",
    "flow_routing_d8_carve",
    "flow_accumulation",
    "flow_accumulation_backward",
    "gradient_secondorder",
    "hillshade",
    "hillshade_fused",
    "hillshade_backward",
    "d8_pipeline",
    "has_gpu",
]
