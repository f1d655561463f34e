"""splatter_gb300: GB300-native (sm_103a) implementation of splatter's per-frame splat pipeline.

The compute path is libsplatter_cuda.so (hand-written CUDA behind the C ABI in include/splatter.h);
this package is its Python host mirror of the reference's Renderer/Scene API.
"""
from .renderer import (SORT_COOPERATIVE, SORT_ONESWEEP, BlendMode, Configuration, DepthSorting, FrameGraph,
                       FrameInfo, ProgressiveLoader, Renderer, Scene, SplatterError, compute_uniforms)

__all__ = ["BlendMode", "Configuration", "DepthSorting", "FrameGraph", "FrameInfo", "ProgressiveLoader", "Renderer",
           "Scene", "SplatterError", "compute_uniforms", "SORT_COOPERATIVE", "SORT_ONESWEEP"]
