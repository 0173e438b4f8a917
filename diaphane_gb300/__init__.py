"""diaphane_gb300: a GB300-native (sm_103a) Yee leapfrog time step.

The product is the CUDA library ``libdiaphane_gb300.so`` behind the C ABI in
``include/diaphane_gb300.h``; this package is its Python binding and the
scene-authoring model that mirrors the reference's Rust types.
"""
from ._abi import DiaphaneError, DP_KERNEL_AUTO, DP_KERNEL_FUSED, DP_KERNEL_NAIVE
from .scene import (Axis, Boundary, Extent, Grid, Material, MaterialTable, Refinement, Scene, Shape, Source,
                    Waveform, COURANT_LIMIT, SPEED_OF_LIGHT)
from .simulation import Energy, ResolvedScene, Simulation, Simulation64, Snapshot
from .batch import Batch
from .timeline import DeviceTimeline, Seek, Timeline

__all__ = [
    "Axis", "Batch", "DeviceTimeline", "Boundary", "COURANT_LIMIT", "DiaphaneError", "DP_KERNEL_AUTO", "DP_KERNEL_FUSED", "DP_KERNEL_NAIVE",
    "Energy", "Extent", "Grid", "Material", "MaterialTable", "Refinement", "ResolvedScene", "Scene", "Seek",
    "Shape", "Simulation", "Simulation64", "Snapshot", "SPEED_OF_LIGHT", "Source", "Timeline", "Waveform",
]
