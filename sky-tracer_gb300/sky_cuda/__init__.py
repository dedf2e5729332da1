"""sky_cuda — GB300 spectral sky path tracer (Python host layer).

The tracing itself runs in libsky_cuda.so (CUDA, sm_103a) behind the C ABI of
include/sky_cuda.h; this package mirrors the reference's host interface
(sky-core scene model, RenderConfig, render, Film) on top of it.
"""

from ._abi import (FLAG_ACCUMULATE, KERNEL_AUTO, KERNEL_PLAIN, KERNEL_WAVEFRONT, PHASE_ISOTROPIC, PHASE_TABULATED,
                   PROJECTION_PANORAMA, PROJECTION_SKY_VIEW_LUT, TRACKING_MERGED_LAYERS, TRACKING_RESIDUAL_CARRY,
                   TRACKING_SEGMENT_RESTART, RenderWatchdog, SkyCudaError, load_library)
from .render import Film, GpuScene, RenderConfig, RenderStats, render
from .scene import (Scene, SceneError, SyntheticAtmosphere, compute_majorant_grid, load_scene_data,
                    sun_from_degrees, synthetic_scene, wavelengths)

__all__ = [
    "FLAG_ACCUMULATE", "KERNEL_AUTO", "KERNEL_PLAIN", "KERNEL_WAVEFRONT", "PHASE_ISOTROPIC", "PHASE_TABULATED",
    "PROJECTION_PANORAMA", "PROJECTION_SKY_VIEW_LUT", "TRACKING_MERGED_LAYERS", "TRACKING_RESIDUAL_CARRY", "TRACKING_SEGMENT_RESTART",
    "RenderWatchdog", "SkyCudaError", "load_library", "Film", "GpuScene", "RenderConfig", "RenderStats", "render",
    "Scene", "SceneError", "SyntheticAtmosphere", "compute_majorant_grid", "load_scene_data", "sun_from_degrees",
    "synthetic_scene", "wavelengths",
]
