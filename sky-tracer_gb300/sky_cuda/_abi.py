"""ctypes mirror of include/sky_cuda.h and the loader of libsky_cuda.so.

The library is built in-tree (sky-tracer_gb300/_build/libsky_cuda.so, see
build.py).  There is no CPU fallback: if the library is missing, importing the
render entry points raises.
"""

from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

PACKAGE_ROOT = Path(__file__).resolve().parent.parent
LIB_PATH = PACKAGE_ROOT / "_build" / "libsky_cuda.so"

SPECIES_COUNT = 4

# Status codes (SkyStatus); 1-6 = RenderError variants (integrator.rs:18-26).
SKY_OK = 0
SKY_ERR_INVALID_CONFIG = 1
SKY_ERR_NO_DEVICE = 2
SKY_ERR_DEVICE_INIT = 3
SKY_ERR_COPY = 4
SKY_ERR_SYNC = 5
SKY_ERR_WATCHDOG = 6
SKY_ERR_OUT_OF_MEMORY = 7
SKY_ERR_LAUNCH = 8
SKY_ERR_IO = 9

PROJECTION_PANORAMA = 0
PROJECTION_SKY_VIEW_LUT = 1
PHASE_ISOTROPIC = 0
PHASE_TABULATED = 1
TRACKING_SEGMENT_RESTART = 0
TRACKING_RESIDUAL_CARRY = 1
TRACKING_MERGED_LAYERS = 2
KERNEL_AUTO = 0
KERNEL_PLAIN = 1
KERNEL_WAVEFRONT = 2
FLAG_ACCUMULATE = 1
FLAG_COUNT_EVENTS = 2

EVENT_NAMES = ("track_step", "segment", "boundary", "scatter", "nee", "ground", "chain")
EVENT_COUNT = 8

# numpy dtypes with the byte layout of the C rows (integrator.rs:77-112).
BAND_DTYPE = np.dtype([
    ("center_nm", "<f4"), ("lower_nm", "<f4"), ("upper_nm", "<f4"),
    ("ozone_cross_section_cm2", "<f4"), ("solar_radiance_w_m2_sr", "<f4"),
    ("rayleigh_cross_section_m2", "<f4"),
])
ATMOSPHERE_DTYPE = np.dtype([
    ("altitude_km", "<f4"), ("temperature_k", "<f4"), ("air_cm3", "<f4"), ("ozone_cm3", "<f4"),
])
AEROSOL_DTYPE = np.dtype([("altitude_km", "<f4"), ("mass_g_m3", "<f4", (4,)), ("_pad", "<f4", (3,))])
OPTICS_DTYPE = np.dtype([("scattering_km_inv_per_g_m3", "<f4"), ("absorption_km_inv_per_g_m3", "<f4")])
assert BAND_DTYPE.itemsize == 24 and ATMOSPHERE_DTYPE.itemsize == 16
assert AEROSOL_DTYPE.itemsize == 32 and OPTICS_DTYPE.itemsize == 8

_f = ctypes.c_float
_u32 = ctypes.c_uint32
_fp = ctypes.POINTER(ctypes.c_float)
_dp = ctypes.POINTER(ctypes.c_double)
_vp = ctypes.c_void_p


class SkySceneDesc(ctypes.Structure):
    _fields_ = [
        ("band_count", _u32), ("atmosphere_len", _u32), ("aerosol_len", _u32),
        ("majorant_layers", _u32), ("phase_bins", _u32), ("_reserved0", _u32),
        ("ground_radius_km", _f), ("atmosphere_radius_km", _f), ("top_altitude_km", _f),
        ("sun_direction", _f * 3), ("sun_angular_radius_rad", _f), ("sun_solid_angle_sr", _f),
        ("ground_albedo", _f), ("_reserved1", _f),
        ("bands", _vp), ("atmosphere", _vp), ("aerosol", _vp), ("aerosol_optics", _vp),
        ("majorants_km_inv", _vp), ("phase_values", _vp), ("band_xyz_weights", _vp),
    ]


class SkyRenderConfig(ctypes.Structure):
    _fields_ = [
        ("width", _u32), ("height", _u32), ("spp", _u32), ("direct_light_samples", _u32),
        ("seed", ctypes.c_uint64),
        ("sun_elevation_deg", _f), ("sun_azimuth_deg", _f), ("observer_altitude_km", _f),
        ("output_projection", _u32),
        ("sample_offset", _u32), ("phase_sampling", _u32), ("rr_start_depth", _u32),
        ("max_orders", _u32), ("watchdog_limit", _u32), ("kernel", _u32), ("flags", _u32),
        ("tracking", _u32), ("row_begin", _u32), ("row_count", _u32),
    ]


class SkyRenderStats(ctypes.Structure):
    _fields_ = [
        ("kernel_ms", ctypes.c_double), ("total_ms", ctypes.c_double), ("chains", ctypes.c_uint64),
        ("events", ctypes.c_uint64 * EVENT_COUNT), ("watchdog", _u32), ("kernel_used", _u32),
    ]


class SkyDeviceOutputs(ctypes.Structure):
    _fields_ = [
        ("cell_sum", _vp), ("cell_sumsq", _vp), ("film", _vp), ("xyz", _vp), ("xyz_var", _vp),
        ("counters", _vp), ("status", _vp), ("rgb", _vp),
    ]


class SkyTuning(ctypes.Structure):
    _fields_ = [
        ("variant", _u32), ("max_blocks_per_sm", _u32), ("all_species", _u32), ("_unused", _u32),
        ("crossing_cost", _f), ("iteration_limit", _u32), ("_reserved", _u32 * 2),
    ]


class SkyBatchJob(ctypes.Structure):
    _fields_ = [
        ("config", SkyRenderConfig), ("sun_direction", _f * 3), ("_reserved", _f), ("outputs", SkyDeviceOutputs),
    ]


class SkyAdjointParams(ctypes.Structure):
    _fields_ = [
        ("layer_params", _vp), ("band_params", _vp), ("sample_layer_params", _vp), ("sample_band_params", _vp),
        ("sun_direction", _f * 3), ("estimator", _u32), ("chain_radiance", _vp), ("chain_radiance_len", ctypes.c_uint64),
    ]


class SkyAdjointGrads(ctypes.Structure):
    _fields_ = [
        ("dloss_dfilm", _vp), ("layer_grad", _vp), ("band_grad", _vp), ("counters", _vp), ("status", _vp),
    ]


class SkyAdjointJob(ctypes.Structure):
    _fields_ = [
        ("config", SkyRenderConfig), ("sun_direction", _f * 3), ("_reserved", _f), ("outputs", SkyDeviceOutputs),
        ("dloss_dfilm", _vp), ("chain_radiance", _vp), ("chain_radiance_len", ctypes.c_uint64),
    ]


class SkyComboScore(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("mean", "rmse", "p50", "p90", "p95", "p99", "max", "score")] + [
        ("finite", ctypes.c_uint64)]


class SkyMieDistribution(ctypes.Structure):
    _fields_ = [("r_mode_um", ctypes.c_double), ("sigma_g", ctypes.c_double), ("r_min_um", ctypes.c_double),
                ("r_max_um", ctypes.c_double), ("r_count", ctypes.c_uint32), ("_reserved", ctypes.c_uint32)]


class SkyMieBand(ctypes.Structure):
    _fields_ = [("sigma_sca_um2", ctypes.c_double), ("sigma_ext_um2", ctypes.c_double), ("g", ctypes.c_double)]


ADJOINT_BAND_PARAMS = 4
ADJOINT_SEGMENT_INTEGRALS = 0
ADJOINT_NULL_COLLISIONS = 1

assert ctypes.sizeof(SkySceneDesc) == 120
assert ctypes.sizeof(SkyRenderConfig) == 80
assert ctypes.sizeof(SkyRenderStats) == 96

# Every symbol include/sky_cuda.h declares, with its ctypes signature.
_SIGNATURES = {
    "sky_cuda_version": (ctypes.c_char_p, []),
    "sky_cuda_last_error": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
    "sky_cuda_device_allocations": (ctypes.c_uint64, []),
    "sky_cuda_probe_shell_geometry": (ctypes.c_int, [_vp, _vp, ctypes.c_uint32, _vp, ctypes.c_uint32, ctypes.c_float,
                                                     _vp, _vp, _vp]),
    "sky_cuda_scene_create": (ctypes.c_int, [ctypes.POINTER(SkySceneDesc), ctypes.POINTER(_vp)]),
    "sky_cuda_scene_destroy": (None, [_vp]),
    "sky_cuda_scene_set_tuning": (ctypes.c_int, [_vp, ctypes.POINTER(SkyTuning)]),
    "sky_cuda_scene_get_tuning": (ctypes.c_int, [_vp, ctypes.POINTER(SkyTuning)]),
    "sky_cuda_render": (ctypes.c_int, [_vp, ctypes.POINTER(SkyRenderConfig), _fp, ctypes.c_size_t,
                                       ctypes.POINTER(SkyRenderStats)]),
    "sky_cuda_render_xyz": (ctypes.c_int, [_vp, ctypes.POINTER(SkyRenderConfig), _fp, ctypes.c_size_t,
                                           ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                           ctypes.c_size_t, ctypes.POINTER(SkyRenderStats)]),
    "sky_cuda_render_rgb": (ctypes.c_int, [_vp, ctypes.POINTER(SkyRenderConfig), _fp, ctypes.c_size_t, _fp,
                                           ctypes.c_size_t, ctypes.POINTER(SkyRenderStats)]),
    "sky_cuda_render_desc": (ctypes.c_int, [ctypes.POINTER(SkySceneDesc), ctypes.POINTER(SkyRenderConfig), _fp,
                                            ctypes.c_size_t, ctypes.POINTER(SkyRenderStats)]),
    "sky_cuda_render_device": (ctypes.c_int, [_vp, ctypes.POINTER(SkyRenderConfig),
                                              ctypes.POINTER(SkyDeviceOutputs), _vp]),
    "sky_cuda_render_batch": (ctypes.c_int, [_vp, ctypes.POINTER(SkyBatchJob), ctypes.c_uint32, _vp]),
    "sky_cuda_batch_graph_create": (ctypes.c_int, [_vp, ctypes.POINTER(SkyBatchJob), ctypes.c_uint32,
                                                   ctypes.POINTER(_vp)]),
    "sky_cuda_batch_graph_launch": (ctypes.c_int, [_vp, _vp]),
    "sky_cuda_batch_graph_destroy": (None, [_vp]),
    "sky_cuda_adjoint_param_count": (ctypes.c_uint32, [_vp]),
    "sky_cuda_adjoint_forward": (ctypes.c_int, [_vp, ctypes.POINTER(SkyRenderConfig),
                                                ctypes.POINTER(SkyAdjointParams), ctypes.POINTER(SkyDeviceOutputs),
                                                _vp]),
    "sky_cuda_adjoint_backward": (ctypes.c_int, [_vp, ctypes.POINTER(SkyRenderConfig),
                                                 ctypes.POINTER(SkyAdjointParams), ctypes.POINTER(SkyAdjointGrads),
                                                 _vp]),
    "sky_cuda_adjoint_forward_batch": (ctypes.c_int, [_vp, ctypes.POINTER(SkyAdjointJob), ctypes.c_uint32,
                                                      ctypes.POINTER(SkyAdjointParams), _vp]),
    "sky_cuda_adjoint_backward_batch": (ctypes.c_int, [_vp, ctypes.POINTER(SkyAdjointJob), ctypes.c_uint32,
                                                       ctypes.POINTER(SkyAdjointParams),
                                                       ctypes.POINTER(SkyAdjointGrads), _vp]),
    "sky_cuda_bake_majorants": (ctypes.c_int, [_vp, ctypes.POINTER(SkyAdjointParams), _vp, _vp]),
    "sky_cuda_score_combos": (ctypes.c_int, [_vp, ctypes.c_uint32, ctypes.c_uint64, _vp, ctypes.c_float,
                                             ctypes.POINTER(ctypes.c_uint32), _fp, ctypes.c_uint32, ctypes.c_uint32,
                                             ctypes.POINTER(SkyComboScore), _vp]),
    "sky_cuda_render_batch_noalloc": (ctypes.c_int, [_vp, ctypes.POINTER(SkyRenderConfig),
                                                     ctypes.POINTER(SkyDeviceOutputs), ctypes.c_uint32, _vp]),
    "sky_cuda_bake_mie_phase": (ctypes.c_int, [ctypes.POINTER(SkyMieDistribution), _dp, _dp, _dp, ctypes.c_uint32,
                                               ctypes.c_uint32, _dp, ctypes.POINTER(SkyMieBand)]),
}
NOALLOC_MAX_JOBS = 16

_LIB = None


def library_path() -> Path:
    return Path(os.environ.get("SKY_CUDA_LIB", str(LIB_PATH)))


def load_library() -> ctypes.CDLL:
    """Load libsky_cuda.so (built by sky-tracer_gb300/build.py); raises if absent."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not path.exists():
        raise RuntimeError(
            f"libsky_cuda.so not found at {path}; build it with "
            "`python sky-tracer_gb300/build.py` (there is no CPU fallback)")
    lib = ctypes.CDLL(str(path))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def declared_symbols() -> list[str]:
    return list(_SIGNATURES)


def last_error(lib=None) -> str:
    lib = lib or load_library()
    buf = ctypes.create_string_buffer(1024)
    lib.sky_cuda_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


class SkyCudaError(RuntimeError):
    """A failed C-ABI call; `status` is the SkyStatus code."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status
        self.message = message


class RenderWatchdog(SkyCudaError):
    """RenderError::Watchdog (integrator.rs:301-304)."""


def check(status: int, lib=None) -> None:
    if status == SKY_OK:
        return
    msg = last_error(lib)
    if status == SKY_ERR_WATCHDOG:
        raise RenderWatchdog(status, msg)
    raise SkyCudaError(status, msg)
