"""Host-side mirror of the reference integrator API over the C ABI.

    render(scene, config) -> Film          # integrator.rs:125-128
    RenderConfig                           # config.rs:2-52
    Film                                   # film.rs:2-62
    RenderError kinds                      # integrator.rs:18-39 (SkyCudaError.status)

GpuScene keeps the scene's tables resident on the device between renders
(sky_cuda_scene_create); render() is the one-shot form that uploads, renders
and frees inside the call, like the reference.
"""

from __future__ import annotations

import ctypes
import weakref
from dataclasses import dataclass

import numpy as np

from . import _abi
from ._abi import (SkyBatchJob, SkyDeviceOutputs, SkyRenderConfig, SkyRenderStats, SkyTuning, check,
                   load_library)
from .scene import Scene

DEFAULT_SEED = 0x5EC7_2026_0430  # config.rs:44


@dataclass
class RenderConfig:
    """RenderConfig (config.rs:2-12, defaults :38-52) plus the extensions of
    SkyRenderConfig; the extension defaults reproduce the reference shader."""

    width: int = 1024
    height: int = 512
    spp: int = 256
    seed: int = DEFAULT_SEED
    sun_elevation_deg: float = 0.0
    sun_azimuth_deg: float = 0.0
    observer_altitude_km: float = 0.2
    direct_light_samples: int = 1
    output_projection: int = _abi.PROJECTION_PANORAMA
    sample_offset: int = 0
    phase_sampling: int = _abi.PHASE_ISOTROPIC
    rr_start_depth: int = 0
    max_orders: int = 0
    watchdog_limit: int = 0
    kernel: int = _abi.KERNEL_AUTO
    flags: int = 0
    tracking: int = _abi.TRACKING_SEGMENT_RESTART
    # pixel-row slab [row_begin, row_begin + row_count); 0 rows = the whole image
    row_begin: int = 0
    row_count: int = 0

    def to_c(self) -> SkyRenderConfig:
        c = SkyRenderConfig()
        for name, _ in SkyRenderConfig._fields_:
            if name.startswith("_"):
                continue
            setattr(c, name, getattr(self, name))
        return c

    @property
    def rows(self) -> int:
        """Image rows this config renders (its slab, or every row)."""
        return self.row_count or self.height

    @property
    def pixels(self) -> int:
        """Pixels of the outputs: the slab's (width * rows)."""
        return self.width * self.rows


@dataclass
class Film:
    """Film (film.rs:2-62): pixel-major, band-minor float32 values."""

    width: int
    height: int
    band_count: int
    values: np.ndarray

    def pixel_spectrum(self, pixel: int) -> np.ndarray:
        return self.values[pixel * self.band_count:(pixel + 1) * self.band_count]

    def as_array(self) -> np.ndarray:
        return self.values.reshape(self.height, self.width, self.band_count)


@dataclass
class RenderStats:
    kernel_ms: float
    total_ms: float
    chains: int
    events: dict
    watchdog: int
    kernel_used: int

    @classmethod
    def from_c(cls, s: SkyRenderStats) -> "RenderStats":
        return cls(s.kernel_ms, s.total_ms, int(s.chains),
                   {n: int(s.events[i]) for i, n in enumerate(_abi.EVENT_NAMES)}, int(s.watchdog),
                   int(s.kernel_used))


def _fptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class GpuScene:
    """A scene uploaded to the current CUDA device (sky_cuda_scene_create)."""

    def __init__(self, scene: Scene):
        self.lib = load_library()
        self.scene = scene
        self.band_count = scene.band_count
        self._desc = scene.desc()
        handle = ctypes.c_void_p()
        check(self.lib.sky_cuda_scene_create(ctypes.byref(self._desc), ctypes.byref(handle)), self.lib)
        self.handle = handle
        self._graphs = weakref.WeakSet()  # batch graphs replay this scene's tables

    def close(self) -> None:
        if getattr(self, "handle", None) and self.handle.value:
            for g in list(getattr(self, "_graphs", ())):
                g.close()
            self.lib.sky_cuda_scene_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_tuning(self) -> dict:
        t = SkyTuning()
        check(self.lib.sky_cuda_scene_get_tuning(self.handle, ctypes.byref(t)), self.lib)
        return {"variant": t.variant, "max_blocks_per_sm": t.max_blocks_per_sm,
                "crossing_cost": float(t.crossing_cost), "iteration_limit": t.iteration_limit,
                "all_species": t.all_species}

    def set_tuning(self, **kw) -> None:
        """Set launch-shape fields of SkyTuning (unnamed fields keep their value)."""
        cur = self.get_tuning()
        cur.update(kw)
        t = SkyTuning()
        for k, v in cur.items():
            setattr(t, k, v)
        check(self.lib.sky_cuda_scene_set_tuning(self.handle, ctypes.byref(t)), self.lib)

    @staticmethod
    def _c_config(config: RenderConfig, count_events: bool):
        c = config.to_c()
        if count_events:
            c.flags |= _abi.FLAG_COUNT_EVENTS
        return c

    def render(self, config: RenderConfig, count_events: bool = False) -> tuple[Film, RenderStats]:
        """Film and stats; the stats' event counts are filled with
        count_events=True (the counting kernels run ~3 % slower)."""
        film = np.empty(config.pixels * self.band_count, dtype=np.float32)
        stats = SkyRenderStats()
        check(self.lib.sky_cuda_render(self.handle, ctypes.byref(self._c_config(config, count_events)), _fptr(film),
                                       film.size, ctypes.byref(stats)), self.lib)
        return Film(config.width, config.rows, self.band_count, film), RenderStats.from_c(stats)

    def render_xyz(self, config: RenderConfig, with_film: bool = True, count_events: bool = False):
        """Film, per-pixel XYZ [pixels, 3] (FP64) and its variance, and stats."""
        film = np.empty(config.pixels * self.band_count, dtype=np.float32) if with_film else None
        xyz = np.empty((config.pixels, 3), dtype=np.float64)
        var = np.empty((config.pixels, 3), dtype=np.float64)
        stats = SkyRenderStats()
        check(self.lib.sky_cuda_render_xyz(self.handle, ctypes.byref(self._c_config(config, count_events)),
                                           _fptr(film) if film is not None else None,
                                           film.size if film is not None else 0, _dptr(xyz), _dptr(var),
                                           config.pixels, ctypes.byref(stats)), self.lib)
        f = Film(config.width, config.rows, self.band_count, film) if film is not None else None
        return f, xyz, var, RenderStats.from_c(stats)

    def render_rgb(self, config: RenderConfig, with_film: bool = True, count_events: bool = False):
        """Film and per-pixel white-balanced linear sRGB [pixels, 3] (float32,
        from the kernel epilogue), and stats."""
        film = np.empty(config.pixels * self.band_count, dtype=np.float32) if with_film else None
        rgb = np.empty((config.pixels, 3), dtype=np.float32)
        stats = SkyRenderStats()
        check(self.lib.sky_cuda_render_rgb(self.handle, ctypes.byref(self._c_config(config, count_events)),
                                           _fptr(film) if film is not None else None,
                                           film.size if film is not None else 0, _fptr(rgb), config.pixels,
                                           ctypes.byref(stats)), self.lib)
        f = Film(config.width, config.rows, self.band_count, film) if film is not None else None
        return f, rgb, RenderStats.from_c(stats)

    def render_batch(self, jobs, stream: int = 0) -> None:
        """One persistent launch over [(RenderConfig, sun_direction or None, outputs), ...]."""
        arr = batch_jobs(jobs)
        check(self.lib.sky_cuda_render_batch(self.handle, arr, len(jobs), ctypes.c_void_p(stream)), self.lib)

    def batch_graph(self, jobs) -> "BatchGraph":
        return BatchGraph(self, jobs)

    def render_device(self, config: RenderConfig, outputs: dict, stream: int = 0) -> None:
        """Queue a render into device buffers given as integer device pointers
        (keys: cell_sum, cell_sumsq, film, xyz, xyz_var, counters, status)."""
        o = SkyDeviceOutputs()
        for name, _ in SkyDeviceOutputs._fields_:
            setattr(o, name, outputs.get(name) or None)
        check(self.lib.sky_cuda_render_device(self.handle, ctypes.byref(config.to_c()), ctypes.byref(o),
                                              ctypes.c_void_p(stream)), self.lib)


def _device_outputs(outputs: dict) -> SkyDeviceOutputs:
    o = SkyDeviceOutputs()
    for name, _ in SkyDeviceOutputs._fields_:
        setattr(o, name, outputs.get(name) or None)
    return o


def batch_jobs(jobs) -> ctypes.Array:
    """SkyBatchJob array from [(RenderConfig, sun_direction or None, outputs dict), ...]."""
    arr = (SkyBatchJob * len(jobs))()
    for i, (cfg, sun, outs) in enumerate(jobs):
        arr[i].config = cfg.to_c()
        arr[i].sun_direction = (ctypes.c_float * 3)(*(sun if sun is not None else (0.0, 0.0, 0.0)))
        arr[i].outputs = _device_outputs(outs)
    return arr


class BatchGraph:
    """A batch captured once into a CUDA graph (sky_cuda_batch_graph_create)
    and replayed with launch(); the outputs must outlive the graph."""

    def __init__(self, gs: "GpuScene", jobs):
        self.lib = gs.lib
        self._jobs = batch_jobs(jobs)
        handle = ctypes.c_void_p()
        check(self.lib.sky_cuda_batch_graph_create(gs.handle, self._jobs, len(jobs), ctypes.byref(handle)),
              self.lib)
        self.handle = handle
        gs._graphs.add(self)

    def launch(self, stream: int = 0) -> None:
        check(self.lib.sky_cuda_batch_graph_launch(self.handle, ctypes.c_void_p(stream)), self.lib)

    def close(self) -> None:
        if getattr(self, "handle", None) and self.handle.value:
            self.lib.sky_cuda_batch_graph_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def render(scene: Scene, config: RenderConfig) -> Film:
    """One-shot render (integrator.rs:125-128): upload, trace, read back, free."""
    lib = load_library()
    desc = scene.desc()
    film = np.empty(config.pixels * scene.band_count, dtype=np.float32)
    check(lib.sky_cuda_render_desc(ctypes.byref(desc), ctypes.byref(config.to_c()), _fptr(film), film.size,
                                   None), lib)
    return Film(config.width, config.rows, scene.band_count, film)
