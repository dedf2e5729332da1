"""Sun-elevation sweeps rendered as batches of the persistent tracer.

The reference bakes sky-view LUTs for a list of elevations by running its CLI
once per elevation with one sample count for all of them
(scripts/bake_skyview_elevations.ps1:1-16).  Here a sweep is a batch: every
elevation is a job of one persistent launch (optionally replayed as a CUDA
graph), and each job gets its own sample budget, proportional to the
variance a short pilot render measured, so that every elevation reaches the
same per-pixel XYZ error.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, replace

import numpy as np

from .render import GpuScene, RenderConfig
from .scene import sun_from_degrees


def elevation_schedule(count: int = 32, lo: float = -6.0, hi: float = 90.0) -> np.ndarray:
    """Uneven elevations, denser near the horizon: lo + (hi - lo) (k/(n-1))^2."""
    k = np.arange(count, dtype=np.float64)
    return lo + (hi - lo) * (k / max(count - 1, 1)) ** 2


def p95_relative_error(xyz: np.ndarray, var: np.ndarray, dark_fraction: float = 1e-3) -> float:
    """95th percentile over pixels of the worst X/Y/Z relative standard error;
    pixels with Y < dark_fraction * p99(Y) are excluded."""
    y = xyz[:, 1]
    keep = y >= dark_fraction * np.percentile(y, 99)
    if not np.any(keep):
        return 0.0
    rel = np.sqrt(np.maximum(var[keep], 0)) / np.maximum(np.abs(xyz[keep]), 1e-30)
    return float(np.percentile(rel.max(axis=1), 95))


def budgets_from_pilot(p95: np.ndarray, lo: int = 64, hi: int = 1024, multiple: int = 32, seed: int = 2026,
                       jitter: float = 0.05) -> np.ndarray:
    """Per-job spp in proportion to the variance a pilot estimated: the pilot's
    p95 relative error squared, scaled so the noisiest job gets `hi`; jittered
    by +-jitter with a seeded generator, rounded up to `multiple`, clamped to
    [lo, hi].  Equal variance per sample budget equalises the jobs' errors."""
    var = np.asarray(p95, dtype=np.float64) ** 2
    spp = hi * var / max(float(var.max()), 1e-300)
    rng = np.random.default_rng(seed)
    spp = spp * (1.0 + jitter * rng.uniform(-1.0, 1.0, size=spp.shape))
    spp = np.ceil(spp / multiple - 1e-6) * multiple
    return np.clip(spp, lo, hi).astype(np.int64)


def spp_for_target(p95: np.ndarray, spp, target: float = 0.01) -> np.ndarray:
    """Samples each job needs for a p95 error of `target` (error^2 ~ 1/spp)."""
    return np.asarray(spp, dtype=np.float64) * (np.asarray(p95, dtype=np.float64) / target) ** 2


@dataclass
class SweepOutputs:
    cell_sum: object
    cell_sumsq: object
    xyz: object
    xyz_var: object
    status: object
    counters: object

    def pointers(self, first: bool, count_events: bool = False) -> dict:
        d = {"cell_sum": self.cell_sum.data_ptr(), "cell_sumsq": self.cell_sumsq.data_ptr(),
             "xyz": self.xyz.data_ptr(), "xyz_var": self.xyz_var.data_ptr()}
        if first:
            d["status"] = self.status.data_ptr()
            if count_events:
                d["counters"] = self.counters.data_ptr()
        return d


class Sweep:
    """Device buffers and batch jobs for one elevation sweep of a scene.
    With count_events the launch also counts events into `counters` (the
    counting kernels run ~3 % slower)."""

    def __init__(self, gs: GpuScene, base: RenderConfig, elevations, spp, azimuth_deg: float = 0.0,
                 count_events: bool = False):
        import torch
        self.gs = gs
        self.elevations = [float(e) for e in elevations]
        self.spp = [int(s) for s in np.broadcast_to(np.asarray(spp), (len(self.elevations),))]
        self.configs = [replace(base, spp=s, sun_elevation_deg=e, sample_offset=0, flags=0)
                        for e, s in zip(self.elevations, self.spp)]
        self.suns = [sun_from_degrees(e, azimuth_deg, gs.scene.sun_angular_radius_rad)[0] for e in self.elevations]
        cells = base.pixels * gs.band_count
        dev = torch.device("cuda")
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self.counters = torch.zeros(8, dtype=torch.int64, device=dev)
        self.out = [SweepOutputs(torch.zeros(cells, dtype=torch.float64, device=dev),
                                 torch.zeros(cells, dtype=torch.float64, device=dev),
                                 torch.zeros(base.pixels * 3, dtype=torch.float64, device=dev),
                                 torch.zeros(base.pixels * 3, dtype=torch.float64, device=dev),
                                 self.status, self.counters) for _ in self.elevations]
        self.jobs = [(c, sun, o.pointers(i == 0, count_events))
                     for i, (c, sun, o) in enumerate(zip(self.configs, self.suns, self.out))]
        self.graph = None

    @property
    def chains(self) -> int:
        return sum(c.pixels * self.gs.band_count * c.spp for c in self.configs)

    def launch(self, stream: int = 0) -> None:
        self.gs.render_batch(self.jobs, stream)

    def capture(self) -> None:
        self.graph = self.gs.batch_graph(self.jobs)

    def replay(self, stream: int = 0) -> None:
        self.graph.launch(stream)

    def errors(self) -> list:
        """p95 worst-component relative XYZ error of every elevation."""
        errs = []
        for o in self.out:
            xyz = o.xyz.cpu().numpy().reshape(-1, 3)
            var = o.xyz_var.cpu().numpy().reshape(-1, 3)
            errs.append(p95_relative_error(xyz, var))
        return errs


def plan_budgets(gs: GpuScene, base: RenderConfig, elevations, pilot_spp: int = 16, **kw):
    """Render a pilot sweep at pilot_spp and derive each elevation's budget
    (budgets_from_pilot); returns (spp, pilot p95 errors)."""
    import torch
    pilot = Sweep(gs, base, elevations, pilot_spp)
    pilot.launch(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    if int(pilot.status.item()) != 0:
        raise RuntimeError("watchdog tripped in the pilot sweep")
    p95 = np.array(pilot.errors())
    return budgets_from_pilot(p95, **kw), p95
