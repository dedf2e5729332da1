"""Autotuner of the wavefront tracer's launch shape.

The reference dispatches a fixed 8x8x1 workgroup per (pixel block, band) and
two samples per dispatch (integrator.rs:254-283); nothing is tuned.  Here the
shape of the wavefront kernel is a per-scene setting (SkyTuning): the
resident blocks per SM it is compiled for (registers per lane against lanes
in flight) and the crossing cost that sets how far the tracking grid is
merged.  `autotune` times each candidate on a reduced-sample probe of the
caller's own render (same image, same scene, fewer samples per pixel) with
CUDA events and keeps the fastest on the scene.
"""

from __future__ import annotations

import itertools
from dataclasses import replace

from .render import GpuScene, RenderConfig

DEFAULT_SPACE = {
    "variant": (0, 1, 2),
    "crossing_cost": (0.1, 0.25, 0.5, 1.0),
}


def _time_render(gs: GpuScene, cfg: RenderConfig, repeats: int) -> float:
    import torch
    cells = cfg.pixels * gs.band_count
    s = torch.empty(cells, dtype=torch.float64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    outs = {"cell_sum": s.data_ptr(), "status": status.data_ptr()}
    gs.render_device(cfg, outs, stream.cuda_stream)  # warm-up (first launch sets attributes)
    best = float("inf")
    for _ in range(repeats):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        gs.render_device(cfg, outs, stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    if int(status.item()) != 0:
        raise RuntimeError("watchdog tripped while tuning")
    return best


def autotune(gs: GpuScene, config: RenderConfig, space: dict | None = None, probe_spp: int | None = None,
             repeats: int = 2, apply: bool = True):
    """Time every combination of `space` on a probe render and keep the best.

    Returns (best_tuning_dict, [(tuning_dict, ms), ...]).  The probe renders
    the caller's full image at `probe_spp` samples (default: spp/8, at least 64
    or the whole render: below two warps' worth of samples per cell the lanes
    of a warp sit idle in a way the render itself does not, and a 64x32 render
    probed at 8 spp picked a shape 24 % slower at its 64 spp).
    """
    space = dict(DEFAULT_SPACE if space is None else space)
    probe = replace(config, spp=probe_spp or min(config.spp, max(64, config.spp // 8)), sample_offset=0, flags=0)
    keys = list(space)
    base = gs.get_tuning()
    results = []
    for values in itertools.product(*(space[k] for k in keys)):
        t = dict(base)
        t.update(zip(keys, values))
        gs.set_tuning(**t)
        results.append((gs.get_tuning(), _time_render(gs, probe, repeats)))
    best = min(results, key=lambda r: r[1])[0]
    gs.set_tuning(**(best if apply else base))
    return best, results
