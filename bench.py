#!/usr/bin/env python
"""Benchmark: spectral path samples/s of the GB300 sky tracer.

Workload (default): the production-size plain render — a 512x256 equirect
panorama, 81 wavelengths at 5 nm from 380 to 780 nm, 256 samples per
pixel and wavelength, Russian roulette after order 8, no order cap, sun at 5
degrees, 64 majorant layers over 0-100 km, tabulated phase sampling.  One
"step" is one full render: 512*256*81*256 = 2,717,908,992 chains (a chain is
one (pixel, wavelength, sample) path).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value   chains/s with the scene resident on the device, CUDA events around the
        render on the launching stream, L2 flushed between timed steps.
e2e     the same metric through the one-shot C-ABI call
        (sky_cuda_render_desc): host tables in, host film out, both copies
        inside the timed region.
Under torchrun the ranks split the one render into contiguous pixel-row
slabs (strong scaling: the render's chains / the slowest rank's time); the
slabs are joined on rank 0.  No collective on the data path.

The default line also carries, on one GPU: the CPU baseline (the oracle in
the reference's tracking, and in the GPU's merged-layer tracking), a parity
block (GPU against that oracle render on its rows), the differentiable-render
block, the elevation-sweep block and a cut-down wavelength-primary fit.
"""

from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "sky-tracer_gb300"))
DATA_DIR = ROOT / "tests" / "golden" / "data"

# DRAM bytes (read + write) of one launch of the wavefront tracing kernel on
# the production render, from a 1-pass ncu capture
# (profiles/wave_kernel_plain-512x256-81wl-256spp_dram.txt).
WAVE_LAUNCH_DRAM_BYTES = {"plain-512x256-81wl-256spp": 198.83e6 + 206.33e6}

# Frozen per-event FP32 work weights (FLOP, an FMA counted as 2), counted
# from the reference shader's arithmetic for each event type.
EVENT_FLOPS = {"track_step": 72, "segment": 48, "boundary": 40, "scatter": 200, "nee": 40, "ground": 150,
               "chain": 46}

WORKLOADS = {
    "plain-512x256-81wl-256spp": dict(width=512, height=256, lam=(380.0, 780.0, 81), spp=256, sun=5.0,
                                      rr_start_depth=8, max_orders=0),
    "plain-64x32-32wl-64spp": dict(width=64, height=32, lam=(380.0, 780.0, 32), spp=64, sun=10.0,
                                   rr_start_depth=0, max_orders=16),
    # the production workload at 1/16 of the pixels and 1/4 of the samples: profiling case
    "profile-128x64-81wl-64spp": dict(width=128, height=64, lam=(380.0, 780.0, 81), spp=64, sun=5.0,
                                      rr_start_depth=8, max_orders=0),
}
DEFAULT_WORKLOAD = "plain-512x256-81wl-256spp"
# the elevation sweep: 32 sun elevations on [-6, 90] (denser near the horizon), each a
# 256x128 sky-view LUT over 40 wavelengths, spp 64-1024 from a 16-spp pilot
SWEEP_WORKLOAD = "sweep-32x256x128-40wl"
ADJOINT_WORKLOAD = "adjoint-128x64-32wl-64spp"
# 4 primary wavelengths + a 4x3 XYZ matrix fitted against 81-wavelength renders at 16 elevations
FIT_WORKLOAD = "fit-16x256x128-4primaries"


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=("ours", "reference"), default="ours")
    p.add_argument("--workload", choices=sorted(WORKLOADS) + [SWEEP_WORKLOAD, ADJOINT_WORKLOAD, FIT_WORKLOAD],
                   default=DEFAULT_WORKLOAD)
    p.add_argument("--kernel", type=int, default=0, help="SkyKernel (0 auto, 1 plain, 2 wavefront)")
    p.add_argument("--tuning", default="",
                   help="SkyTuning fields set before autotuning, e.g. variant=0,crossing_cost=0.25")
    p.add_argument("--tracking", type=int, default=2, help="SkyTracking (2 = residual carry, merged layers)")
    p.add_argument("--e2e-steps", type=int, default=4)
    p.add_argument("--no-peak", action="store_true", help="skip the SGEMM FP32-peak measurement")
    p.add_argument("--cpu-seconds", type=float, default=15.0, help="budget of the CPU-baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-autotune", action="store_true", help="keep the default launch shape")
    p.add_argument("--no-adjoint", action="store_true", help="leave the differentiable-render block out")
    p.add_argument("--fit-iterations", type=int, default=200, help="Adam steps of each primary fit")
    p.add_argument("--fit-summary-iterations", type=int, default=60,
                   help="Adam steps of the cut-down fit in the default line (0 leaves the fit block out)")
    p.add_argument("--no-sweep", action="store_true", help="leave the elevation-sweep block out")
    p.add_argument("--equal-slabs", action="store_true",
                   help="N > 1: equal-row slabs instead of the cost-balanced ones of a pilot render")
    p.add_argument("--no-adjoint-checks", action="store_true",
                   help="time the differentiable render only (no gradient checks)")
    return p.parse_args()


def make_scene(w, rank: int = 0):
    from sky_cuda import synthetic_scene, wavelengths
    lo, hi, n = w["lam"]
    return synthetic_scene(wavelengths(lo, hi, n), DATA_DIR, sun_elevation_deg=w["sun"])


def make_config(w, args, rank: int = 0):
    """The whole image's config (every rank renders a slab of the same render)."""
    from sky_cuda import RenderConfig
    from sky_cuda import _abi
    return RenderConfig(width=w["width"], height=w["height"], spp=w["spp"], seed=0x5EC7_2026_0430,
                        sun_elevation_deg=w["sun"], phase_sampling=_abi.PHASE_TABULATED,
                        rr_start_depth=w["rr_start_depth"], max_orders=w["max_orders"], tracking=args.tracking,
                        kernel=args.kernel)


def apply_tuning(gs, args):
    """--tuning k=v,...: SkyTuning fields set on a scene the benchmark creates."""
    if getattr(args, "tuning", None):
        gs.set_tuning(**{k: (float(v) if k == "crossing_cost" else int(v))
                         for k, v in (kv.split("=") for kv in args.tuning.split(","))})
    return gs


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except FileNotFoundError:
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)

    def summary(self):
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({names[i] for r in self.rows if len(r) >= 9 for i in range(4) if r[5 + i] == "Active"})
        power = [float(r[3]) for r in self.rows if len(r) > 3 and r[3].replace(".", "").isdigit()]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows),
                "power_w_max": max(power) if power else None}


def measure_fp32_peak(torch, dev):
    """FP32 FMA peak measured with cuBLAS SGEMM (TF32 off), best of 5, TFLOP/s."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    n = 8192
    a = torch.randn(n, n, device=dev, dtype=torch.float32)
    b = torch.randn(n, n, device=dev, dtype=torch.float32)
    c = torch.empty(n, n, device=dev, dtype=torch.float32)
    for _ in range(2):
        torch.matmul(a, b, out=c)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b, out=c)
        e1.record()
        e1.synchronize()
        best = max(best, 2.0 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    torch.backends.cuda.matmul.allow_tf32 = prev
    del a, b, c
    return best


def time_to_1pct(xyz, var, seconds_per_render):
    """Time to 1 % per-pixel XYZ error: the 95th percentile over pixels of the
    worst X/Y/Z relative standard error (pixels with Y < 1e-3 p99(Y)
    excluded), scaled as 1/sqrt(samples)."""
    from sky_cuda.sweep import p95_relative_error
    p95 = p95_relative_error(xyz, var)
    return p95, seconds_per_render * (p95 / 0.01) ** 2


def workload_config(name, w, world):
    """The `config` of both arms' lines: the workload alone (what each arm
    ran it with is in the line's `algorithm` key)."""
    return {"workload": name, "width": w["width"], "height": w["height"], "wavelengths": w["lam"][2],
            "spp": w["spp"], "chains_per_render": w["width"] * w["height"] * w["lam"][2] * w["spp"],
            "sun_elevation_deg": w["sun"], "rr_start_depth": w["rr_start_depth"] or 4,
            "max_orders": w["max_orders"] or "unbounded", "phase_sampling": "tabulated", "projection": "panorama",
            "l2": "GPU arm: L2 flushed between timed steps (256 MB write); scene tables < 1 MB",
            "parallelism": f"row-slabs{world}"}


TRACKING_NAMES = ("segment-restart", "residual-carry", "merged-layers")
# the oracle's random streams: independent of the GPU render's seed
ORACLE_SEED_XOR = 0x9E3779B97F4A7C15


def cpu_baseline_run(w, args, budget_s, tracking=0):
    """The oracle (C++ restatement of the reference shader) on all host cores,
    on a bounded row sample of the same render at full spp, by default in the
    reference's own segment-restart tracking.  Returns a dict: chains/s,
    threads, the sample's description, its duration, and the rows with their
    per-cell sums (for the parity block)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import sky_oracle
    from sky_cuda import RenderConfig
    sky_oracle.load()
    scene = make_scene(w, 0)
    base = make_config(w, args, 0)
    cfg = RenderConfig(**{**base.__dict__, "tracking": tracking, "seed": base.seed ^ ORACLE_SEED_XOR})
    threads = os.cpu_count() or 1
    # pilot: one row at 1/8 of the samples to size the sample
    pilot = RenderConfig(**{**cfg.__dict__, "spp": max(1, cfg.spp // 8)})
    t0 = time.perf_counter()
    sky_oracle.render(scene, pilot, row_begin=cfg.height // 2, row_step=cfg.height, threads=threads)
    pilot_s = time.perf_counter() - t0
    per_row_s = pilot_s * cfg.spp / pilot.spp
    rows = int(max(1, min(cfg.height, budget_s / max(per_row_s, 1e-6))))
    step = max(1, cfg.height // rows)
    t0 = time.perf_counter()
    s, q, _, wd = sky_oracle.render(scene, cfg, row_begin=step // 2, row_step=step, threads=threads)
    dt = time.perf_counter() - t0
    row_ids = list(range(step // 2, cfg.height, step))
    chains = len(row_ids) * cfg.width * scene.band_count * cfg.spp
    return {"value": chains / dt, "threads": threads, "seconds": dt, "chains": chains, "rows": row_ids,
            "sum": s, "sumsq": q, "watchdog": wd, "tracking": TRACKING_NAMES[tracking],
            "sample": (f"every {step}th row ({len(row_ids)} of {cfg.height} rows) at full spp, "
                       f"{TRACKING_NAMES[tracking]} tracking: {chains} chains in {dt:.1f} s")}


def parity_block(scene, cfg, gpu_sum, gpu_sumsq, cpu):
    """Per-pixel XYZ of the GPU render against the oracle's on the rows the
    CPU baseline rendered (independent seeds): the fraction of pixels beyond
    3 combined standard errors, the mean z-score and the summed bias."""
    sys.path.insert(0, str(ROOT / "tests"))
    from skystats import parity_report, xyz_from_sums
    B = scene.band_count
    pix = (np.asarray(cpu["rows"])[:, None] * cfg.width + np.arange(cfg.width)[None, :]).reshape(-1)
    g, gq = gpu_sum.reshape(-1, B)[pix], gpu_sumsq.reshape(-1, B)[pix]
    o, oq = cpu["sum"].reshape(-1, B)[pix], cpu["sumsq"].reshape(-1, B)[pix]
    xg, vg = xyz_from_sums(g, gq, cfg.spp, scene.band_xyz)
    xo, vo = xyz_from_sums(o, oq, cfg.spp, scene.band_xyz)
    r = parity_report(xg, vg, xo, vo)
    return {"against": f"oracle, {cpu['tracking']} tracking, independent seed", "rows": cpu["rows"],
            "pixels_compared": r["pixels"], "frac_beyond_3se": r["frac_beyond_3se"], "mean_z": r["mean_z"],
            "max_abs_z": r["max_abs_z"], "bias_xyz": r["bias_xyz"], "bias_se_xyz": r["bias_se_xyz"],
            "pass": bool(r["frac_beyond_3se"] <= 0.01 and abs(r["mean_z"]) < 0.1)}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    w = WORKLOADS[args.workload]
    import platform
    # each step a bounded sample, sized so that the whole run stays within a few minutes
    budget = min(args.cpu_seconds, max(2.0, 150.0 / max(args.steps, 1)))
    for _ in range(max(1, args.warmup // 3) if args.warmup else 0):
        cpu_baseline_run(w, args, min(2.0, budget))
    runs = [cpu_baseline_run(w, args, budget) for _ in range(args.steps)]
    value = statistics.median(r["value"] for r in runs)
    step_ms = statistics.median(r["seconds"] for r in runs) * 1e3
    # the same oracle with the GPU arm's merged-layer tracking: splits the GPU / CPU ratio into
    # algorithm (tracking) and hardware
    merged = cpu_baseline_run(w, args, budget, tracking=2)
    out = {"impl": "reference", "metric": "spectral path samples/s (chains/s)", "value": value,
           "unit": "chains/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": step_ms,  # one step = one timed row sample of the render
           "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic", "config": workload_config(args.workload, w, world),
           "algorithm": {"tracking": "segment-restart (the reference shader's)", "runs_on": "host CPU, rank 0",
                         "step": "a row sample of the render at full spp (see cpu_baseline.sample)"},
           "cpu_baseline": {"value": value, "unit": "chains/s", "cores": runs[-1]["threads"], "kind": "port",
                            "sample": runs[-1]["sample"], "cpu": platform.processor() or platform.machine()},
           "cpu_merged_layer_tracking": {"value": merged["value"], "unit": "chains/s", "sample": merged["sample"],
                                         "speedup_over_reference_tracking": merged["value"] / value},
           "e2e": {"value": value, "unit": "chains/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "note": "the reference tracer is WGSL run through wgpu, which needs a graphics API absent on "
                   "this machine; this arm times the oracle, a C++ restatement of that shader"}
    print(json.dumps(out))


def sweep_report(args, steps, warmup, rank=0, world=1):
    """Batched elevation sweep (one wavefront launch of 32 jobs replayed as a
    CUDA graph, per-elevation budgets) against 32 separate plain-kernel
    launches and 32 separate single-job wavefront launches.  Under N ranks
    each renders whole elevations, dealt out by their sample budgets (from a
    pilot of all elevations) so that the ranks' totals are close; rank 0's
    assignment is broadcast to all."""
    import torch
    from sky_cuda import GpuScene, RenderConfig, synthetic_scene, wavelengths
    from sky_cuda import _abi
    from sky_cuda.parallel import balanced_shards, broadcast_object, max_over_ranks
    from sky_cuda.sweep import Sweep, elevation_schedule, p95_relative_error, plan_budgets, spp_for_target
    scene = synthetic_scene(wavelengths(380.0, 780.0, 40), DATA_DIR, sun_elevation_deg=10.0)
    base = RenderConfig(width=256, height=128, spp=64, phase_sampling=_abi.PHASE_TABULATED,
                        tracking=args.tracking, rr_start_depth=8, output_projection=_abi.PROJECTION_SKY_VIEW_LUT)
    all_elev = elevation_schedule(32, -6.0, 90.0)
    stream = torch.cuda.current_stream().cuda_stream
    gs = apply_tuning(GpuScene(scene), args)
    all_budgets, pilot_p95 = plan_budgets(gs, base, all_elev, pilot_spp=16)
    # the twilight elevations need up to 16x the samples of the high ones: equal-count blocks
    # would leave rank 0 with ~40 % of the work at N = 8
    shards = broadcast_object(balanced_shards(all_budgets, world) if rank == 0 else None) if world > 1 else None
    mine = shards[rank] if shards else list(range(len(all_elev)))
    elevations = np.asarray(all_elev)[mine]
    budgets = np.asarray(all_budgets)[mine]
    seeded = RenderConfig(**{**base.__dict__, "seed": 0x5EC7_2026_0430})
    sweep = Sweep(gs, seeded, elevations, budgets)
    sweep.capture()
    for _ in range(max(warmup, 1)):
        sweep.replay(stream)
    torch.cuda.synchronize()
    times = []
    for _ in range(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        sweep.replay(stream)
        e1.record()
        e1.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3)
    t_batched = max_over_ranks(statistics.median(times))
    errs_batched = sweep.errors()
    chains_batched = sweep.chains

    # the same elevations as separate launches: one scene per elevation
    singles = [GpuScene(scene.with_sun(float(e))) for e in elevations]
    from sky_cuda.autotune import DEFAULT_SPACE, autotune
    mid = len(singles) // 2
    probe = RenderConfig(**{**base.__dict__, "spp": 256, "sun_elevation_deg": float(elevations[mid]),
                            "kernel": _abi.KERNEL_PLAIN})
    # the plain kernel at its own fastest crossing cost, tuned on the middle elevation
    plain_tuning, _ = autotune(singles[mid], probe, space={"crossing_cost": DEFAULT_SPACE["crossing_cost"]})
    cells = base.pixels * scene.band_count
    bufs = [torch.zeros(cells, dtype=torch.float64, device="cuda") for _ in range(2)]
    xyz = torch.zeros(base.pixels * 3, dtype=torch.float64, device="cuda")
    var = torch.zeros(base.pixels * 3, dtype=torch.float64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")

    def separate_pass(spps, kernel, keep_errors=False):
        errs = []
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for g, e, n in zip(singles, elevations, spps):
            cfg = RenderConfig(**{**seeded.__dict__, "spp": int(n), "sun_elevation_deg": float(e), "kernel": kernel})
            g.render_device(cfg, {"cell_sum": bufs[0].data_ptr(), "cell_sumsq": bufs[1].data_ptr(),
                                  "xyz": xyz.data_ptr(), "xyz_var": var.data_ptr(), "status": status.data_ptr()},
                            stream)
            if keep_errors:
                torch.cuda.synchronize()
                errs.append(p95_relative_error(xyz.cpu().numpy().reshape(-1, 3), var.cpu().numpy().reshape(-1, 3)))
        e1.record()
        e1.synchronize()
        return max_over_ranks(e0.elapsed_time(e1) * 1e-3), errs

    for g in singles:
        g.set_tuning(crossing_cost=plain_tuning["crossing_cost"])
    separate_pass([16] * len(elevations), _abi.KERNEL_PLAIN)  # warm-up
    t_plain_budget, _ = separate_pass(budgets, _abi.KERNEL_PLAIN)
    uniform = int(all_budgets.max())
    t_plain_uniform, errs_plain = separate_pass([uniform] * len(elevations), _abi.KERNEL_PLAIN, keep_errors=True)
    # single-job wavefront launches at the batch's launch shape: what batching alone adds
    shape = gs.get_tuning()
    for g in singles:
        g.set_tuning(variant=shape["variant"], crossing_cost=shape["crossing_cost"])
    separate_pass([16] * len(elevations), _abi.KERNEL_WAVEFRONT)  # warm-up
    t_wave_budget, _ = separate_pass(budgets, _abi.KERNEL_WAVEFRONT)
    # time to bring every elevation to 1 % p95 error, extrapolated (error^2 ~ 1/spp)
    need_b = spp_for_target(errs_batched, budgets, 0.01)
    t1_batched = t_batched * float(need_b.sum()) / float(np.sum(budgets))
    need_u = spp_for_target(errs_plain, [uniform] * len(elevations), 0.01)
    t1_plain_uniform = t_plain_uniform * float(need_u.max()) / uniform
    speed_vs_plain = t_plain_budget / t_batched

    # where batching itself pays: small jobs (one band at 550 nm per elevation, 32 spp: ~1 M
    # chains each), one graph replay of all of them against one single-job launch per job
    small_scene = synthetic_scene(np.array([550.0]), DATA_DIR, sun_elevation_deg=10.0)
    gsm = apply_tuning(GpuScene(small_scene), args)
    small = Sweep(gsm, seeded, elevations, 32)
    small.capture()
    solo = [(c, sun, {**o, "status": small.status.data_ptr()}) for c, sun, o in small.jobs]

    def timed_small(run, reps=5):
        ts = []
        for _ in range(reps + 2):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            run()
            e1.record()
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) * 1e-3)
        return max_over_ranks(statistics.median(ts[2:]))

    t_small_batched = timed_small(lambda: small.replay(stream))
    t_small_singles = timed_small(lambda: [gsm.render_batch([j], stream) for j in solo])
    if int(small.status.item()) != 0:
        raise SystemExit("watchdog tripped in the small-job sweep")
    small_block = {"jobs": len(solo), "chains_per_job": small.chains // max(len(solo), 1),
                   "batched_graph_s": t_small_batched, "single_launches_s": t_small_singles,
                   "speedup_batching": t_small_singles / t_small_batched}
    gsm.close()
    rep = {
        "elevations": [round(float(e), 3) for e in elevations], "spp_per_elevation": [int(b) for b in budgets],
        "pilot_spp": 16, "pilot_p95": [round(float(pilot_p95[i]), 5) for i in mine],
        "batched_graph_s": t_batched, "batched_chains": chains_batched,
        "batched_chains_per_s": chains_batched / t_batched,
        "batched_p95_error_max": max(errs_batched), "batched_p95_error": [round(x, 5) for x in errs_batched],
        "plain_same_budgets_s": t_plain_budget, "plain_same_budgets_chains_per_s": chains_batched / t_plain_budget,
        "wavefront_singles_same_budgets_s": t_wave_budget,
        "wavefront_singles_chains_per_s": chains_batched / t_wave_budget,
        "speedup_chains_per_s_vs_plain_same_error": speed_vs_plain,
        "speedup_batching_alone_vs_wavefront_singles": t_wave_budget / t_batched,
        "plain_uniform_spp": uniform, "plain_uniform_s": t_plain_uniform,
        "plain_uniform_p95_error_max": max(errs_plain),
        "speedup_vs_plain_uniform_at_equal_worst_error": t_plain_uniform / t_batched,
        "time_to_1pct_batched_s": t1_batched, "time_to_1pct_plain_uniform_s": t1_plain_uniform,
        "speedup_time_to_1pct": t1_plain_uniform / t1_batched,
        "target": "batched >= 3x the plain kernel's path samples/s at the same per-elevation error",
        "target_value": speed_vs_plain, "target_met": bool(speed_vs_plain >= 3.0),
        "plain_crossing_cost": round(float(plain_tuning["crossing_cost"]), 3),
        "batched_tuning": shape, "gpu_launches_per_replay": 3,
        "small_jobs": small_block,
    }
    for g in singles:
        g.close()
    gs.close()
    return rep


def run_sweep(args):
    import torch
    import torch.distributed as dist
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    clocks = ClockSampler(local)
    clocks.start()
    rep = sweep_report(args, args.steps, args.warmup, rank, world)
    clocks.stop()
    total = int(sum_over_ranks(rep["batched_chains"]))
    if rank == 0:
        out = {"metric": "spectral path samples/s (chains/s)", "value": total / rep["batched_graph_s"],
               "unit": "chains/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
               "ms_per_step": rep["batched_graph_s"] * 1e3, "higher_is_better": True, "scaling": "strong",
               "vs_baseline": None, "dtype": "f32", "data": "synthetic",
               "config": {"workload": SWEEP_WORKLOAD, "elevations": 32, "width": 256, "height": 128,
                          "wavelengths": 40, "projection": "sky-view LUT", "spp": "64-1024 from a 16-spp pilot",
                          "l2": "outputs > L2 per replay", "parallelism": f"elevation-shards{world}"},
               "algorithm": {"tracking": TRACKING_NAMES[args.tracking]},
               "sweep": rep, "clocks": clocks.summary(), "gpu_launches": 3 * args.steps}
        print(json.dumps(out))
    if world > 1:
        dist.destroy_process_group()


def sum_over_ranks(v):
    """Sum of a per-rank count over ranks (the whole job's chains)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return v
    t = torch.tensor([float(v)], dtype=torch.float64, device="cuda")
    dist.all_reduce(t)
    return float(t.item())


def _sun_pixel_mask(scene, cfg):
    """Panorama pixels whose footprint holds part of the sun disc."""
    x, y, z = scene.sun_direction
    u = math.atan2(x, z) / (2 * math.pi) + 0.5
    v = 0.5 - math.asin(y) / math.pi
    r = scene.sun_angular_radius_rad
    du, dv = r / (2 * math.pi * max(math.cos(math.asin(y)), 1e-3)), r / math.pi
    px = np.arange(cfg.pixels) % cfg.width
    py = np.arange(cfg.pixels) // cfg.width
    return (((px + 1) / cfg.width >= u - du) & (px / cfg.width <= u + du) &
            ((py + 1) / cfg.height >= v - dv) & (py / cfg.height <= v + dv))


def adjoint_report(args, steps, warmup, checks=True):
    """Differentiable render of a 128x64 panorama, 32 wavelengths, 64 spp: L2
    loss on XYZ against a target rendered at perturbed parameters (64 layers x
    3 density scales ~ 1 + N(0, 0.05), seed 3, plus Mie albedo and g), the
    pixels holding the sun disc left out of the loss.  Times
    forward + backward (path replay) and checks the gradient against central
    differences (h = 1e-3, 16 parameters, seed 4) of the same estimator with
    shared samples, against the 4096-spp adjoint gradient, and, along five
    whole-atmosphere directions, against central differences of the plain
    tracer at 4096 spp."""
    import dataclasses
    import torch
    from sky_cuda import GpuScene, RenderConfig, synthetic_scene, wavelengths
    from sky_cuda import _abi
    from sky_cuda.adjoint import (NULL_COLLISIONS, AdjointRenderer, fd_check_parameters, initial_layer_params,
                                  param_names)
    from sky_cuda.scene import SPECIES_COUNT, hg_phase_values
    g0 = 0.76
    scene = synthetic_scene(wavelengths(380.0, 780.0, 32), DATA_DIR, sun_elevation_deg=10.0)
    cfg = RenderConfig(width=128, height=64, spp=64, phase_sampling=_abi.PHASE_TABULATED,
                       tracking=_abi.TRACKING_MERGED_LAYERS, rr_start_depth=8, seed=0x5EC7_2026_0430)
    B, L = scene.band_count, scene.layer_count
    cells = cfg.pixels * B
    dev = torch.device("cuda", 0)
    t = lambda a: torch.as_tensor(np.asarray(a), device=dev, dtype=torch.float32).contiguous()  # noqa: E731
    theta0 = initial_layer_params(scene, g0)
    rng = np.random.default_rng(3)
    theta_t = theta0.copy()
    theta_t[:3 * L] = (1.0 + rng.normal(0.0, 0.05, 3 * L)).astype(np.float32)
    theta_t[3 * L] *= np.float32(1.0 + rng.normal(0.0, 0.02))
    theta_t[3 * L + 1] += np.float32(rng.normal(0.0, 0.02))
    w = torch.as_tensor(np.asarray(scene.band_xyz, np.float64), device=dev)
    gs = apply_tuning(GpuScene(scene), args)
    r = AdjointRenderer(gs, cfg)
    th0 = t(theta0)

    # the pixels holding the sun disc stay out of the loss: rare sun hits dominate their value
    keep = torch.as_tensor(~_sun_pixel_mask(scene, cfg), device=dev, dtype=torch.float64)[:, None]

    def xyz_of(out, spp):
        return (out["cell_sum"] / spp).reshape(cfg.pixels, B) @ w

    tgt = AdjointRenderer(gs, dataclasses.replace(cfg, spp=1024, seed=cfg.seed ^ 0xABCDEF)).forward(t(theta_t))
    txyz = xyz_of(tgt, 1024)

    def dloss(out):
        return (2.0 * keep * (xyz_of(out, cfg.spp) - txyz) @ w.T).float()

    # the forward keeps each chain's radiance (one float per chain), so the backward
    # replays each chain once (as the autograd Function does)
    chain_buf = r.new_chain_buffer()

    def step():
        out = r.forward(th0, check_status=False, chains=chain_buf)
        return out, r.backward(th0, None, dloss(out), check_status=False, chains=chain_buf)

    for _ in range(max(warmup, 1)):
        step()
    torch.cuda.synchronize()
    fwd_ms, bwd_ms, bwd_retrace_ms = [], [], []
    stream = torch.cuda.current_stream()
    for _ in range(steps):
        e0, e1, e2, e3 = (torch.cuda.Event(enable_timing=True) for _ in range(4))
        e0.record(stream)
        out = r.forward(th0, check_status=False, chains=chain_buf)
        e1.record(stream)
        d = dloss(out)
        e_b = torch.cuda.Event(enable_timing=True)
        e_b.record(stream)
        grad, _ = r.backward(th0, None, d, check_status=False, chains=chain_buf)
        e2.record(stream)
        # the same backward without the chain buffer: every chain traced twice
        r.backward(th0, None, d, check_status=False)
        e3.record(stream)
        e3.synchronize()
        fwd_ms.append(e0.elapsed_time(e1))
        bwd_ms.append(e_b.elapsed_time(e2))
        bwd_retrace_ms.append(e2.elapsed_time(e3))
    r._check_status()
    chains = cells * cfg.spp
    f_ms, b_ms = statistics.median(fwd_ms), statistics.median(bwd_ms)
    rep = {"workload": "adjoint-128x64-32wl-64spp", "params": int(theta0.size), "chains_per_render": chains,
           "forward_ms": f_ms, "backward_ms": b_ms, "step_ms": f_ms + b_ms,
           "forward_chains_per_s": chains / (f_ms * 1e-3), "backward_chains_per_s": chains / (b_ms * 1e-3),
           "step_chains_per_s": chains / ((f_ms + b_ms) * 1e-3), "estimator": "segment integrals",
           "chain_buffer_bytes": chains * 4, "backward_ms_without_chain_buffer": statistics.median(bwd_retrace_ms),
           "gpu_launches_per_step": 5}
    if not checks:
        gs.close()
        return rep
    # central differences of the same estimator, samples shared (h = 1e-3, 16 parameters, seed 4)
    rn = AdjointRenderer(gs, cfg, estimator=NULL_COLLISIONS)
    d0 = dloss(rn.forward(th0))
    gnull = rn.backward(th0, None, d0)[0].cpu().numpy()

    def loss_of(out):
        return float((keep * (xyz_of(out, cfg.spp) - txyz) ** 2).sum().item())

    names = param_names(L)
    rows = []
    # 16 parameters that carry a gradient: every species' layer scales, the Mie albedo and g
    for i in fd_check_parameters(gnull, L, count=16, seed=4):
        tp, tm = theta0.copy(), theta0.copy()
        tp[i] += np.float32(1e-3)
        tm[i] -= np.float32(1e-3)
        fd = (loss_of(rn.forward(t(tp), sample_layer=th0)) - loss_of(rn.forward(t(tm), sample_layer=th0))) / \
            float(tp[i] - tm[i])
        rows.append((names[int(i)], fd, float(gnull[i])))
    scale = float(np.abs(gnull).max())
    rel = [abs(fd - g) / abs(fd) if fd else float("inf") for n, fd, g in rows]
    rep["fd_check"] = {
        "h": 1e-3, "params": [[n, fd, g] for n, fd, g in rows], "estimator": "null collisions",
        "selection": "seed 4, evenly over Rayleigh / Mie / ozone layer scales with a gradient, plus albedo and g",
        "max_rel_err": max(rel), "all_within_1e-2": bool(max(rel) <= 1e-2),
        "max_abs_err_over_max_grad": max(abs(fd - g) for n, fd, g in rows) / scale}
    # the 64-spp gradient against the 4096-spp gradient with the same dLoss/dfilm
    batches, bspp = 16, 256
    dfix = d0.clone()
    g64 = r.backward(th0, None, dfix)[0].cpu().numpy()
    gref = np.zeros_like(g64)
    for k in range(batches):
        rk = AdjointRenderer(gs, dataclasses.replace(cfg, spp=bspp, sample_offset=k * bspp))
        gref += rk.backward(th0, None, dfix)[0].cpu().numpy() / batches
    rep["vs_4096spp"] = {"rel_l2_err_64spp": float(np.linalg.norm(g64 - gref) / np.linalg.norm(gref)),
                         "cosine_64spp": float(g64 @ gref / (np.linalg.norm(g64) * np.linalg.norm(gref)))}
    # the plain tracer at 4096 spp along whole-atmosphere directions (linearised loss, sun disc excluded)
    wcell = dfix.double().reshape(cfg.pixels, B).cpu().numpy()
    wcell[_sun_pixel_mask(scene, cfg)] = 0.0
    wt = torch.as_tensor(wcell.reshape(-1), device=dev, dtype=torch.float32)
    dirs = {"rayleigh": (0.05, lambda g: g[0:3 * L:3].sum()), "mie": (0.05, lambda g: g[1:3 * L:3].sum()),
            "ozone": (0.2, lambda g: g[2:3 * L:3].sum()), "albedo": (0.02, lambda g: g[3 * L]),
            "g": (0.02, lambda g: g[3 * L + 1])}

    def moved(direction, delta):
        s = dataclasses.replace(scene)
        bands, optics, phase = scene.bands.copy(), scene.aerosol_optics.copy(), scene.phase_values.copy()
        sca = optics["scattering_km_inv_per_g_m3"][0::SPECIES_COUNT].astype(np.float64)
        ab = optics["absorption_km_inv_per_g_m3"][0::SPECIES_COUNT].astype(np.float64)
        if direction == "rayleigh":
            bands["rayleigh_cross_section_m2"] *= np.float32(1 + delta)
        elif direction == "mie":
            optics["scattering_km_inv_per_g_m3"][0::SPECIES_COUNT] = sca * (1 + delta)
            optics["absorption_km_inv_per_g_m3"][0::SPECIES_COUNT] = ab * (1 + delta)
        elif direction == "ozone":
            bands["ozone_cross_section_cm2"] *= np.float32(1 + delta)
        elif direction == "albedo":
            ext = sca + ab
            optics["scattering_km_inv_per_g_m3"][0::SPECIES_COUNT] = ext * (sca / ext + delta)
            optics["absorption_km_inv_per_g_m3"][0::SPECIES_COUNT] = ext * (1 - sca / ext - delta)
        else:
            phase[0] = hg_phase_values(g0 + delta, scene.phase_bins)[None, :]
        s.bands, s.aerosol_optics, s.phase_values = bands, optics, phase
        return s.bake_majorants(L)

    wnp = wcell.reshape(-1)
    plain = {}
    for name, (delta, proj) in dirs.items():
        gp = apply_tuning(GpuScene(moved(name, delta)), args)
        gm = apply_tuning(GpuScene(moved(name, -delta)), args)
        fd, adj = [], []
        for k in range(batches):
            c = dataclasses.replace(cfg, spp=bspp, sample_offset=k * bspp)
            js = []
            for g in (gp, gm):
                sm = torch.zeros(cells, dtype=torch.float64, device=dev)
                st = torch.zeros(1, dtype=torch.int32, device=dev)
                g.render_device(c, {"cell_sum": sm.data_ptr(), "status": st.data_ptr()}, stream.cuda_stream)
                torch.cuda.synchronize()
                js.append(float(sm.cpu().numpy() @ wnp) / bspp)
            fd.append((js[0] - js[1]) / (2 * delta))
            rk = AdjointRenderer(gs, c)
            adj.append(float(proj(rk.backward(th0, None, wt)[0].cpu().numpy())))
        gp.close()
        gm.close()
        fd, adj = np.array(fd), np.array(adj)
        se_fd, se_adj = fd.std(ddof=1) / math.sqrt(batches), adj.std(ddof=1) / math.sqrt(batches)
        plain[name] = {"delta": delta, "plain_fd": float(fd.mean()), "plain_fd_se": float(se_fd),
                       "adjoint": float(adj.mean()), "adjoint_se": float(se_adj),
                       "z": float((adj.mean() - fd.mean()) / math.hypot(se_fd, se_adj))}
    rep["vs_plain_tracer_4096spp"] = plain
    gs.close()
    return rep


def run_adjoint(args):
    import torch
    torch.cuda.set_device(0)
    clocks = ClockSampler(0)
    clocks.start()
    rep = adjoint_report(args, args.steps, args.warmup, checks=not args.no_adjoint_checks)
    clocks.stop()
    out = {"metric": "spectral path samples/s (chains/s), forward + path-replay backward",
           "value": rep["step_chains_per_s"], "unit": "chains/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": rep["step_ms"], "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": ADJOINT_WORKLOAD, "width": 128, "height": 64, "wavelengths": 32, "spp": 64,
                      "l2": "tables < 1 MB; compute-bound"},
           "adjoint": rep, "clocks": clocks.summary(), "gpu_launches": 5 * args.steps}
    print(json.dumps(out))


def fit_report(args, iterations):
    """Wavelength-primary fit driven by the adjoint against the same fit
    driven by central differences of the plain tracer: final error of each
    (plain-tracer evaluation at the target's sample count) and wall time.
    The Oklab score of the reference optimizer (main.rs:414-488) is the
    acceptance metric; the debiased relative RMS XYZ error is reported with
    its resolution (the Monte Carlo noise left after the subtraction)."""
    from sky_cuda.primaries import PrimaryFitConfig, evaluate, fit_adjoint, fit_finite_differences, target_xyz
    cfg = PrimaryFitConfig(data_dir=str(DATA_DIR), iterations=iterations)
    t0 = time.perf_counter()
    target, target_var = target_xyz(cfg)
    t_target = time.perf_counter() - t0
    start = fit_adjoint(cfg, target, iterations=0)
    adj = fit_adjoint(cfg, target)
    fd = fit_finite_differences(cfg, target)
    res = {}
    for name, fit in (("initial", start), ("adjoint", adj), ("finite_differences", fd)):
        ev = evaluate(cfg, fit["lambda_nm"], fit["matrix"], target, target_var)
        res[name] = {"lambda_nm": [round(float(v), 3) for v in fit["lambda_nm"]],
                     "min_spacing_nm": round(float(np.min(np.diff(np.sort(fit["lambda_nm"])))), 3),
                     "oklab_score": ev["oklab"]["score"], "oklab": ev["oklab"],
                     "relative_xyz_error": ev["relative_xyz_error"],
                     "relative_rms_error": ev["relative_rms_error"],
                     "relative_rms_error_debiased": ev["relative_rms_error_debiased"],
                     "relative_rms_resolution": ev["relative_rms_resolution"],
                     "relative_rms_noise": ev["relative_rms_noise"],
                     "wall_s": fit["seconds"], "setup_s": fit["setup_seconds"], "iterations": fit["iterations"],
                     "loss_first": fit["loss"][0] if fit["loss"] else None,
                     "loss_last": fit["loss"][-1] if fit["loss"] else None}
    return {"workload": FIT_WORKLOAD, "iterations": iterations, "target_render_s": t_target,
            "elevations": len(cfg.elevations), "fit_spp": cfg.fit_spp, "target_spp": cfg.target_spp,
            "min_spacing_nm": cfg.min_spacing_nm, "loss": cfg.loss, "acceptance": "Oklab score (lower is better)",
            "fit": res, "speedup_wall_adjoint_vs_fd": fd["seconds"] / adj["seconds"] if adj["seconds"] else None,
            "adjoint_ms_per_iteration": adj["seconds"] / max(iterations, 1) * 1e3}


def run_fit(args):
    import torch
    torch.cuda.set_device(0)
    clocks = ClockSampler(0)
    clocks.start()
    rep = fit_report(args, args.fit_iterations)
    clocks.stop()
    out = {"metric": "wavelength-primary fit: Oklab score of the fitted primaries (adjoint-driven)",
           "value": rep["fit"]["adjoint"]["oklab_score"], "unit": "Oklab score", "n_gpus": 1,
           "steps": args.fit_iterations, "warmup": 0, "ms_per_step": rep["adjoint_ms_per_iteration"],
           "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": FIT_WORKLOAD, "elevations": rep["elevations"], "width": 256, "height": 128,
                      "fit_spp": rep["fit_spp"], "target_wavelengths": 81, "target_spp": rep["target_spp"],
                      "projection": "sky-view LUT", "l2": "n/a (compute-bound)", "parallelism": "single GPU"},
           "fit": rep, "clocks": clocks.summary(), "gpu_launches": None}
    print(json.dumps(out))


def main():
    args = parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == SWEEP_WORKLOAD:
        return run_sweep(args)
    if args.workload == ADJOINT_WORKLOAD:
        return run_adjoint(args)
    if args.workload == FIT_WORKLOAD:
        return run_fit(args)
    import torch
    import torch.distributed as dist
    from sky_cuda import GpuScene, render
    from sky_cuda import _abi
    from sky_cuda.parallel import (balanced_row_slabs, broadcast_object, broadcast_slabs, gather_to_rank0,
                                   max_over_ranks, pilot_row_costs, slab_config)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    w = WORKLOADS[args.workload]
    scene = make_scene(w)
    full = make_config(w, args)
    gs = apply_tuning(GpuScene(scene), args)
    # one render split into contiguous pixel-row slabs, one per rank (the whole image at N = 1):
    # slabs of equal cost from rank 0's pilot render, broadcast to every rank
    slabs, slab_log = None, "whole image"
    if world > 1:
        if args.equal_slabs:
            slab_log = "equal rows"
        else:
            if rank == 0:
                t0 = time.perf_counter()
                slabs = balanced_row_slabs(pilot_row_costs(gs, full), world)
                slab_log = f"cost-balanced: pilot of 16 row blocks at 32 spp on rank 0, {time.perf_counter() - t0:.2f} s"
            slabs = broadcast_slabs(slabs)
            slab_log = broadcast_object(slab_log)
    cfg = slab_config(full, rank, world, slabs)
    B = scene.band_count
    cells = cfg.pixels * B
    full_chains = full.pixels * B * full.spp

    tuning_log = None
    if not args.no_autotune:
        from sky_cuda.autotune import DEFAULT_SPACE, autotune
        t0 = time.perf_counter()
        # the plain kernel has one shape: only its crossing cost is tuned
        space = None if cfg.kernel != 1 else {"crossing_cost": DEFAULT_SPACE["crossing_cost"]}
        best, trials = autotune(gs, cfg, space=space)
        tuning_log = {"chosen": best, "seconds": round(time.perf_counter() - t0, 2),
                      "trials": [[t["variant"], round(t["crossing_cost"], 3), round(ms, 3)]
                                 for t, ms in trials]}
    stream = torch.cuda.current_stream(dev)
    s = torch.zeros(cells, dtype=torch.float64, device=dev)
    q = torch.zeros(cells, dtype=torch.float64, device=dev)
    film = torch.zeros(cells, dtype=torch.float32, device=dev)
    xyz = torch.zeros(cfg.pixels * 3, dtype=torch.float64, device=dev)
    xyz_var = torch.zeros(cfg.pixels * 3, dtype=torch.float64, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    counters = torch.zeros(8, dtype=torch.int64, device=dev)
    outs = {"cell_sum": s.data_ptr(), "cell_sumsq": q.data_ptr(), "film": film.data_ptr(), "xyz": xyz.data_ptr(),
            "xyz_var": xyz_var.data_ptr(), "status": status.data_ptr()}
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > 129 MB L2

    # warm-up; the first step also counts events (identical work: same seed)
    for i in range(max(args.warmup, 1)):
        o = dict(outs)
        if i == 0:
            o["counters"] = counters.data_ptr()
        gs.render_device(cfg, o, stream.cuda_stream)
    torch.cuda.synchronize()
    if int(status.item()) != 0:
        raise SystemExit("watchdog tripped during warm-up")
    ev = {k: int(v) for k, v in zip(_abi.EVENT_NAMES, counters.cpu().tolist())}
    flops_per_step = sum(EVENT_FLOPS[k] * ev[k] for k in EVENT_FLOPS)

    clocks = ClockSampler(local)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    times = []
    for _ in range(args.steps):
        flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        gs.render_device(cfg, outs, stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3)
    torch.cuda.synchronize()
    clocks.stop()
    if world > 1:
        dist.barrier()
    own_step_s = sum(times) / args.steps
    step_s = max_over_ranks(own_step_s, dev)
    value = full_chains / step_s
    if int(status.item()) != 0:
        raise SystemExit("watchdog tripped during the timed renders")

    # time to 1 % XYZ error from the last render (rank 0's slab)
    p95, t1pct = time_to_1pct(xyz.cpu().numpy().reshape(-1, 3), xyz_var.cpu().numpy().reshape(-1, 3), step_s)
    # the slabs joined on rank 0 make the whole film
    parts = gather_to_rank0(film.cpu().numpy()) if world > 1 else None
    if parts is not None:
        assert sum(p.size for p in parts) == full.pixels * B

    # end to end through the one-shot C ABI (host tables in, host film out), each rank its slab,
    # joined on rank 0
    e2e_times = []
    for i in range(args.e2e_steps + 1 if args.e2e_steps > 0 else 0):
        if world > 1:
            dist.barrier()
        t0 = time.perf_counter()
        part = render(scene, cfg).values
        if world > 1:
            joined = gather_to_rank0(part)
            if joined is not None:
                np.concatenate(joined)
        dt = time.perf_counter() - t0
        if i > 0:
            e2e_times.append(dt)
    desc_bytes = sum(a.nbytes for a in scene._keep)
    e2e_s = max_over_ranks(statistics.median(e2e_times), dev) if e2e_times else float("nan")

    blocks = {}
    if rank == 0 and world == 1:
        peak = None if args.no_peak else measure_fp32_peak(torch, dev)
        if not args.no_cpu_baseline:
            import platform
            cpu = cpu_baseline_run(w, args, args.cpu_seconds)
            merged = cpu_baseline_run(w, args, args.cpu_seconds / 3, tracking=2)
            blocks["cpu_baseline"] = {
                "value": cpu["value"], "unit": "chains/s", "cores": cpu["threads"], "kind": "port",
                "sample": cpu["sample"], "cpu": platform.machine(),
                "value_merged_layer_tracking": merged["value"], "sample_merged_layer_tracking": merged["sample"]}
            blocks["parity"] = parity_block(scene, cfg, s.cpu().numpy(), q.cpu().numpy(), cpu)
        if not args.no_adjoint:
            blocks["adjoint"] = adjoint_report(args, 3, 2)
        if not args.no_sweep:
            blocks["sweep"] = sweep_report(args, 2, 1)
        if args.fit_summary_iterations > 0:
            blocks["fit"] = fit_report(args, args.fit_summary_iterations)
    else:
        peak = None
    if rank == 0:
        achieved = flops_per_step / own_step_s / 1e12
        out = {
            "metric": "spectral path samples/s (chains/s)", "value": value, "unit": "chains/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(args.workload, w, world),
            "algorithm": {"tracking": TRACKING_NAMES[cfg.tracking],
                          "kernel": ("wavefront", "plain", "wavefront")[cfg.kernel],
                          "slab_rows": [cfg.row_begin, cfg.rows], "slabs": slab_log, "tuning": gs.get_tuning(),
                          "autotune": tuning_log},
            "e2e": {"value": full_chains / e2e_s if e2e_times else None, "unit": "chains/s",
                    "h2d_bytes_per_step": int(desc_bytes),
                    "d2h_bytes_per_step": int(cells * 4 + 8 * 8 + 4)},
            "time_to_1pct_xyz_s": t1pct, "p95_rel_se_at_spp": p95,
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak if peak else None,
                         # the captured traffic is one launch over the whole image (N = 1)
                         "traffic": WAVE_LAUNCH_DRAM_BYTES.get(args.workload)
                         if cfg.kernel != 1 and world == 1 else None,
                         "scope": "the whole render" if world == 1 else "rank 0's slab",
                         "traffic_unit": "bytes per launch (ncu dram__bytes_read.sum + dram__bytes_write.sum)",
                         "peak_source": "measured: cuBLAS SGEMM 8192^3 with TF32 off (MEASURED_PEAKS.json "
                                        "has no FP32 figure)",
                         "flops_per_step": flops_per_step, "events_per_step": ev},
            "cpu_baseline": blocks.get("cpu_baseline"),
            "parity": blocks.get("parity"),
            "adjoint": blocks.get("adjoint"),
            "sweep": blocks.get("sweep"),
            "fit": blocks.get("fit"),
            "clocks": clocks.summary(),
            "gpu_launches": (2 if cfg.kernel == 1 else 3) * args.steps,
        }
        print(json.dumps(out))
    gs.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
