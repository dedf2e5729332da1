"""Batched sweeps: CPU checks of the sweep schedule and budgets, GPU checks
that a batch renders exactly what separate renders with the same suns do."""

import numpy as np
import pytest

from sky_cuda import GpuScene, RenderConfig, sun_from_degrees
from sky_cuda import _abi
from sky_cuda.sweep import (Sweep, budgets_from_pilot, elevation_schedule, p95_relative_error, plan_budgets,
                             spp_for_target)


def test_elevation_schedule_is_dense_near_the_horizon():
    e = elevation_schedule(32, -6.0, 90.0)
    assert e[0] == -6.0 and e[-1] == 90.0 and len(e) == 32
    d = np.diff(e)
    assert np.all(d > 0) and np.all(np.diff(d) > 0)


def test_budgets_are_proportional_rounded_and_clamped():
    p95 = np.array([0.4, 0.2, 0.1, 0.05, 0.2 * np.sqrt(0.5)])
    spp = budgets_from_pilot(p95, jitter=0.0)
    assert list(spp) == [1024, 256, 64, 64, 128]
    spp_j = budgets_from_pilot(np.linspace(0.05, 0.3, 8), seed=2026)
    assert np.all(spp_j % 32 == 0) and np.all((spp_j >= 64) & (spp_j <= 1024)) and spp_j[-1] >= 992
    assert np.array_equal(spp_j, budgets_from_pilot(np.linspace(0.05, 0.3, 8), seed=2026))
    assert np.allclose(spp_for_target([0.1, 0.02], [100, 100], 0.01), [10000.0, 400.0])


def test_p95_relative_error_excludes_dark_pixels():
    xyz = np.array([[1.0, 1.0, 1.0]] * 99 + [[0.0, 1e-9, 0.0]])
    var = np.array([[1e-4, 1e-4, 1e-4]] * 99 + [[1.0, 1.0, 1.0]])
    assert abs(p95_relative_error(xyz, var) - 0.01) < 1e-12


def _sums(gs, cfg):
    import torch
    cells = cfg.pixels * gs.band_count
    s = torch.zeros(cells, dtype=torch.float64, device="cuda")
    q = torch.zeros(cells, dtype=torch.float64, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    gs.render_device(cfg, {"cell_sum": s.data_ptr(), "cell_sumsq": q.data_ptr(), "status": st.data_ptr()},
                     torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return s.cpu().numpy(), q.cpu().numpy()


@pytest.mark.gpu
def test_batch_equals_separate_renders(gpu, dome_scene):
    import torch
    base = RenderConfig(width=24, height=12, spp=32, phase_sampling=_abi.PHASE_TABULATED,
                        tracking=_abi.TRACKING_MERGED_LAYERS, output_projection=_abi.PROJECTION_SKY_VIEW_LUT)
    elevations = [-3.0, 2.0, 45.0]
    spp = [32, 64, 16]
    with GpuScene(dome_scene) as gs:
        sweep = Sweep(gs, base, elevations, spp, count_events=True)
        sweep.launch(torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        assert int(sweep.status.item()) == 0
        assert int(sweep.counters[6].item()) == sweep.chains
        got = [(o.cell_sum.cpu().numpy(), o.cell_sumsq.cpu().numpy()) for o in sweep.out]
    for e, n, (s, q) in zip(elevations, spp, got):
        with GpuScene(dome_scene.with_sun(e)) as single:
            rs, rq = _sums(single, RenderConfig(**{**base.__dict__, "spp": n, "sun_elevation_deg": e}))
        np.testing.assert_allclose(s, rs, rtol=1e-12, atol=0)
        np.testing.assert_allclose(q, rq, rtol=1e-12, atol=0)


@pytest.mark.gpu
def test_graph_replay_equals_batch(gpu, dome_scene):
    import torch
    base = RenderConfig(width=16, height=16, spp=32, phase_sampling=_abi.PHASE_TABULATED,
                        tracking=_abi.TRACKING_MERGED_LAYERS, output_projection=_abi.PROJECTION_SKY_VIEW_LUT)
    with GpuScene(dome_scene) as gs:
        sweep = Sweep(gs, base, [0.0, 10.0, 60.0], [32, 64, 32])
        stream = torch.cuda.current_stream().cuda_stream
        sweep.launch(stream)
        torch.cuda.synchronize()
        want = [o.cell_sum.cpu().numpy().copy() for o in sweep.out]
        sweep.capture()
        for _ in range(2):
            for o in sweep.out:
                o.cell_sum.zero_()
            sweep.replay(stream)
            torch.cuda.synchronize()
            for o, w in zip(sweep.out, want):
                np.testing.assert_allclose(o.cell_sum.cpu().numpy(), w, rtol=1e-12, atol=0)
        assert int(sweep.status.item()) == 0


@pytest.mark.gpu
def test_pilot_budgets_equalise_errors(gpu, dome_scene):
    """Budgets proportional to the pilot's variance give the sweep's jobs
    about the same error (the sun above the horizon, where a 16-spp pilot
    estimates the error well)."""
    import torch
    base = RenderConfig(width=32, height=16, spp=16, phase_sampling=_abi.PHASE_TABULATED,
                        tracking=_abi.TRACKING_MERGED_LAYERS, output_projection=_abi.PROJECTION_SKY_VIEW_LUT)
    with GpuScene(dome_scene) as gs:
        elevations = [3.0, 15.0, 60.0]
        spp, p95 = plan_budgets(gs, base, elevations, pilot_spp=64, lo=32, hi=2048, jitter=0.0)
        sweep = Sweep(gs, RenderConfig(**{**base.__dict__, "seed": 99}), elevations, spp)
        sweep.launch(torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        errs = np.array(sweep.errors())
    assert np.all(spp % 32 == 0) and spp.max() == 2048
    assert errs.max() / errs.min() < 1.6, (spp, p95, errs)


@pytest.mark.gpu
@pytest.mark.parametrize("elevation", [4.0, 35.0])
def test_single_job_batch_uses_its_own_sun(gpu, dome_scene, elevation):
    """A one-job batch runs the single-job kernel, which takes the sun frame
    from the job's own scene parameters: with a sun other than the scene's it
    still renders what a scene with that sun renders."""
    import torch
    base = RenderConfig(width=24, height=12, spp=32, phase_sampling=_abi.PHASE_TABULATED,
                        tracking=_abi.TRACKING_MERGED_LAYERS, output_projection=_abi.PROJECTION_SKY_VIEW_LUT)
    with GpuScene(dome_scene) as gs:
        sweep = Sweep(gs, base, [elevation], [32])
        sweep.launch(torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        assert int(sweep.status.item()) == 0
        s = sweep.out[0].cell_sum.cpu().numpy()
    with GpuScene(dome_scene.with_sun(elevation)) as single:
        rs, _ = _sums(single, RenderConfig(**{**base.__dict__, "sun_elevation_deg": elevation}))
    np.testing.assert_allclose(s, rs, rtol=1e-12, atol=0)
