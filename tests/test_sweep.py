"""Batched sweeps: CPU checks of the sweep schedule and budgets, GPU checks
that a batch renders exactly what separate renders with the same suns do."""

import numpy as np
import pytest

from sky_cuda import GpuScene, RenderConfig, sun_from_degrees
from sky_cuda import _abi
from sky_cuda.sweep import Sweep, budgets_from_pilot, elevation_schedule, p95_relative_error, plan_budgets


def test_elevation_schedule_is_dense_near_the_horizon():
    e = elevation_schedule(32, -6.0, 90.0)
    assert e[0] == -6.0 and e[-1] == 90.0 and len(e) == 32
    d = np.diff(e)
    assert np.all(d > 0) and np.all(np.diff(d) > 0)


def test_budgets_are_proportional_rounded_and_clamped():
    p95 = np.array([0.01, 0.02, 0.04, 0.2, 0.001])
    spp = budgets_from_pilot(p95, 16, jitter=0.0)
    assert list(spp) == [64, 64, 256, 1024, 64]
    spp_j = budgets_from_pilot(np.full(8, 0.05), 16, seed=2026)
    assert np.all(spp_j % 32 == 0) and np.all((spp_j >= 64) & (spp_j <= 1024))
    assert np.array_equal(spp_j, budgets_from_pilot(np.full(8, 0.05), 16, seed=2026))


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
def test_batch_equals_separate_renders(gpu, cfg0_scene):
    import torch
    base = RenderConfig(width=24, height=12, spp=32, phase_sampling=_abi.PHASE_TABULATED,
                        tracking=_abi.TRACKING_MERGED_LAYERS, output_projection=_abi.PROJECTION_SKY_VIEW_LUT)
    elevations = [-3.0, 2.0, 45.0]
    spp = [32, 64, 16]
    with GpuScene(cfg0_scene) as gs:
        sweep = Sweep(gs, base, elevations, spp)
        sweep.launch(torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        assert int(sweep.status.item()) == 0
        assert int(sweep.counters[6].item()) == sweep.chains
        got = [(o.cell_sum.cpu().numpy(), o.cell_sumsq.cpu().numpy()) for o in sweep.out]
    for e, n, (s, q) in zip(elevations, spp, got):
        with GpuScene(cfg0_scene.with_sun(e)) as single:
            rs, rq = _sums(single, RenderConfig(**{**base.__dict__, "spp": n, "sun_elevation_deg": e}))
        np.testing.assert_allclose(s, rs, rtol=1e-12, atol=0)
        np.testing.assert_allclose(q, rq, rtol=1e-12, atol=0)


@pytest.mark.gpu
def test_graph_replay_equals_batch(gpu, cfg0_scene):
    import torch
    base = RenderConfig(width=16, height=16, spp=32, phase_sampling=_abi.PHASE_TABULATED,
                        tracking=_abi.TRACKING_MERGED_LAYERS, output_projection=_abi.PROJECTION_SKY_VIEW_LUT)
    with GpuScene(cfg0_scene) as gs:
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
def test_pilot_budgets_reach_the_target(gpu, cfg0_scene):
    import torch
    base = RenderConfig(width=32, height=16, spp=16, phase_sampling=_abi.PHASE_TABULATED,
                        tracking=_abi.TRACKING_MERGED_LAYERS, output_projection=_abi.PROJECTION_SKY_VIEW_LUT)
    with GpuScene(cfg0_scene) as gs:
        elevations = [-4.0, 5.0, 40.0]
        spp, p95 = plan_budgets(gs, base, elevations, pilot_spp=16, target=0.02, lo=32, hi=4096)
        sweep = Sweep(gs, RenderConfig(**{**base.__dict__, "seed": 99}), elevations, spp)
        sweep.launch(torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        errs = sweep.errors()
    assert np.all(spp % 32 == 0)
    assert max(errs) < 0.02 * 1.3, (spp, p95, errs)
