"""GPU parity: the CUDA tracer, called through the C ABI, against the oracle
and against analytic answers.  Runs on the GB300 machine (`-m gpu`)."""

import math

import numpy as np
import pytest

import analytic
import sky_oracle as oracle
from sky_cuda import (FLAG_ACCUMULATE, GpuScene, RenderConfig, RenderWatchdog, SkyCudaError, SyntheticAtmosphere,
                      render, synthetic_scene, wavelengths)
from sky_cuda import _abi
from skystats import parity_report, xyz_from_sums

pytestmark = pytest.mark.gpu

MODES = [(t, p) for t in (_abi.TRACKING_SEGMENT_RESTART, _abi.TRACKING_RESIDUAL_CARRY,
                          _abi.TRACKING_MERGED_LAYERS)
         for p in (_abi.PHASE_ISOTROPIC, _abi.PHASE_TABULATED)]


def gpu_sums(gs: GpuScene, cfg: RenderConfig):
    import torch
    cells = cfg.pixels * gs.band_count
    s = torch.zeros(cells, dtype=torch.float64, device="cuda")
    q = torch.zeros(cells, dtype=torch.float64, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    ctr = torch.zeros(8, dtype=torch.int64, device="cuda")
    gs.render_device(cfg, {"cell_sum": s.data_ptr(), "cell_sumsq": q.data_ptr(), "status": st.data_ptr(),
                           "counters": ctr.data_ptr()}, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    shape = (cfg.pixels, gs.band_count)
    return s.cpu().numpy().reshape(shape), q.cpu().numpy().reshape(shape), ctr.cpu().numpy(), int(st.item())


def test_smoke_film(gpu, ref_scene):
    # smoke.rs:7-24 through the one-shot entry point
    film = render(ref_scene, RenderConfig(width=32, height=16, spp=2))
    v = film.values
    assert v.shape == (32 * 16 * 41,)
    assert np.all(np.isfinite(v)) and np.all(v >= 0) and np.any(v > 0)


KERNELS = (_abi.KERNEL_PLAIN, _abi.KERNEL_WAVEFRONT)


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("tracking,phase", MODES)
def test_chains_match_oracle(gpu, dome_scene, tracking, phase, kernel):
    """One sample per cell: each GPU chain against the oracle's chain with the
    same counter-based random stream.  Differences come only from rounding
    (fast-math intrinsics, the impact-parameter geometry), which flips a
    decision in a small fraction of chains."""
    agree = total = 0
    with GpuScene(dome_scene) as gs:
        for offset in (0, 7, 1000):
            cfg = RenderConfig(width=16, height=8, spp=1, sample_offset=offset, seed=0x5EC7_2026_0430 + offset,
                               phase_sampling=phase, tracking=tracking, max_orders=16, kernel=kernel)
            g, _, _, st = gpu_sums(gs, cfg)
            o, _, _, wd = oracle.render(dome_scene, cfg)
            assert st == 0 and wd == 0
            close = np.abs(g - o) <= 2e-3 * np.maximum(np.abs(g), np.abs(o)) + 1e-9
            agree += int(close.sum())
            total += close.size
    frac = agree / total
    print(f"chain agreement kernel={kernel} tracking={tracking} phase={phase}: {frac:.4f} of {total}")
    assert frac >= 0.95


@pytest.mark.parametrize("kernel", KERNELS)
def test_sky_view_lut_chains_match_oracle(gpu, dome_scene, kernel):
    """The sky-view LUT camera (sky_trace.wgsl:625-681), chain by chain against
    the oracle, with the sun off the LUT's axis so that the sun-aligned azimuth
    frame matters."""
    agree = total = 0
    with GpuScene(dome_scene) as gs:
        for offset in (0, 9):
            cfg = RenderConfig(width=16, height=12, spp=1, sample_offset=offset, seed=0x5EC7_2026_0430 + offset,
                               phase_sampling=_abi.PHASE_TABULATED, tracking=_abi.TRACKING_MERGED_LAYERS,
                               max_orders=16, kernel=kernel, output_projection=_abi.PROJECTION_SKY_VIEW_LUT,
                               observer_altitude_km=0.3)
            g, _, _, st = gpu_sums(gs, cfg)
            o, _, _, wd = oracle.render(dome_scene, cfg)
            assert st == 0 and wd == 0
            close = np.abs(g - o) <= 2e-3 * np.maximum(np.abs(g), np.abs(o)) + 1e-9
            agree += int(close.sum())
            total += close.size
    frac = agree / total
    print(f"sky-view LUT chain agreement kernel={kernel}: {frac:.4f} of {total}")
    assert frac >= 0.95


@pytest.mark.parametrize("kernel", KERNELS)
def test_several_light_samples_match_oracle(gpu, dome_scene, kernel):
    """Three sun samples per vertex (direct_sun_at_scatter / ground_radiance
    loop over direct_light_samples, sky_trace.wgsl:566-608): the wavefront
    kernel traces them as successive shadow rays of one vertex; chain by chain
    against the oracle."""
    agree = total = 0
    with GpuScene(dome_scene) as gs:
        for offset in (0, 5):
            cfg = RenderConfig(width=16, height=8, spp=1, sample_offset=offset, seed=0x5EC7_2026_0430 + offset,
                               phase_sampling=_abi.PHASE_TABULATED, tracking=_abi.TRACKING_MERGED_LAYERS,
                               max_orders=16, kernel=kernel, direct_light_samples=3)
            g, _, _, st = gpu_sums(gs, cfg)
            o, _, _, wd = oracle.render(dome_scene, cfg)
            assert st == 0 and wd == 0
            close = np.abs(g - o) <= 2e-3 * np.maximum(np.abs(g), np.abs(o)) + 1e-9
            agree += int(close.sum())
            total += close.size
    frac = agree / total
    print(f"three light samples, chain agreement kernel={kernel}: {frac:.4f} of {total}")
    assert frac >= 0.95


@pytest.mark.parametrize("phase", [_abi.PHASE_ISOTROPIC, _abi.PHASE_TABULATED])
@pytest.mark.parametrize("tracking", [_abi.TRACKING_RESIDUAL_CARRY, _abi.TRACKING_MERGED_LAYERS])
def test_wavefront_matches_plain_chains(gpu, dome_scene, tracking, phase):
    """The persistent kernel consumes each chain's random stream in the plain
    kernel's order: chain by chain, the two kernels trace the same paths."""
    with GpuScene(dome_scene) as gs:
        cfg = RenderConfig(width=32, height=16, spp=1, sample_offset=3, phase_sampling=phase, tracking=tracking,
                           max_orders=16, rr_start_depth=8)
        a, _, ca, _ = gpu_sums(gs, RenderConfig(**{**cfg.__dict__, "kernel": _abi.KERNEL_PLAIN}))
        b, _, cb, _ = gpu_sums(gs, RenderConfig(**{**cfg.__dict__, "kernel": _abi.KERNEL_WAVEFRONT}))
    close = np.abs(a - b) <= 1e-5 * np.maximum(np.abs(a), np.abs(b)) + 1e-12
    print(f"plain/wavefront chain agreement tracking={tracking} phase={phase}: {close.mean():.5f}")
    assert close.mean() >= 0.999
    np.testing.assert_allclose(ca[:7], cb[:7], rtol=2e-3)


@pytest.mark.parametrize("tracking,phase", [MODES[0], MODES[3], MODES[5]])
def test_statistical_parity_dome(gpu, dome_scene, tracking, phase):
    """The CPU-runnable benchmark scene (64x32, 32 bands, 64 spp): per-pixel
    XYZ of GPU and oracle within 3 combined standard errors, and no bias."""
    cfg = RenderConfig(width=64, height=32, spp=64, sun_elevation_deg=10.0, phase_sampling=phase,
                       tracking=tracking, max_orders=16)
    with GpuScene(dome_scene) as gs:
        gs_, gq, _, st = gpu_sums(gs, cfg)
    cfg_o = RenderConfig(**{**cfg.__dict__, "seed": 12345})
    os_, oq, _, wd = oracle.render(dome_scene, cfg_o)
    assert st == 0 and wd == 0
    xg, vg = xyz_from_sums(gs_, gq, cfg.spp, dome_scene.band_xyz)
    xo, vo = xyz_from_sums(os_, oq, cfg.spp, dome_scene.band_xyz)
    r = parity_report(xg, vg, xo, vo)
    print("dome parity", r)
    assert r["frac_beyond_3se"] <= 0.01
    assert abs(r["mean_z"]) < 0.1
    for b, se in zip(r["bias_xyz"], r["bias_se_xyz"]):
        assert abs(b) < 0.005 + 3 * se


def test_high_spp_mean_relative_error(gpu, dome_scene):
    """The CPU-runnable scene and settings (32 bands, sun 10 deg, at most 16
    orders) on an 8x4 view at matched high sample counts (GPU 2^20, oracle
    2^16 per pixel and band): per-pixel mean relative XYZ error under 0.5 %,
    and the image-summed bias under 0.5 %."""
    cfg = RenderConfig(width=8, height=4, spp=1 << 20, phase_sampling=_abi.PHASE_TABULATED,
                       tracking=_abi.TRACKING_MERGED_LAYERS, max_orders=16)
    cfg_o = RenderConfig(**{**cfg.__dict__, "spp": 1 << 16, "seed": 4242})
    with GpuScene(dome_scene) as gs:
        gs_, gq, _, _ = gpu_sums(gs, cfg)
    os_, oq, _, _ = oracle.render(dome_scene, cfg_o)
    xg, vg = xyz_from_sums(gs_, gq, cfg.spp, dome_scene.band_xyz)
    xo, vo = xyz_from_sums(os_, oq, cfg_o.spp, dome_scene.band_xyz)
    r = parity_report(xg, vg, xo, vo)
    print("high-spp parity", r)
    assert r["frac_beyond_3se"] <= 0.05
    assert r["noise_rel_err_per_pixel"] < 0.003
    assert r["mean_rel_err_per_pixel"] < 0.005
    assert max(abs(b) for b in r["bias_xyz"]) < 0.005


def test_vacuum_ground_known_answer(gpu, data_dir):
    a = SyntheticAtmosphere(rayleigh_ext_km=0.0, mie_ext_km=0.0, ozone_peak_km=0.0)
    scene = synthetic_scene(wavelengths(450, 650, 3), data_dir, sun_elevation_deg=30.0, atmosphere=a)
    cfg = RenderConfig(width=1, height=8, spp=2048, output_projection=_abi.PROJECTION_SKY_VIEW_LUT)
    with GpuScene(scene) as gs:
        s, q, _, st = gpu_sums(gs, cfg)
    mean = s / cfg.spp
    se = np.sqrt(np.maximum(q / cfg.spp - mean * mean, 0) / cfg.spp)
    for y in range(8):
        d = analytic.lut_direction(1, 8, 0, y, 0.2, scene.ground_radius_km, scene.sun_direction)
        for band in range(3):
            if y >= 6:
                want = analytic.vacuum_ground(scene, band, d)
                assert abs(mean[y, band] - want) <= 4 * se[y, band] + 1e-4 * want
            else:
                assert mean[y, band] == 0.0


@pytest.mark.parametrize("tracking", [_abi.TRACKING_SEGMENT_RESTART, _abi.TRACKING_RESIDUAL_CARRY,
                                      _abi.TRACKING_MERGED_LAYERS])
def test_single_scatter_known_answer(gpu, data_dir, tracking):
    a = SyntheticAtmosphere(ground_albedo=0.0)
    scene = synthetic_scene(wavelengths(440, 640, 3), data_dir, sun_elevation_deg=35.0, atmosphere=a)
    cfg = RenderConfig(width=1, height=8, spp=262144, max_orders=1, output_projection=_abi.PROJECTION_SKY_VIEW_LUT,
                       tracking=tracking)
    with GpuScene(scene) as gs:
        s, q, _, st = gpu_sums(gs, cfg)
    assert st == 0
    for y in (0, 3, 5):
        d = analytic.lut_direction(1, 8, 0, y, 0.2, scene.ground_radius_km, scene.sun_direction)
        for band in range(3):
            want = analytic.single_scatter(scene, band, d,
                                           lambda sp, b, mu: oracle.mie_phase(scene, sp, b, [mu])[0])
            mean = s[y, band] / cfg.spp
            se = math.sqrt(max(q[y, band] / cfg.spp - mean * mean, 0) / cfg.spp)
            assert abs(mean - want) <= 4 * se + 0.002 * want, (y, band, mean, want, se)


@pytest.mark.parametrize("kernel", KERNELS)
def test_film_matches_sums_and_progressive_is_exact(gpu, dome_scene, kernel):
    """Film = clamped mean of the sums; two progressive halves add up to one
    render (bit for bit on the plain kernel, whose sums have a fixed order;
    to FP64 rounding on the persistent kernel, whose cells add in the order
    chains finish)."""
    cfg = RenderConfig(width=16, height=8, spp=64, phase_sampling=_abi.PHASE_TABULATED,
                       tracking=_abi.TRACKING_MERGED_LAYERS, kernel=kernel)
    with GpuScene(dome_scene) as gs:
        film, stats = gs.render(cfg, count_events=True)
        _, uncounted = gs.render(cfg)  # events only on request (SKY_FLAG_COUNT_EVENTS)
        assert all(v == 0 for v in uncounted.events.values()) and uncounted.chains == stats.chains
        s, q, _, _ = gpu_sums(gs, cfg)
        np.testing.assert_array_equal(film.values, np.maximum((s / 64).astype(np.float32), 0).ravel())
        # two progressive halves == one render, bit for bit
        import torch
        cells = cfg.pixels * gs.band_count
        ps = torch.zeros(cells, dtype=torch.float64, device="cuda")
        pq = torch.zeros(cells, dtype=torch.float64, device="cuda")
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        for off in (0, 32):
            c = RenderConfig(**{**cfg.__dict__, "spp": 32, "sample_offset": off,
                                "flags": FLAG_ACCUMULATE if off else 0})
            gs.render_device(c, {"cell_sum": ps.data_ptr(), "cell_sumsq": pq.data_ptr(), "status": st.data_ptr()},
                             torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        if kernel == _abi.KERNEL_PLAIN:
            np.testing.assert_array_equal(ps.cpu().numpy().reshape(s.shape), s)
            np.testing.assert_array_equal(pq.cpu().numpy().reshape(q.shape), q)
        else:
            np.testing.assert_allclose(ps.cpu().numpy().reshape(s.shape), s, rtol=1e-12)
            np.testing.assert_allclose(pq.cpu().numpy().reshape(q.shape), q, rtol=1e-12)
    assert stats.chains == cells * 64 and stats.kernel_ms > 0
    assert stats.events["chain"] == stats.chains


def test_xyz_outputs(gpu, dome_scene):
    cfg = RenderConfig(width=16, height=8, spp=64)
    with GpuScene(dome_scene) as gs:
        film, xyz, var, _ = gs.render_xyz(cfg)
        s, q, _, _ = gpu_sums(gs, cfg)
    x_ref, v_ref = xyz_from_sums(s, q, 64, dome_scene.band_xyz)
    np.testing.assert_allclose(xyz, x_ref, rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(var, v_ref, rtol=1e-9, atol=1e-20)


def test_watchdog_and_errors(gpu, dome_scene):
    with GpuScene(dome_scene) as gs:
        # a forced one-event watchdog trips on any scattered path (integrator.rs:301-304)
        with pytest.raises(RenderWatchdog):
            gs.render(RenderConfig(width=8, height=4, spp=4, watchdog_limit=1))
        with pytest.raises(SkyCudaError) as e:
            gs.render(RenderConfig(width=0, height=4, spp=4))
        assert e.value.status == _abi.SKY_ERR_INVALID_CONFIG
        # sample counts that the kernels' 32-bit sample counters could not step through
        with pytest.raises(SkyCudaError, match="spp must be below"):
            gs.render(RenderConfig(width=1, height=1, spp=0x80000000))
        # NEE sample counts that would keep a launch running for hours
        with pytest.raises(SkyCudaError, match="direct_light_samples"):
            gs.render(RenderConfig(width=1, height=1, spp=1, direct_light_samples=1025))
        # the scene stays usable after the failures
        film, _ = gs.render(RenderConfig(width=8, height=4, spp=4))
        assert np.all(np.isfinite(film.values))


def test_reference_default_band_count(gpu, ref_scene):
    """The drop-in scene: 41 bands, 1024-bin phase tables, isotropic sampling,
    the reference's defaults throughout."""
    cfg = RenderConfig(width=16, height=8, spp=32)
    with GpuScene(ref_scene) as gs:
        s, q, _, st = gpu_sums(gs, cfg)
    o, oq, _, _ = oracle.render(ref_scene, RenderConfig(**{**cfg.__dict__, "seed": 99}))
    xg, vg = xyz_from_sums(s, q, 32, ref_scene.band_xyz)
    xo, vo = xyz_from_sums(o, oq, 32, ref_scene.band_xyz)
    r = parity_report(xg, vg, xo, vo)
    print("reference scene parity", r)
    assert st == 0 and r["frac_beyond_3se"] <= 0.03


@pytest.mark.parametrize("variant,cost", [(0, 0.25), (1, 0.5), (2, 0.1), (2, 1.0)])
def test_wavefront_shapes_trace_the_same_chains(gpu, dome_scene, variant, cost):
    """Every launch shape the autotuner can pick traces the plain kernel's
    paths (the crossing cost changes the tracking grid for both kernels)."""
    with GpuScene(dome_scene) as gs:
        gs.set_tuning(variant=variant, crossing_cost=cost)
        t = gs.get_tuning()
        assert t["variant"] == variant and abs(t["crossing_cost"] - cost) < 1e-6
        cfg = RenderConfig(width=32, height=16, spp=2, sample_offset=5, phase_sampling=_abi.PHASE_TABULATED,
                           tracking=_abi.TRACKING_MERGED_LAYERS, max_orders=16)
        a, _, _, _ = gpu_sums(gs, RenderConfig(**{**cfg.__dict__, "kernel": _abi.KERNEL_PLAIN}))
        b, _, _, _ = gpu_sums(gs, RenderConfig(**{**cfg.__dict__, "kernel": _abi.KERNEL_WAVEFRONT}))
    close = np.abs(a - b) <= 1e-5 * np.maximum(np.abs(a), np.abs(b)) + 1e-12
    assert close.mean() >= 0.999


def test_autotuner_picks_a_measured_shape(gpu, dome_scene):
    from sky_cuda.autotune import autotune
    cfg = RenderConfig(width=64, height=32, spp=64, phase_sampling=_abi.PHASE_TABULATED,
                       tracking=_abi.TRACKING_MERGED_LAYERS)
    with GpuScene(dome_scene) as gs:
        best, results = autotune(gs, cfg, space={"variant": (0, 2), "crossing_cost": (0.25, 0.5)})
        assert len(results) == 4 and all(ms > 0 for _, ms in results)
        assert best == min(results, key=lambda r: r[1])[0]
        assert gs.get_tuning() == best
        film, _ = gs.render(cfg)
        assert np.all(np.isfinite(film.values))


@pytest.mark.parametrize("tracking", [_abi.TRACKING_SEGMENT_RESTART, _abi.TRACKING_MERGED_LAYERS])
def test_event_counting_does_not_change_the_render(gpu, dome_scene, tracking):
    """The wavefront kernel is instantiated with and without event counting
    (counting only when SkyDeviceOutputs.counters is given): both trace the
    same chains, so the cell sums agree to FP64 rounding, and the counted run
    reports one chain event per chain."""
    import torch
    cfg = RenderConfig(width=32, height=16, spp=64, phase_sampling=_abi.PHASE_TABULATED, tracking=tracking)
    with GpuScene(dome_scene) as gs:
        cells = cfg.pixels * gs.band_count
        runs = []
        for count in (False, True):
            s = torch.zeros(cells, dtype=torch.float64, device="cuda")
            q = torch.zeros(cells, dtype=torch.float64, device="cuda")
            st = torch.zeros(1, dtype=torch.int32, device="cuda")
            ctr = torch.zeros(8, dtype=torch.int64, device="cuda")
            outs = {"cell_sum": s.data_ptr(), "cell_sumsq": q.data_ptr(), "status": st.data_ptr()}
            if count:
                outs["counters"] = ctr.data_ptr()
            gs.render_device(cfg, outs, torch.cuda.current_stream().cuda_stream)
            torch.cuda.synchronize()
            assert int(st.item()) == 0
            runs.append((s.cpu().numpy(), q.cpu().numpy(), ctr.cpu().numpy()))
    np.testing.assert_allclose(runs[0][0], runs[1][0], rtol=1e-12, atol=0)
    np.testing.assert_allclose(runs[0][1], runs[1][1], rtol=1e-12, atol=0)
    assert runs[0][2].sum() == 0
    assert runs[1][2][6] == cells * cfg.spp and runs[1][2][0] > 0


@pytest.mark.parametrize("kernel", KERNELS)
@pytest.mark.parametrize("phase", [_abi.PHASE_ISOTROPIC, _abi.PHASE_TABULATED])
def test_single_species_kernels_match_four_species(gpu, dome_scene, kernel, phase):
    """The synthetic scene carries aerosol in species 0 only, so the kernels
    evaluate that species alone; SkyTuning.all_species = 1 forces the
    four-species instantiations.  Both trace the same chains: the plain
    kernel's sums are equal bit for bit, the wavefront kernel's to FP64
    rounding (its lanes add to a cell in no fixed order), and the event
    counts are equal."""
    cfg = RenderConfig(width=32, height=16, spp=16, phase_sampling=phase, tracking=_abi.TRACKING_MERGED_LAYERS,
                       rr_start_depth=8, kernel=kernel)
    with GpuScene(dome_scene) as gs:
        assert gs.get_tuning()["all_species"] == 0
        a, qa, ca, sa = gpu_sums(gs, cfg)
        gs.set_tuning(all_species=1)
        assert gs.get_tuning()["all_species"] == 1
        b, qb, cb, sb = gpu_sums(gs, cfg)
        with pytest.raises(SkyCudaError):
            gs.set_tuning(all_species=2)
    assert sa == 0 and sb == 0 and ca[6] == cfg.pixels * dome_scene.band_count * cfg.spp
    if kernel == _abi.KERNEL_PLAIN:
        np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(qa, qb)
    else:
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=0)
        np.testing.assert_allclose(qa, qb, rtol=1e-12, atol=0)
    np.testing.assert_array_equal(ca, cb)


@pytest.mark.parametrize("kernel", KERNELS)
def test_four_species_chains_match_oracle(gpu, ref_scene, kernel):
    """The reference tables carry four aerosol species, so the four-species
    instantiations run: chain by chain against the oracle."""
    agree = total = 0
    with GpuScene(ref_scene) as gs:
        for offset in (0, 11):
            cfg = RenderConfig(width=16, height=8, spp=1, sample_offset=offset, seed=0x5EC7_2026_0430 + offset,
                               phase_sampling=_abi.PHASE_TABULATED, tracking=_abi.TRACKING_MERGED_LAYERS,
                               max_orders=16, kernel=kernel)
            g, _, _, st = gpu_sums(gs, cfg)
            o, _, _, wd = oracle.render(ref_scene, cfg)
            assert st == 0 and wd == 0
            close = np.abs(g - o) <= 2e-3 * np.maximum(np.abs(g), np.abs(o)) + 1e-9
            agree += int(close.sum())
            total += close.size
    frac = agree / total
    print(f"four aerosol species, chain agreement kernel={kernel}: {frac:.4f} of {total}")
    assert frac >= 0.95


def _device_buffers(cells: int, pixels: int):
    import torch
    return {"s": torch.zeros(cells, dtype=torch.float64, device="cuda"),
            "q": torch.zeros(cells, dtype=torch.float64, device="cuda"),
            "film": torch.zeros(cells, dtype=torch.float32, device="cuda"),
            "xyz": torch.zeros(pixels * 3, dtype=torch.float64, device="cuda"),
            "st": torch.zeros(1, dtype=torch.int32, device="cuda")}


def _outs(b, first=True):
    o = {"cell_sum": b["s"].data_ptr(), "cell_sumsq": b["q"].data_ptr(), "film": b["film"].data_ptr(),
         "xyz": b["xyz"].data_ptr()}
    if first:
        o["status"] = b["st"].data_ptr()
    return o


def test_one_pixel_odd_spp_matches_plain(gpu, dome_scene):
    """A 1x1 image at 5 samples: one cell whose samples do not fill a warp."""
    cfg = RenderConfig(width=1, height=1, spp=5, sample_offset=3, phase_sampling=_abi.PHASE_TABULATED,
                       tracking=_abi.TRACKING_MERGED_LAYERS)
    with GpuScene(dome_scene) as gs:
        a, qa, _, sa = gpu_sums(gs, RenderConfig(**{**cfg.__dict__, "kernel": _abi.KERNEL_PLAIN}))
        b, qb, _, sb = gpu_sums(gs, RenderConfig(**{**cfg.__dict__, "kernel": _abi.KERNEL_WAVEFRONT}))
    assert sa == 0 and sb == 0
    np.testing.assert_allclose(b, a, rtol=1e-12, atol=0)
    np.testing.assert_allclose(qb, qa, rtol=1e-12, atol=0)


def test_batch_of_unequal_jobs_matches_separate_renders(gpu, dome_scene):
    """Jobs of different image sizes, projections and spp in one launch (the
    cell-to-job lookup and the per-job finalize), one of them accumulating
    onto sums it already holds, against the same renders made one by one."""
    import torch
    stream = torch.cuda.current_stream().cuda_stream
    cfgs = [RenderConfig(width=24, height=12, spp=16, phase_sampling=_abi.PHASE_TABULATED,
                         tracking=_abi.TRACKING_MERGED_LAYERS, seed=11),
            RenderConfig(width=7, height=3, spp=40, phase_sampling=_abi.PHASE_TABULATED,
                         tracking=_abi.TRACKING_MERGED_LAYERS, output_projection=_abi.PROJECTION_SKY_VIEW_LUT,
                         seed=12),
            RenderConfig(width=16, height=16, spp=8, sample_offset=8, flags=FLAG_ACCUMULATE,
                         phase_sampling=_abi.PHASE_TABULATED, tracking=_abi.TRACKING_MERGED_LAYERS, seed=13)]
    with GpuScene(dome_scene) as gs:
        B = gs.band_count
        bufs = [_device_buffers(c.pixels * B, c.pixels) for c in cfgs]
        # the accumulating job continues a render of samples 0..7 already in its buffers
        first = RenderConfig(**{**cfgs[2].__dict__, "spp": 8, "sample_offset": 0, "flags": 0})
        gs.render_device(first, _outs(bufs[2]), stream)
        gs.render_batch([(c, None, _outs(b, i == 0)) for i, (c, b) in enumerate(zip(cfgs, bufs))], stream)
        torch.cuda.synchronize()
        assert int(bufs[0]["st"].item()) == 0
        want = []
        for c in cfgs:
            b = _device_buffers(c.pixels * B, c.pixels)
            if c.flags:
                gs.render_device(first, _outs(b), stream)
            gs.render_device(c, _outs(b), stream)
            want.append(b)
        torch.cuda.synchronize()
    for got, ref in zip(bufs, want):
        np.testing.assert_allclose(got["s"].cpu().numpy(), ref["s"].cpu().numpy(), rtol=1e-12, atol=0)
        np.testing.assert_allclose(got["film"].cpu().numpy(), ref["film"].cpu().numpy(), rtol=1e-6, atol=0)
        np.testing.assert_allclose(got["xyz"].cpu().numpy(), ref["xyz"].cpu().numpy(), rtol=1e-12, atol=1e-300)
