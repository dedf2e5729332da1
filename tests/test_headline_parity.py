"""Oracle parity on the production workload, the one the benchmark times.

Scene and settings are those of `plain-512x256-81wl-256spp`: a 512x256
equirect panorama, 81 wavelengths at 5 nm from 380 to 780 nm, 256 samples,
Russian roulette after order 8, no order cap, sun at 5 degrees, 64 majorant
layers over 0-100 km, tabulated phase sampling, the GPU tracking over the
merged-layer grid.

1. Every 32nd pixel row at 256 spp: the GPU's per-pixel XYZ against the
   oracle running the reference's own segment-restart tracking
   (sky_trace.wgsl:405-475) with an independent seed lies within 3 combined
   standard errors on at least 99 % of the pixels.
2. Matched high sample counts (the GPU at 2^20, the oracle at 2^16 samples
   per pixel and band) on an 8x4 view of the same scene and settings: the
   per-pixel mean relative XYZ error is under 0.5 %.
"""

import numpy as np
import pytest

import sky_oracle as oracle
from sky_cuda import GpuScene, RenderConfig, synthetic_scene, wavelengths
from sky_cuda import _abi
from skystats import parity_report, xyz_from_sums

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def production_scene(data_dir):
    return synthetic_scene(wavelengths(380.0, 780.0, 81), data_dir, sun_elevation_deg=5.0)


def _config(**kw):
    base = dict(width=512, height=256, spp=256, seed=0x5EC7_2026_0430, sun_elevation_deg=5.0,
                phase_sampling=_abi.PHASE_TABULATED, rr_start_depth=8, max_orders=0,
                tracking=_abi.TRACKING_MERGED_LAYERS)
    base.update(kw)
    return RenderConfig(**base)


def _gpu_sums(gs, cfg):
    import torch
    cells = cfg.pixels * gs.band_count
    s = torch.zeros(cells, dtype=torch.float64, device="cuda")
    q = torch.zeros(cells, dtype=torch.float64, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    gs.render_device(cfg, {"cell_sum": s.data_ptr(), "cell_sumsq": q.data_ptr(), "status": st.data_ptr()},
                     torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    B = gs.band_count
    return s.cpu().numpy().reshape(-1, B), q.cpu().numpy().reshape(-1, B)


def test_production_rows_within_three_standard_errors(gpu, production_scene):
    cfg = _config()
    with GpuScene(production_scene) as gs:
        gs_, gq = _gpu_sums(gs, cfg)
    row_begin, row_step = 16, 32
    cfg_o = _config(seed=0x9E3779B97F4A7C15, tracking=_abi.TRACKING_SEGMENT_RESTART)
    os_, oq, _, wd = oracle.render(production_scene, cfg_o, row_begin=row_begin, row_step=row_step)
    assert wd == 0
    rows = np.arange(row_begin, cfg.height, row_step)
    pix = (rows[:, None] * cfg.width + np.arange(cfg.width)[None, :]).reshape(-1)
    w = production_scene.band_xyz
    xg, vg = xyz_from_sums(gs_[pix], gq[pix], cfg.spp, w)
    xo, vo = xyz_from_sums(os_[pix], oq[pix], cfg.spp, w)
    r = parity_report(xg, vg, xo, vo)
    print("production rows parity", r)
    assert r["pixels"] >= 0.9 * pix.size
    assert r["frac_beyond_3se"] <= 0.01
    assert abs(r["mean_z"]) < 0.1
    for b, se in zip(r["bias_xyz"], r["bias_se_xyz"]):
        assert abs(b) < 0.005 + 3 * se


def test_production_settings_mean_relative_error_at_high_spp(gpu, production_scene):
    view = dict(width=8, height=4)
    cfg_g = _config(spp=1 << 20, **view)
    cfg_o = _config(spp=1 << 16, seed=0x51ED2701, **view)
    with GpuScene(production_scene) as gs:
        gs_, gq = _gpu_sums(gs, cfg_g)
    os_, oq, _, wd = oracle.render(production_scene, cfg_o)
    assert wd == 0
    w = production_scene.band_xyz
    xg, vg = xyz_from_sums(gs_, gq, cfg_g.spp, w)
    xo, vo = xyz_from_sums(os_, oq, cfg_o.spp, w)
    r = parity_report(xg, vg, xo, vo)
    print("production settings, high spp", r)
    assert r["regular_pixels"] >= 24  # all but the sun-disc pixel and the darkest
    # the noise of the two estimates alone keeps the error well below the bar
    assert r["noise_rel_err_per_pixel"] < 0.003
    assert r["mean_rel_err_per_pixel"] < 0.005
    assert r["frac_beyond_3se"] <= 0.05


@pytest.mark.parametrize("tracking", [_abi.TRACKING_SEGMENT_RESTART, _abi.TRACKING_MERGED_LAYERS])
@pytest.mark.parametrize("elevation", [-2.0, 0.5, 3.0])
def test_twilight_sky_view_lut_parity(gpu, ref_scene, elevation, tracking):
    """The reference's own scene (data/ tables, 41 bands) as its elevation bake
    renders it (sky-view LUT, scripts/bake_skyview_elevations.ps1), at the low
    sun elevations where shadow rays descend to a tangent point: a 16x8 LUT at
    2^17 (GPU) and 2^13-2^14 (oracle) samples, tabulated phase sampling,
    independent seeds, the same tracking on both sides.

    With the reference's segment rule (segment restart) both sides skip
    optical depth on shallow descending rays as the reference does
    (tests/test_oracle.py::test_transmittance_on_descending_rays): at -2
    degrees that makes the sky 6-11 % brighter than exact tracking, and the
    GPU reproduces it.  With merged-layer tracking neither side skips any."""
    scene = ref_scene.with_sun(elevation)
    base = dict(width=16, height=8, sun_elevation_deg=elevation, output_projection=_abi.PROJECTION_SKY_VIEW_LUT,
                phase_sampling=_abi.PHASE_TABULATED, tracking=tracking)
    cfg_g = RenderConfig(spp=1 << 17, seed=0x5EC7_2026_0430, **base)
    oracle_spp = 1 << 14 if tracking == _abi.TRACKING_MERGED_LAYERS else 1 << 13
    cfg_o = RenderConfig(spp=oracle_spp, seed=0x2BAD5EED, **base)
    with GpuScene(scene) as gs:
        gs_, gq = _gpu_sums(gs, cfg_g)
    os_, oq, _, wd = oracle.render(scene, cfg_o)
    assert wd == 0
    w = scene.band_xyz
    xg, vg = xyz_from_sums(gs_, gq, cfg_g.spp, w)
    xo, vo = xyz_from_sums(os_, oq, cfg_o.spp, w)
    r = parity_report(xg, vg, xo, vo)
    print(f"twilight {elevation} deg", r)
    assert r["pixels"] >= 64
    assert r["frac_beyond_3se"] <= 0.03
    assert abs(r["mean_z"]) < 0.35
    for b, se in zip(r["bias_xyz"], r["bias_se_xyz"]):
        assert abs(b) < 0.005 + 3 * se
