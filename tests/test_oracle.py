"""CPU suite: the oracle pinned against the reference's own known answers and
against analytic answers.  No GPU needed."""

import math

import numpy as np
import pytest

import analytic
import sky_oracle as oracle
from sky_cuda import RenderConfig, SyntheticAtmosphere, synthetic_scene, wavelengths
from sky_cuda import _abi
from sky_cuda.scene import (PHASE_BINS, cie_1931_2deg, hg_phase_values, load_cie_1931, rayleigh_cross_section_m2)
from skystats import parity_report, xyz_from_sums

M32 = 0xFFFFFFFF


def pcg4d_py(v):
    """Independent restatement of pcg4d (sky_trace.wgsl:156-168)."""
    x, y, z, w = [(a * 1664525 + 1013904223) & M32 for a in v]
    x = (x + y * w) & M32
    y = (y + z * x) & M32
    z = (z + x * y) & M32
    w = (w + y * z) & M32
    x ^= x >> 16
    y ^= y >> 16
    z ^= z >> 16
    w ^= w >> 16
    x = (x + y * w) & M32
    y = (y + z * x) & M32
    z = (z + x * y) & M32
    w = (w + y * z) & M32
    return x, y, z, w


# ---- RNG ---------------------------------------------------------------------------


@pytest.mark.parametrize("v", [(0, 0, 0, 0), (1, 2, 3, 4), (0xFFFFFFFF, 0x12345678, 40, 9),
                               (0x20260430 ^ 77, 0x5EC7 ^ 3, 12, 1000)])
def test_pcg4d_bit_exact(v):
    assert oracle.pcg4d(v) == pcg4d_py(v)


def test_rng_stream_matches_counter_definition():
    seed = 0x5EC7_2026_0430
    pixel, sample, band = 1234, 17, 5
    u, f = oracle.rng_stream(pixel, sample, band, seed, 64)
    for dim in range(64):
        h = pcg4d_py(((pixel ^ (seed & M32)) & M32, (sample ^ (seed >> 32)) & M32, band, dim))
        want = h[0] ^ h[1] ^ h[2] ^ h[3]
        assert int(u[dim]) == want
        assert f[dim] == np.float32((want >> 8) * 2.0 ** -24)
    assert np.all((f >= 0) & (f < 1))


# ---- reference known answers ----------------------------------------------------------


def test_geometry_known_answers():
    # geometry.rs:101-117: 0.2 km observer, up exits at 119.8 km, down hits ground at 0.2 km
    hit, t, kind = oracle.next_boundary(6360.0, 6480.0, [0, 6360.2, 0], [0, 1, 0])
    assert hit and kind == 1 and abs(t - 119.8) < 0.01
    hit, t, kind = oracle.next_boundary(6360.0, 6480.0, [0, 6360.2, 0], [0, -1, 0])
    assert hit and kind == 0 and abs(t - 0.2) < 0.01


def test_uniform_table_samples_isotropic_pdf(ref_scene):
    # phase.rs:163-169 with a uniform table
    s = ref_scene.with_sun(0.0)
    s.phase_values = np.ones_like(s.phase_values)
    mu, pdf = oracle.sample_mu_pdf(s, 0, 0, [0.5])
    assert -1.0 <= mu[0] <= 1.0
    assert abs(pdf[0] - 1.0 / (4.0 * math.pi)) < 1e-3
    assert abs(oracle.sampling_pdf(s, 0, 0, mu)[0] - pdf[0]) < 1e-6


def test_rayleigh_inverse_cdf_endpoints():
    # sampling.rs:269-274
    assert abs(oracle.invert_rayleigh_cdf(0.0) + 1.0) < 1e-6
    assert abs(oracle.invert_rayleigh_cdf(0.5)) < 1e-6
    assert abs(oracle.invert_rayleigh_cdf(1.0) - 1.0) < 1e-6


def test_cie_table_range(data_dir):
    # spectrum.rs:375-382
    t = load_cie_1931(data_dir / "CIE_xyz_1931_2deg.csv")
    assert t[0, 0] == 360.0 and t[-1, 0] == 830.0
    assert abs(cie_1931_2deg(t, 555.0)[0, 1] - 1.0) < 0.01


def test_repository_data_loads(ref_scene):
    # data.rs:204-220
    assert ref_scene.band_count == 41
    assert ref_scene.majorants.shape == (41, 64)
    assert np.all(np.isfinite(ref_scene.majorants)) and np.all(ref_scene.majorants.max(axis=1) > 0)


def test_majorants_dominate_extinction(ref_scene):
    # data.rs:253-276: 241 altitudes x 41 bands, CPU extinction vs the baked grid
    top = ref_scene.top_altitude_km
    L = ref_scene.layer_count
    for band in range(ref_scene.band_count):
        for i in range(241):
            alt = np.float32(top) * np.float32(i) / np.float32(240)
            ext = oracle.cpu_extinction(ref_scene, float(alt), band)
            layer = min(int(math.floor(min(max(alt, 0), top - 1.1920929e-7) / top * L)), L - 1)
            assert ext <= ref_scene.majorants[band, layer] * 1.001
            assert ref_scene.minorants[band, layer] <= ext * 1.001 + 1e-8


def test_python_bake_matches_oracle_bake(ref_scene, dome_scene):
    for scene in (ref_scene, dome_scene):
        maj, mino = oracle.bake_majorant_grid(scene, scene.layer_count)
        np.testing.assert_array_equal(maj, scene.majorants)
        np.testing.assert_array_equal(mino, scene.minorants)


def test_synthesized_phase_is_normalized():
    # data.rs:222-251 integration rule applied to the HG tables that stand in
    # for the missing mie_phase.csv
    for bins in (PHASE_BINS, 256):
        p = hg_phase_values(0.76, bins).astype(np.float64)
        u = (np.arange(bins) + 0.5) / bins
        mu = 1 - 2 * u ** 3
        integral = np.sum(0.5 * (p[1:] + p[:-1]) * np.abs(mu[:-1] - mu[1:]) * 2 * math.pi)
        assert abs(integral - 1.0) < 0.01  # the bin-centre rule truncates the two end half-bins


def test_coefficients_non_negative(ref_scene):
    # medium.rs:171-214
    for alt in (0.0, 0.5, 3.0, 11.0, 30.0, 119.0):
        for band in (0, 20, 40):
            c = oracle.coefficients(ref_scene, alt, band)
            assert np.all(c >= 0)
            assert c[11] >= c[10] > 0


def test_packed_layouts(ref_scene):
    # integrator.rs:479-510: band-major optics, band-major majorants, phase size
    d = ref_scene.desc()
    assert d.band_count == 41
    assert ref_scene.aerosol_optics.size == 41 * 4
    assert ref_scene.majorants.size == 41 * ref_scene.layer_count
    assert ref_scene.phase_values.size == 4 * 41 * PHASE_BINS
    assert ref_scene.aerosol_optics["absorption_km_inv_per_g_m3"][3] == \
        ref_scene.aerosol_optics.reshape(41, 4)["absorption_km_inv_per_g_m3"][0, 3]
    flat = ref_scene.majorants.ravel()
    assert flat[ref_scene.layer_count] == ref_scene.majorants[1, 0]


def test_rayleigh_cross_section():
    # medium.rs:104-106
    assert rayleigh_cross_section_m2(550.0) == np.float32(5.8e-31)
    assert abs(float(rayleigh_cross_section_m2(440.0)) / 5.8e-31 - (550 / 440) ** 4) < 1e-5


# ---- oracle images ----------------------------------------------------------------------


def test_oracle_smoke_film(ref_scene):
    # smoke.rs:7-24: 32x16 at 2 spp with the default config
    cfg = RenderConfig(width=32, height=16, spp=2)
    s, sq, counters, wd = oracle.render(ref_scene, cfg)
    film = np.maximum((s / cfg.spp).astype(np.float32), 0)
    assert wd == 0
    assert np.all(np.isfinite(film)) and np.all(film >= 0) and np.any(film > 0)
    assert counters[6] == 32 * 16 * 41 * 2


def _vacuum_scene(data_dir, sun_elevation=30.0):
    a = SyntheticAtmosphere(rayleigh_ext_km=0.0, mie_ext_km=0.0, ozone_peak_km=0.0)
    return synthetic_scene(wavelengths(450, 650, 3), data_dir, sun_elevation_deg=sun_elevation, atmosphere=a)


def test_oracle_vacuum_ground_and_sky(data_dir):
    scene = _vacuum_scene(data_dir)
    cfg = RenderConfig(width=1, height=8, spp=2048, output_projection=_abi.PROJECTION_SKY_VIEW_LUT)
    s, sq, _, wd = oracle.render(scene, cfg)
    mean = s / cfg.spp
    se = np.sqrt(np.maximum(sq / cfg.spp - mean * mean, 0) / cfg.spp)
    assert wd == 0
    for y in range(8):
        d = analytic.lut_direction(1, 8, 0, y, 0.2, scene.ground_radius_km, scene.sun_direction)
        for band in range(scene.band_count):
            if y >= 6:  # ground rows: only the sun-cone sampling is random
                want = analytic.vacuum_ground(scene, band, d)
                assert abs(mean[y, band] - want) <= 4 * se[y, band] + 2e-5 * want
            else:
                assert mean[y, band] == 0.0


@pytest.mark.parametrize("tracking", [_abi.TRACKING_SEGMENT_RESTART, _abi.TRACKING_RESIDUAL_CARRY,
                                      _abi.TRACKING_MERGED_LAYERS])
def test_oracle_single_scatter_integral(data_dir, tracking):
    a = SyntheticAtmosphere(ground_albedo=0.0)
    scene = synthetic_scene(wavelengths(440, 640, 3), data_dir, sun_elevation_deg=35.0, atmosphere=a)
    cfg = RenderConfig(width=1, height=8, spp=40000, max_orders=1, output_projection=_abi.PROJECTION_SKY_VIEW_LUT,
                       tracking=tracking)
    s, sq, _, wd = oracle.render(scene, cfg)
    assert wd == 0
    for y in (0, 3, 5):
        d = analytic.lut_direction(1, 8, 0, y, 0.2, scene.ground_radius_km, scene.sun_direction)
        for band in range(3):
            want = analytic.single_scatter(scene, band, d,
                                           lambda sp, b, mu: oracle.mie_phase(scene, sp, b, [mu])[0])
            mean = s[y, band] / cfg.spp
            se = math.sqrt(max(sq[y, band] / cfg.spp - mean * mean, 0) / cfg.spp)
            assert abs(mean - want) <= 4 * se + 0.003 * want, (y, band, mean, want, se)


def _small_parity(scene, cfg_a, cfg_b):
    sa, qa, _, _ = oracle.render(scene, cfg_a)
    sb, qb, _, _ = oracle.render(scene, cfg_b)
    xa, va = xyz_from_sums(sa, qa, cfg_a.spp, scene.band_xyz)
    xb, vb = xyz_from_sums(sb, qb, cfg_b.spp, scene.band_xyz)
    return parity_report(xa, va, xb, vb)


@pytest.mark.parametrize("other", [_abi.TRACKING_RESIDUAL_CARRY, _abi.TRACKING_MERGED_LAYERS])
def test_oracle_tracking_modes_agree(data_dir, other):
    scene = synthetic_scene(wavelengths(400, 700, 4), data_dir, sun_elevation_deg=10.0)
    base = dict(width=8, height=6, spp=256, phase_sampling=_abi.PHASE_TABULATED, max_orders=16)
    r = _small_parity(scene, RenderConfig(**base, tracking=_abi.TRACKING_SEGMENT_RESTART),
                      RenderConfig(**base, tracking=other, seed=99))
    assert r["frac_beyond_3se"] <= 0.05 and abs(r["mean_z"]) < 1.0, r


def test_oracle_light_sample_counts_agree(data_dir):
    """direct_light_samples averages that many sun samples per vertex: the
    expectation does not depend on the count."""
    scene = synthetic_scene(wavelengths(400, 700, 4), data_dir, sun_elevation_deg=10.0)
    base = dict(width=8, height=6, spp=256, phase_sampling=_abi.PHASE_TABULATED, max_orders=16,
                tracking=_abi.TRACKING_MERGED_LAYERS)
    r = _small_parity(scene, RenderConfig(**base), RenderConfig(**base, direct_light_samples=3, seed=5))
    assert r["frac_beyond_3se"] <= 0.05 and abs(r["mean_z"]) < 1.0, r


def test_oracle_phase_sampling_modes_agree(data_dir):
    scene = synthetic_scene(wavelengths(400, 700, 4), data_dir, sun_elevation_deg=10.0)
    base = dict(width=8, height=6, spp=256, max_orders=16)
    r = _small_parity(scene, RenderConfig(**base, phase_sampling=0),
                      RenderConfig(**base, phase_sampling=1, seed=7))
    assert r["frac_beyond_3se"] <= 0.05 and abs(r["mean_z"]) < 1.0, r


def _group_cost(maj, starts, dz, crossing_cost=0.1):
    m = np.maximum(np.asarray(maj, dtype=np.float64), 1e-8)
    bounds = list(starts) + [len(m)]
    return sum(crossing_cost + dz * (m[a:b].max() * (b - a) - m[a:b].sum()) for a, b in zip(bounds[:-1], bounds[1:]))


def test_merge_groups_is_optimal():
    """Tracking mode 2's layer grouping is the partition of least cost (a crossing
    costs 0.1 null collisions, a group costs its majorant excess times dz): checked
    against every partition of small random grids."""
    import itertools
    rng = np.random.default_rng(8)
    for trial in range(40):
        L = int(rng.integers(1, 10))
        dz = float(rng.choice([0.05, 0.5, 1.5625, 4.0]))
        maj = (rng.lognormal(-3.0, 1.5, size=L) * (rng.random(L) < 0.9)).astype(np.float32)
        starts = oracle.merge_groups(maj, dz)
        assert starts[0] == 0 and all(a < b for a, b in zip(starts, starts[1:])) and starts[-1] < L
        best = min(_group_cost(maj, [0] + [i + 1 for i in range(L - 1) if cut[i]], dz)
                   for cut in itertools.product((False, True), repeat=L - 1))
        assert _group_cost(maj, starts, dz) <= best * (1 + 1e-12) + 1e-15, (trial, L, dz, starts)
    # a uniform grid has no excess to pay for: one group; far-apart majorants in thick layers: none merge
    assert oracle.merge_groups(np.full(12, 0.02, np.float32), 1.0) == [0]
    assert oracle.merge_groups(np.array([1.0, 0.001, 1.0, 0.001], np.float32), 10.0) == [0, 1, 2, 3]


@pytest.mark.parametrize("tracking", [_abi.TRACKING_SEGMENT_RESTART, _abi.TRACKING_RESIDUAL_CARRY,
                                      _abi.TRACKING_MERGED_LAYERS])
def test_oracle_transmittance_known_answer(ref_scene, tracking):
    """The binary transmittance estimator (delta_transmittance,
    sky_trace.wgsl:441-475) averages to exp(-optical depth) along rays through
    the repository's medium, in every tracking mode: a vertical ray and a 5-degree
    ray from 100 m, in the bluest and the reddest band."""
    rg, rt, top = ref_scene.ground_radius_km, ref_scene.atmosphere_radius_km, ref_scene.top_altitude_km
    z, _, _, ext = analytic.knot_tables(ref_scene)
    o = np.array([0.0, rg + 0.1, 0.0])
    n = 40000
    for elev in (90.0, 5.0):
        d = np.array([math.cos(math.radians(elev)), math.sin(math.radians(elev)), 0.0])
        t_exit, _ = analytic._sphere_exit(o, d, rt)
        t = np.linspace(0.0, float(t_exit), 40001)
        alt = np.linalg.norm(o[None, :] + t[:, None] * d[None, :], axis=1) - rg
        for band in (0, ref_scene.band_count - 1):
            want = math.exp(-np.trapezoid(analytic._interp_alt(z, ext[band], alt, top), t))
            got = oracle.transmittance(ref_scene, tracking, o, d, band, n)
            se = math.sqrt(max(want * (1.0 - want), 1e-12) / n)
            assert abs(got - want) <= 4.0 * se + 1e-3, (elev, band, got, want, se)


def test_transmittance_on_descending_rays(ref_scene):
    """Rays that descend through shells to a tangent point, as shadow rays do
    at twilight.  Merged-layer tracking (mode 2) averages to exp(-optical
    depth) on all of them.  The reference's segment rule (modes 0 and 1,
    next_majorant_segment_end, sky_trace.wgsl:284-294) takes the next layer
    from the f32 altitude 5 m along the ray; a ray descending at a few degrees
    drops less than that altitude's resolution in 5 m, so at a downward shell
    crossing the probe still reads the upper layer and the segment runs past
    the tangent point under the upper layer's majorant: optical depth is
    skipped and the transmittance comes out too high.  The oracle keeps that
    behaviour in modes 0 and 1, since they restate the reference."""
    rg, rt, top = ref_scene.ground_radius_km, ref_scene.atmosphere_radius_km, ref_scene.top_altitude_km
    z, _, _, ext = analytic.knot_tables(ref_scene)
    n = 20000
    band = ref_scene.band_count - 1
    skipped = 0
    for h0, elev in ((10.0, -0.5), (10.0, -2.0), (20.0, -1.0), (20.0, -4.0), (40.0, -2.0), (40.0, -4.0)):
        o = np.array([0.0, rg + h0, 0.0])
        d = np.array([math.cos(math.radians(elev)), math.sin(math.radians(elev)), 0.0])
        t_exit, _ = analytic._sphere_exit(o, d, rt)
        t = np.linspace(0.0, float(t_exit), 80001)
        alt = np.linalg.norm(o[None, :] + t[:, None] * d[None, :], axis=1) - rg
        want = math.exp(-np.trapezoid(analytic._interp_alt(z, ext[band], alt, top), t))
        se = math.sqrt(max(want * (1.0 - want), 1e-12) / n)
        got = oracle.transmittance(ref_scene, _abi.TRACKING_MERGED_LAYERS, o, d, band, n)
        assert abs(got - want) <= 4.0 * se + 1e-3, (h0, elev, got, want)
        ref = oracle.transmittance(ref_scene, _abi.TRACKING_SEGMENT_RESTART, o, d, band, n)
        skipped += ref > want + 10.0 * se
    assert skipped >= 3  # the reference rule skips optical depth on the steeper of these rays
