"""Differentiable rendering through the C ABI (sky_cuda_adjoint_*).

  * the primal over the parameterised medium at the scene's own parameters
    traces the plain tracer's chains (same random numbers) and matches its
    statistics;
  * the device majorant bake reproduces the scene's grid and a numpy bake of
    a perturbed medium;
  * the path-replay gradient equals central finite differences (h = 1e-3) of
    the same estimator with its samples held fixed (the sampling parameters
    stay at the evaluation point while the evaluated ones move);
  * summed along whole-atmosphere directions it agrees, within statistical
    error, with central differences of the plain tracer at 4096 spp;
  * the torch.autograd.Function returns the same gradient.
"""

import dataclasses

import numpy as np
import pytest

from sky_cuda import GpuScene, RenderConfig, SkyCudaError, synthetic_scene, wavelengths
from sky_cuda import _abi
from sky_cuda.adjoint import (BAND_PARAMS, NULL_COLLISIONS, SEGMENT_INTEGRALS, AdjointRenderer, fd_check_parameters,
                              film_to_xyz,
                              initial_layer_params, param_names, render_film)
from sky_cuda.scene import SPECIES_COUNT, hg_phase_values
from skystats import parity_report, xyz_from_sums

pytestmark = pytest.mark.gpu

G0 = 0.76  # HG asymmetry of the synthetic scene's aerosol


def _t(x, dtype=None):
    import torch
    return torch.as_tensor(np.asarray(x), device="cuda", dtype=dtype or torch.float32).contiguous()


def plain_sums(gs, cfg):
    import torch
    cells = cfg.pixels * gs.band_count
    s = torch.zeros(cells, dtype=torch.float64, device="cuda")
    q = torch.zeros(cells, dtype=torch.float64, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    gs.render_device(cfg, {"cell_sum": s.data_ptr(), "cell_sumsq": q.data_ptr(), "status": st.data_ptr()},
                     torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    return s.cpu().numpy(), q.cpu().numpy()


@pytest.fixture(scope="module")
def small_scene(data_dir):
    """8 bands (400-700 nm) of the benchmark atmosphere, sun at 10 degrees."""
    return synthetic_scene(wavelengths(400.0, 700.0, 8), data_dir, sun_elevation_deg=10.0)


@pytest.mark.parametrize("phase,lights", [(_abi.PHASE_ISOTROPIC, 1), (_abi.PHASE_TABULATED, 1),
                                          (_abi.PHASE_TABULATED, 3)])
def test_primal_traces_the_plain_chains(gpu, dome_scene, phase, lights):
    """One sample per cell: the adjoint primal (residual carry over the
    device-baked uniform layers) and the plain tracer (residual carry over the
    scene's grid) consume the same random numbers; their chains agree except
    where float rounding flips a decision (also with three sun samples per
    vertex)."""
    cfg = RenderConfig(width=32, height=16, spp=1, sample_offset=3, phase_sampling=phase,
                       tracking=_abi.TRACKING_RESIDUAL_CARRY, direct_light_samples=lights)
    with GpuScene(dome_scene) as gs:
        want, _ = plain_sums(gs, dataclasses.replace(cfg, kernel=_abi.KERNEL_PLAIN))
        r = AdjointRenderer(gs, cfg)
        got = r.forward(_t(initial_layer_params(dome_scene, G0)))["cell_sum"].cpu().numpy()
    close = np.abs(got - want) <= 1e-3 * np.maximum(np.abs(got), np.abs(want)) + 1e-30
    print("chain agreement", close.mean())
    assert close.mean() >= 0.98


def test_primal_statistics_match_plain_tracer(gpu, dome_scene):
    cfg = RenderConfig(width=32, height=16, spp=256, phase_sampling=_abi.PHASE_TABULATED,
                       tracking=_abi.TRACKING_MERGED_LAYERS)
    with GpuScene(dome_scene) as gs:
        s_p, q_p = plain_sums(gs, cfg)
        out = AdjointRenderer(gs, dataclasses.replace(cfg, seed=cfg.seed + 1)).forward(
            _t(initial_layer_params(dome_scene, G0)))
    s_a, q_a = out["cell_sum"].cpu().numpy(), out["cell_sumsq"].cpu().numpy()
    shape = (cfg.pixels, dome_scene.band_count)
    xa, va = xyz_from_sums(s_a.reshape(shape), q_a.reshape(shape), cfg.spp, dome_scene.band_xyz)
    xp, vp = xyz_from_sums(s_p.reshape(shape), q_p.reshape(shape), cfg.spp, dome_scene.band_xyz)
    rep = parity_report(xa, va, xp, vp)
    print("adjoint primal vs plain", rep)
    assert rep["frac_beyond_3se"] <= 0.02
    for b, se in zip(rep["bias_xyz"], rep["bias_se_xyz"]):
        assert abs(b) <= 4 * se + 1e-3


def _numpy_bake(scene, params, layers):
    """compute_majorant_grid's probe rule over the parameterised medium."""
    top = np.float32(scene.atmosphere_radius_km) - np.float32(scene.ground_radius_km)
    dz = top / np.float32(layers)
    atm, aer = scene.atmosphere, scene.aerosol
    opt = scene.aerosol_optics.reshape(scene.band_count, SPECIES_COUNT)[:, 0]
    ext0 = opt["scattering_km_inv_per_g_m3"].astype(np.float64) + opt["absorption_km_inv_per_g_m3"]
    xs_r = scene.bands["rayleigh_cross_section_m2"].astype(np.float64) * 1e9
    xs_o = scene.bands["ozone_cross_section_cm2"].astype(np.float64) * 1e5
    knots = np.concatenate([atm["altitude_km"], aer["altitude_km"]]).astype(np.float64)
    out = np.zeros((scene.band_count, layers))
    for l in range(layers):
        lo, hi = float(np.float32(l) * dz), float(np.float32(l + 1) * dz)
        h = np.array([lo, hi, 0.5 * (lo + hi)] + [z for z in knots if lo < z < hi])
        air = np.interp(h, atm["altitude_km"], atm["air_cm3"])
        o3 = np.interp(h, atm["altitude_km"], atm["ozone_cm3"])
        m0 = np.interp(h, aer["altitude_km"], aer["mass_g_m3"][:, 0])
        sr, sm, so = params[3 * l:3 * l + 3]
        ext = sr * xs_r[:, None] * air + sm * ext0[:, None] * m0 + so * xs_o[:, None] * o3
        out[:, l] = np.maximum(ext.max(axis=1) * 1.05, 1e-8)
    return out


def test_device_majorant_bake(gpu, dome_scene):
    layers = dome_scene.layer_count
    theta0 = initial_layer_params(dome_scene, G0)
    rng = np.random.default_rng(3)
    theta = theta0.copy()
    theta[:3 * layers] = (1.0 + rng.normal(0.0, 0.05, 3 * layers)).astype(np.float32)
    with GpuScene(dome_scene) as gs:
        r = AdjointRenderer(gs, RenderConfig(width=4, height=4, spp=1, tracking=_abi.TRACKING_MERGED_LAYERS))
        base = r.bake_majorants(_t(theta0)).cpu().numpy()
        moved = r.bake_majorants(_t(theta)).cpu().numpy()
    np.testing.assert_allclose(base, dome_scene.majorants, rtol=2e-5)
    np.testing.assert_allclose(moved, _numpy_bake(dome_scene, theta, layers), rtol=1e-4)


def _loss_setup(gs, scene, cfg, target_spp=256):
    """The adjoint benchmark's loss: L2 on XYZ against a target rendered at
    perturbed parameters.  The loss reads the FP64 cell sums (the float32
    film's rounding would swamp finite differences of small gradients)."""
    import torch
    layers = scene.layer_count
    theta0 = initial_layer_params(scene, G0)
    rng = np.random.default_rng(3)
    theta_t = theta0.copy()
    theta_t[:3 * layers] = (1.0 + rng.normal(0.0, 0.05, 3 * layers)).astype(np.float32)
    theta_t[3 * layers] *= np.float32(1.0 + rng.normal(0.0, 0.02))
    theta_t[3 * layers + 1] += np.float32(rng.normal(0.0, 0.02))
    tcfg = dataclasses.replace(cfg, spp=target_spp, seed=cfg.seed ^ 0xABCDEF)
    w = torch.as_tensor(np.asarray(scene.band_xyz, np.float64), device="cuda")

    def xyz_of(out, spp):
        return (out["cell_sum"] / spp).reshape(cfg.pixels, scene.band_count) @ w

    txyz = xyz_of(AdjointRenderer(gs, tcfg).forward(_t(theta_t)), target_spp)

    def loss_of(out):
        return float(((xyz_of(out, cfg.spp) - txyz) ** 2).sum().item())

    def dloss(out):
        return (2.0 * (xyz_of(out, cfg.spp) - txyz) @ w.T).float()

    return theta0, loss_of, dloss


@pytest.mark.parametrize("estimator", [SEGMENT_INTEGRALS, NULL_COLLISIONS])
def test_chain_buffer_backward_matches_retrace(gpu, small_scene, estimator):
    """A backward given the forward's chain radiance (one float per chain)
    replays each chain once instead of tracing it first for its radiance, and
    skips the chains that collected nothing: the same gradient, to the
    rounding of the per-warp FP32 gradient sums, with both estimators; band
    gradients too.  The buffer holds every chain's radiance (before the solar
    multiplier): per cell, the mean of its chains is the forward's film."""
    import torch
    cfg = RenderConfig(width=16, height=8, spp=32, phase_sampling=_abi.PHASE_TABULATED,
                       tracking=_abi.TRACKING_MERGED_LAYERS)
    B = small_scene.band_count
    with GpuScene(small_scene) as gs:
        theta0, _, dloss = _loss_setup(gs, small_scene, cfg)
        r = AdjointRenderer(gs, cfg, estimator=estimator)
        th0 = _t(theta0)
        band0 = _t(np.ones(B * BAND_PARAMS, dtype=np.float32))
        chains = r.new_chain_buffer()
        chains.fill_(-1.0)
        out = r.forward(th0, band0, chains=chains)
        d = dloss(out)
        lg_a, bg_a = r.backward(th0, band0, d, chains=chains)
        lg_b, bg_b = r.backward(th0, band0, d)
        with pytest.raises(ValueError):
            r.backward(th0, band0, d, chains=chains, decorrelate=True)
        with pytest.raises(SkyCudaError):
            r.forward(th0, band0, sample_layer=_t(theta0 * np.float32(1.01)), chains=chains)
    c = chains.cpu().numpy().reshape(cfg.pixels * B, cfg.spp)
    assert np.all(c >= 0.0) and np.any(c > 0.0)
    np.testing.assert_allclose(c.mean(axis=1), out["film"].cpu().numpy(), rtol=1e-5, atol=1e-7)
    for a, b in ((lg_a, lg_b), (bg_a, bg_b)):
        a, b = a.cpu().numpy(), b.cpu().numpy()
        assert np.any(a != 0.0)
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-4 * np.abs(b).max())


def test_decorrelated_backward_replays_its_own_chains_once(gpu, small_scene):
    """A decorrelated backward traces chains of another seed: it renders their
    radiance with the forward kernel into a buffer of its own, then replays
    each once.  Its gradient equals the backward of a renderer whose seed is
    that other seed (both passes in the gradient kernel), to the rounding of
    the per-warp FP32 gradient sums."""
    from sky_cuda.adjoint import DECORRELATE_SEED
    cfg = RenderConfig(width=16, height=8, spp=32, phase_sampling=_abi.PHASE_TABULATED,
                       tracking=_abi.TRACKING_MERGED_LAYERS)
    B = small_scene.band_count
    with GpuScene(small_scene) as gs:
        theta0, _, dloss = _loss_setup(gs, small_scene, cfg)
        r = AdjointRenderer(gs, cfg)
        th0 = _t(theta0)
        band0 = _t(np.ones(B * BAND_PARAMS, dtype=np.float32))
        d = dloss(r.forward(th0, band0))
        lg_a, bg_a = r.backward(th0, band0, d, decorrelate=True)
        other = AdjointRenderer(gs, dataclasses.replace(cfg, seed=cfg.seed ^ DECORRELATE_SEED))
        lg_b, bg_b = other.backward(th0, band0, d)
        lg_c, _ = r.backward(th0, band0, d)  # the forward's own chains: another estimate
    for a, b in ((lg_a, lg_b), (bg_a, bg_b)):
        a, b = a.cpu().numpy(), b.cpu().numpy()
        assert np.any(a != 0.0)
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-4 * np.abs(b).max())
    assert not np.allclose(lg_a.cpu().numpy(), lg_c.cpu().numpy(), rtol=1e-3)


def test_gradient_matches_central_differences(gpu, dome_scene):
    """The adjoint benchmark's finite-difference check (h = 1e-3) on a 32x16
    image, 32 bands, 64 spp: 16 parameters that all carry a gradient, drawn
    with seed 4 evenly from the Rayleigh, Mie and ozone layer scales, plus the
    Mie albedo and g; each within 1e-2 relative of central differences."""
    cfg = RenderConfig(width=32, height=16, spp=64, phase_sampling=_abi.PHASE_TABULATED,
                       tracking=_abi.TRACKING_MERGED_LAYERS)
    h = 1e-3
    with GpuScene(dome_scene) as gs:
        theta0, loss_of, dloss = _loss_setup(gs, dome_scene, cfg)
        r = AdjointRenderer(gs, cfg, estimator=NULL_COLLISIONS)
        th0 = _t(theta0)
        grad, _ = r.backward(th0, None, dloss(r.forward(th0)))
        grad = grad.cpu().numpy()
        L = dome_scene.layer_count
        idx = fd_check_parameters(grad, L, count=16, seed=4)
        assert len(idx) == 16 and 3 * L in idx and 3 * L + 1 in idx
        assert {i % 3 for i in idx if i < 3 * L} == {0, 1, 2}  # every species
        names = param_names(L)
        rows = []
        for i in idx:
            tp, tm = theta0.copy(), theta0.copy()
            tp[i] += np.float32(h)
            tm[i] -= np.float32(h)
            jp = loss_of(r.forward(_t(tp), sample_layer=th0))
            jm = loss_of(r.forward(_t(tm), sample_layer=th0))
            rows.append((names[i], (jp - jm) / float(tp[i] - tm[i]), grad[i]))
    scale = np.abs(grad).max()
    for name, fd, g in rows:
        print(f"{name:14s} fd {fd: .6e} adjoint {g: .6e} rel {abs(fd - g) / abs(fd):.2e}")
    for name, fd, g in rows:
        assert fd != 0.0 and abs(fd - g) <= 1e-2 * abs(fd), name


def test_band_gradients_match_central_differences(gpu, small_scene):
    cfg = RenderConfig(width=16, height=8, spp=64, phase_sampling=_abi.PHASE_TABULATED,
                       tracking=_abi.TRACKING_MERGED_LAYERS)
    h = 1e-3
    B = small_scene.band_count
    with GpuScene(small_scene) as gs:
        theta0, loss_of, dloss = _loss_setup(gs, small_scene, cfg)
        r = AdjointRenderer(gs, cfg, estimator=NULL_COLLISIONS)
        th0 = _t(theta0)
        band0 = np.ones(B * BAND_PARAMS, dtype=np.float32)
        b0 = _t(band0)
        lg, bg = r.backward(th0, b0, dloss(r.forward(th0, b0)))
        bg = bg.cpu().numpy()
        rows = []
        for b in (1, 5):
            for k in range(BAND_PARAMS):
                i = b * BAND_PARAMS + k
                bp, bm = band0.copy(), band0.copy()
                bp[i] += np.float32(h)
                bm[i] -= np.float32(h)
                jp = loss_of(r.forward(th0, _t(bp), sample_band=b0))
                jm = loss_of(r.forward(th0, _t(bm), sample_band=b0))
                rows.append((f"band{b}.{('R', 'M', 'O', 'S')[k]}", (jp - jm) / float(bp[i] - bm[i]), bg[i]))
    scale = np.abs(bg).max()
    for name, fd, g in rows:
        print(f"{name:10s} fd {fd: .6e} adjoint {g: .6e}")
    for name, fd, g in rows:
        assert abs(fd - g) <= 1e-2 * abs(fd) + 2e-5 * scale, name


def _scene_along(scene, direction, delta):
    """The synthetic scene moved along one whole-atmosphere direction."""
    s = dataclasses.replace(scene)
    bands = scene.bands.copy()
    optics = scene.aerosol_optics.copy()
    phase = scene.phase_values.copy()
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
        omega = sca / ext + delta
        optics["scattering_km_inv_per_g_m3"][0::SPECIES_COUNT] = ext * omega
        optics["absorption_km_inv_per_g_m3"][0::SPECIES_COUNT] = ext * (1 - omega)
    elif direction == "g":
        phase[0] = hg_phase_values(G0 + delta, scene.phase_bins)[None, :]
    s.bands, s.aerosol_optics, s.phase_values = bands, optics, phase
    return s.bake_majorants(scene.layer_count)


def _sun_pixels(scene, cfg):
    """Panorama pixels whose footprint holds part of the sun disc
    (panorama_dir, sky_trace.wgsl:614-623, inverted)."""
    x, y, z = scene.sun_direction
    u = np.arctan2(x, z) / (2 * np.pi) + 0.5
    v = 0.5 - np.arcsin(y) / np.pi
    r = scene.sun_angular_radius_rad
    px = np.arange(cfg.pixels) % cfg.width
    py = np.arange(cfg.pixels) // cfg.width
    du, dv = r / (2 * np.pi * max(np.cos(np.arcsin(y)), 1e-3)), r / np.pi
    return ((px + 1) / cfg.width >= u - du) & (px / cfg.width <= u + du) & \
        ((py + 1) / cfg.height >= v - dv) & (py / cfg.height <= v + dv)


@pytest.mark.parametrize("estimator", [SEGMENT_INTEGRALS, NULL_COLLISIONS])
@pytest.mark.parametrize("direction,delta", [("rayleigh", 0.05), ("mie", 0.05), ("ozone", 0.2), ("albedo", 0.02),
                                             ("g", 0.02)])
def test_gradient_matches_plain_tracer_differences(gpu, small_scene, direction, delta, estimator):
    """The adjoint gradient projected on a whole-atmosphere direction against
    central differences of the plain tracer (scene tables moved along the
    direction, 4096 spp in 16 batches, common seeds), for the linear loss
    J = sum_cells w_cell film_cell (pixels holding the sun disc weighted 0)."""
    import torch
    batches, spp = 16, 256
    L = small_scene.layer_count
    cfg = RenderConfig(width=16, height=8, spp=spp, phase_sampling=_abi.PHASE_TABULATED,
                       tracking=_abi.TRACKING_MERGED_LAYERS)
    cells = cfg.pixels * small_scene.band_count
    w = np.random.default_rng(7).uniform(0.5, 1.5, (cfg.pixels, small_scene.band_count)) / cells
    w[_sun_pixels(small_scene, cfg)] = 0.0  # the sun disc's rare hits would dominate both variances
    w = w.reshape(-1)
    proj = {"rayleigh": lambda g: g[0:3 * L:3].sum(), "mie": lambda g: g[1:3 * L:3].sum(),
            "ozone": lambda g: g[2:3 * L:3].sum(), "albedo": lambda g: g[3 * L], "g": lambda g: g[3 * L + 1]}[direction]
    fd, adj = [], []
    with GpuScene(_scene_along(small_scene, direction, +delta)) as gp, \
            GpuScene(_scene_along(small_scene, direction, -delta)) as gm, GpuScene(small_scene) as g0:
        th0 = _t(initial_layer_params(small_scene, G0))
        wt = _t(w)
        for k in range(batches):
            c = dataclasses.replace(cfg, sample_offset=k * spp)
            jp = float(np.dot(plain_sums(gp, c)[0], w)) / spp
            jm = float(np.dot(plain_sums(gm, c)[0], w)) / spp
            fd.append((jp - jm) / (2 * delta))
            rk = AdjointRenderer(g0, c, estimator=estimator)
            lg, _ = rk.backward(th0, None, wt)
            adj.append(proj(lg.cpu().numpy()))
    fd, adj = np.array(fd), np.array(adj)
    se = np.sqrt(fd.var(ddof=1) / batches + adj.var(ddof=1) / batches)
    print(f"{direction} (estimator {estimator}): plain FD {fd.mean():.6e} +- {fd.std(ddof=1) / 4:.2e}, "
          f"adjoint {adj.mean():.6e} +- {adj.std(ddof=1) / 4:.2e}")
    assert abs(fd.mean() - adj.mean()) <= 4 * se + 0.02 * abs(fd.mean())


def test_autograd_function_matches_direct_backward(gpu, small_scene):
    import torch
    cfg = RenderConfig(width=16, height=8, spp=32, phase_sampling=_abi.PHASE_TABULATED,
                       tracking=_abi.TRACKING_MERGED_LAYERS)
    with GpuScene(small_scene) as gs:
        r = AdjointRenderer(gs, cfg)
        layer = _t(initial_layer_params(small_scene, G0)).requires_grad_(True)
        band = _t(np.ones(small_scene.band_count * BAND_PARAMS, np.float32)).requires_grad_(True)
        target = torch.zeros((cfg.height, cfg.width, 3), dtype=torch.float64, device="cuda")
        film = render_film(r, layer, band)
        assert film.shape == (cfg.height, cfg.width, small_scene.band_count)
        xyz = film_to_xyz(film, small_scene)
        loss = ((xyz - target) ** 2).sum()
        loss.backward()
        w = torch.as_tensor(np.asarray(small_scene.band_xyz, np.float64), device="cuda")
        d = (2.0 * xyz.detach().reshape(-1, 3) @ w.T).float()
        lg, bg = r.backward(layer.detach(), band.detach(), d)
    np.testing.assert_allclose(layer.grad.cpu().numpy(), lg.float().cpu().numpy(), rtol=1e-4,
                               atol=1e-6 * float(lg.abs().max()))
    np.testing.assert_allclose(band.grad.cpu().numpy(), bg.float().cpu().numpy(), rtol=1e-4,
                               atol=1e-6 * float(bg.abs().max()))


def test_batch_matches_separate_renders(gpu, small_scene):
    """The batched forward and backward (one launch per direction for every
    sun) against the single-render calls at each sun: films and cell sums
    equal to FP64 rounding (the same chains), the gradient of the summed loss
    to the per-warp FP32 rounding; also with chain-radiance buffers, with a
    decorrelated backward, and through the batched autograd Function."""
    import torch
    from sky_cuda import sun_from_degrees
    from sky_cuda.adjoint import render_films
    cfg = RenderConfig(width=16, height=8, spp=32, phase_sampling=_abi.PHASE_TABULATED,
                       tracking=_abi.TRACKING_MERGED_LAYERS)
    B = small_scene.band_count
    suns = [sun_from_degrees(e, 0.0, small_scene.sun_angular_radius_rad)[0] for e in (-2.0, 5.0, 30.0)]
    rng = np.random.default_rng(11)
    with GpuScene(small_scene) as gs:
        r = AdjointRenderer(gs, cfg)
        th0 = _t(initial_layer_params(small_scene, G0))
        band0 = _t(np.ones(B * BAND_PARAMS, dtype=np.float32))
        single = [r.forward(th0, band0, sun=s) for s in suns]
        batch = r.forward_batch(th0, band0, suns)
        for a, b in zip(single, batch):
            np.testing.assert_allclose(b["cell_sum"].cpu().numpy(), a["cell_sum"].cpu().numpy(), rtol=1e-12, atol=0)
            np.testing.assert_allclose(b["film"].cpu().numpy(), a["film"].cpu().numpy(), rtol=1e-6, atol=0)
        ds = [_t(rng.normal(size=cfg.pixels * B).astype(np.float32)) for _ in suns]
        lg_b, bg_b = r.backward_batch(th0, band0, ds, suns)
        parts = [r.backward(th0, band0, d, sun=s) for d, s in zip(ds, suns)]
        lg_s = sum(p_[0] for p_ in parts)
        bg_s = sum(p_[1] for p_ in parts)
        chains = [r.new_chain_buffer() for _ in suns]
        r.forward_batch(th0, band0, suns, chains=chains)
        lg_c, bg_c = r.backward_batch(th0, band0, ds, suns, chains=chains)
        lg_d, _ = r.backward_batch(th0, band0, ds, suns, decorrelate=True)
        lg_ds = sum(r.backward(th0, band0, d, sun=s, decorrelate=True)[0] for d, s in zip(ds, suns))
        # the batched autograd Function: films stacked, gradient of their summed loss
        layer = th0.clone().requires_grad_(True)
        films = render_films(r, layer, band0, suns=suns)
        assert films.shape == (len(suns), cfg.height, cfg.width, B)
        np.testing.assert_allclose(films[1].reshape(-1).detach().cpu().numpy(),
                                   single[1]["film"].cpu().numpy(), rtol=1e-6, atol=0)
        (films.reshape(len(suns), -1) * torch.stack(ds)).sum().backward()
    for a, b in ((lg_b, lg_s), (bg_b, bg_s), (lg_c, lg_s), (bg_c, bg_s), (lg_d, lg_ds),
                 (layer.grad.double(), lg_s)):
        a, b = a.cpu().numpy(), b.cpu().numpy()
        assert np.any(b != 0.0)
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-4 * np.abs(b).max())


def test_batch_beyond_one_launch(gpu, small_scene):
    """33 renders take two launches per direction (32 + 1): each film equals
    its single render, the gradient of the summed loss equals the sum of the
    single gradients; a 33-render batch whose last render is refused returns
    SKY_ERR_INVALID_CONFIG before any launch, so no render's outputs change."""
    import ctypes
    import torch
    from sky_cuda import sun_from_degrees
    cfg = RenderConfig(width=4, height=4, spp=4, phase_sampling=_abi.PHASE_TABULATED,
                       tracking=_abi.TRACKING_MERGED_LAYERS)
    B = small_scene.band_count
    suns = [sun_from_degrees(e, 10.0 * e, small_scene.sun_angular_radius_rad)[0]
            for e in np.linspace(-3.0, 60.0, 33)]
    rng = np.random.default_rng(3)
    with GpuScene(small_scene) as gs:
        r = AdjointRenderer(gs, cfg)
        th = _t(initial_layer_params(small_scene, G0))
        band = _t(np.ones(B * BAND_PARAMS, dtype=np.float32))
        batch = r.forward_batch(th, band, suns)
        for i in (0, 31, 32):
            single = r.forward(th, band, sun=suns[i])
            np.testing.assert_allclose(batch[i]["cell_sum"].cpu().numpy(), single["cell_sum"].cpu().numpy(),
                                       rtol=1e-12, atol=0)
        ds = [_t(rng.normal(size=cfg.pixels * B).astype(np.float32)) for _ in suns]
        lg_b, _ = r.backward_batch(th, band, ds, suns)
        lg_s = sum(r.backward(th, band, d, sun=sn)[0] for d, sn in zip(ds, suns))
        # the refused batch: every render's cell sums hold a sentinel before and after
        outs = [{"cell_sum": torch.full((cfg.pixels * B,), -7.0, dtype=torch.float64, device="cuda")}
                for _ in suns]
        jobs = r._jobs(suns, r._c_config, outputs=outs)
        jobs[32].config.tracking = _abi.TRACKING_RESIDUAL_CARRY
        p = r._params(th, band)
        assert gs.lib.sky_cuda_adjoint_forward_batch(gs.handle, jobs, len(suns), ctypes.byref(p),
                                                     None) == _abi.SKY_ERR_INVALID_CONFIG
        assert "same tracking" in _abi.last_error(gs.lib)
        torch.cuda.synchronize()
        assert all(bool((o["cell_sum"] == -7.0).all()) for o in outs)
    a, b = lg_b.cpu().numpy(), lg_s.cpu().numpy()
    assert np.any(b != 0.0)
    np.testing.assert_allclose(a, b, rtol=0, atol=1e-4 * np.abs(b).max())


def test_adjoint_errors(gpu, ref_scene, dome_scene):
    import ctypes
    import torch
    with GpuScene(ref_scene) as gs:  # the reference's four aerosol species
        r = AdjointRenderer(gs, RenderConfig(width=4, height=4, spp=1))
        with pytest.raises(SkyCudaError, match="species"):
            r.forward(torch.ones(r.param_count, device="cuda"))
    with GpuScene(dome_scene) as gs:
        lib = gs.lib
        cfg = RenderConfig(width=4, height=4, spp=1, tracking=_abi.TRACKING_SEGMENT_RESTART).to_c()
        th = _t(initial_layer_params(dome_scene, G0))
        p = _abi.SkyAdjointParams()
        p.layer_params = th.data_ptr()
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        s = torch.zeros(16 * dome_scene.band_count, dtype=torch.float64, device="cuda")
        o = _abi.SkyDeviceOutputs()
        o.cell_sum, o.status = s.data_ptr(), st.data_ptr()
        assert lib.sky_cuda_adjoint_forward(gs.handle, ctypes.byref(cfg), ctypes.byref(p), ctypes.byref(o),
                                            None) == _abi.SKY_ERR_INVALID_CONFIG
        assert "RESIDUAL_CARRY" in _abi.last_error(lib)
        r = AdjointRenderer(gs, RenderConfig(width=4, height=4, spp=1))
        other = th.clone()  # a second parameter set is refused by the backward call
        p.sample_layer_params = other.data_ptr()
        g = _abi.SkyAdjointGrads()
        d = torch.zeros(16 * dome_scene.band_count, device="cuda")
        lg = torch.zeros(r.param_count, dtype=torch.float64, device="cuda")
        g.dloss_dfilm, g.layer_grad, g.status = d.data_ptr(), lg.data_ptr(), st.data_ptr()
        assert lib.sky_cuda_adjoint_backward(gs.handle, ctypes.byref(r._c_config), ctypes.byref(p),
                                             ctypes.byref(g), None) == _abi.SKY_ERR_INVALID_CONFIG
        assert lib.sky_cuda_adjoint_param_count(gs.handle) == 3 * dome_scene.layer_count + 2
        # batches: one parameter set, one tracking mode, phase sampling and accumulate flag
        assert lib.sky_cuda_adjoint_forward_batch(gs.handle, None, 0, ctypes.byref(p),
                                                  None) == _abi.SKY_ERR_INVALID_CONFIG
        p.sample_layer_params = None
        jobs = (_abi.SkyAdjointJob * 2)()
        for j in jobs:
            j.config = RenderConfig(width=4, height=4, spp=1, tracking=_abi.TRACKING_MERGED_LAYERS).to_c()
            j.outputs.cell_sum, j.outputs.status = s.data_ptr(), st.data_ptr()
            j.dloss_dfilm = d.data_ptr()
        jobs[1].config.tracking = _abi.TRACKING_RESIDUAL_CARRY
        assert lib.sky_cuda_adjoint_forward_batch(gs.handle, jobs, 2, ctypes.byref(p),
                                                  None) == _abi.SKY_ERR_INVALID_CONFIG
        assert "same tracking" in _abi.last_error(lib)
        jobs[1].config.tracking = _abi.TRACKING_MERGED_LAYERS
        jobs[1].config.phase_sampling = _abi.PHASE_TABULATED
        assert lib.sky_cuda_adjoint_backward_batch(gs.handle, jobs, 2, ctypes.byref(p), ctypes.byref(g),
                                                   None) == _abi.SKY_ERR_INVALID_CONFIG
        assert "phase sampling" in _abi.last_error(lib)
        jobs[1].config.phase_sampling = _abi.PHASE_ISOTROPIC
        jobs[1].config.flags = _abi.FLAG_ACCUMULATE
        assert lib.sky_cuda_adjoint_forward_batch(gs.handle, jobs, 2, ctypes.byref(p),
                                                  None) == _abi.SKY_ERR_INVALID_CONFIG
        assert "accumulate" in _abi.last_error(lib)
        jobs[1].config.flags = 0
        assert lib.sky_cuda_adjoint_forward_batch(gs.handle, jobs, 2, ctypes.byref(p), None) == _abi.SKY_OK
        torch.cuda.synchronize()
        assert int(st.item()) == 0
