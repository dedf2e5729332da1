"""Host side of the wavelength-primary fit (no GPU): the band model's
multipliers against scenes built at the shifted wavelengths, their
derivatives, and the Oklab scoring."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from sky_cuda import synthetic_scene
from sky_cuda.primaries import BandModel, oklab_score_host as oklab_score, xyz_to_oklab


def test_band_multipliers_match_rebuilt_scenes(data_dir):
    lam0 = np.array([450.0, 520.0, 570.0, 630.0])
    lam1 = lam0 + np.array([-7.3, 4.1, 12.6, -2.2])
    model = BandModel(data_dir, lam0, device="cpu")
    k = model.multipliers(torch.as_tensor(lam1)).numpy()
    s0 = synthetic_scene(lam0, data_dir, sun_elevation_deg=10.0)
    s1 = synthetic_scene(lam1, data_dir, sun_elevation_deg=10.0)
    for col, field in ((0, "rayleigh_cross_section_m2"), (2, "ozone_cross_section_cm2"),
                       (3, "solar_radiance_w_m2_sr")):
        want = s1.bands[field].astype(np.float64) / s0.bands[field].astype(np.float64)
        np.testing.assert_allclose(k[:, col], want, rtol=2e-6)
    np.testing.assert_array_equal(k[:, 1], 1.0)
    np.testing.assert_allclose(model.multipliers(torch.as_tensor(lam0)).numpy(), 1.0, rtol=1e-7)


def test_band_multiplier_derivatives(data_dir):
    lam0 = np.array([455.0, 610.0])
    model = BandModel(data_dir, lam0, device="cpu")
    lam = torch.tensor([458.3, 603.7], dtype=torch.float64, requires_grad=True)
    k = model.multipliers(lam).double()
    # Rayleigh: d/dlambda (lambda0/lambda)^4 = -4 k / lambda
    g = torch.autograd.grad(k[:, 0].sum(), lam, retain_graph=True)[0].numpy()
    np.testing.assert_allclose(g, -4.0 * k[:, 0].detach().numpy() / lam.detach().numpy(), rtol=1e-6)
    # ozone / sun: slope of the bands.csv segment holding lambda (piecewise linear)
    for col, tab in ((2, 1), (3, 2)):
        g = torch.autograd.grad(k[:, col].sum(), lam, retain_graph=True)[0].numpy()
        eps = 1e-4
        ref = model.ref[tab].numpy()
        hi = model.tables(lam.detach() + eps)[tab].numpy() / ref
        lo = model.tables(lam.detach() - eps)[tab].numpy() / ref
        np.testing.assert_allclose(g, (hi - lo) / (2 * eps), rtol=1e-5)


def test_oklab_of_d65_white_is_neutral():
    # Oklab maps the D65 white point (normalised Y = 1) to L = 1, a = b = 0
    lab = xyz_to_oklab(torch.tensor([[0.95047, 1.0, 1.08883]], dtype=torch.float64)).numpy()[0]
    np.testing.assert_allclose(lab, [1.0, 0.0, 0.0], atol=2e-4)


def test_oklab_score_of_identity_is_zero():
    xyz = torch.rand(1000, 3, dtype=torch.float64) + 0.01
    s = oklab_score(xyz, xyz)
    assert s["rmse"] == 0.0 and s["score"] == 0.0
    s = oklab_score(xyz * 1.1, xyz)
    assert s["rmse"] > 0 and s["score"] == pytest.approx(s["rmse"] + 0.25 * s["p95"])


def test_spacing_penalty_pushes_close_primaries_apart():
    from sky_cuda.primaries import PrimaryFitConfig, spacing_penalty
    cfg = PrimaryFitConfig()
    far = torch.tensor([450.0, 520.0, 570.0, 630.0], dtype=torch.float64)
    assert float(spacing_penalty(far, cfg)) == 0.0
    # two pairs 1 nm apart (what the unconstrained fit converged to): each pair costs (9/10)^2
    lam = torch.tensor([479.0, 480.0, 579.0, 580.0], dtype=torch.float64, requires_grad=True)
    pen = spacing_penalty(lam, cfg)
    assert pen.item() == pytest.approx(cfg.spacing_weight * 2 * 0.81)
    pen.backward()
    g = lam.grad.numpy()
    # descending the penalty separates each pair
    assert g[0] > 0 > g[1] and g[2] > 0 > g[3]
    off = PrimaryFitConfig(min_spacing_nm=0.0)
    assert float(spacing_penalty(lam.detach(), off)) == 0.0


def test_oklab_objective_matches_score_and_stays_finite():
    from sky_cuda.primaries import Objective, PrimaryFitConfig, oklab_smooth
    gen = torch.Generator().manual_seed(7)
    # away from zero the smoothed cube root is the exact one
    xyz = torch.rand(500, 3, generator=gen, dtype=torch.float64) * 0.8 + 0.2
    np.testing.assert_allclose(oklab_smooth(xyz, 1e-6).numpy(), xyz_to_oklab(xyz).numpy(), rtol=1e-9, atol=1e-9)
    # the objective of two elevations x 40 pixels, pixel 0 of each row left out
    cfg = PrimaryFitConfig(width=8, height=5)
    target = torch.rand(2, 40, 3, generator=gen, dtype=torch.float64)
    keep = (torch.arange(40) % 8 >= 1).to(torch.float64)[:, None]
    obj = Objective(cfg, target, keep)
    assert float(obj(target)) == 0.0
    # it is the mean squared Oklab distance with XYZ scaled by the targets' p99 Y
    # (the rmse term of the score, squared), here where no LMS value is near zero
    xyz_hat = target * 1.05 + 0.01
    sel = keep[:, 0].bool()
    ref = oklab_score(xyz_hat[:, sel], target[:, sel])["rmse"] ** 2
    assert float(obj(xyz_hat)) == pytest.approx(ref, rel=2e-3)
    # finite gradients through reconstructions at and below zero
    xyz_hat = torch.zeros(2, 40, 3, dtype=torch.float64, requires_grad=True)
    obj(xyz_hat - 1e-9).backward()
    assert torch.all(torch.isfinite(xyz_hat.grad))
    with pytest.raises(ValueError):
        Objective(PrimaryFitConfig(width=8, height=5, loss="l1"), target, keep)
