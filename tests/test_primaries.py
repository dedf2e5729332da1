"""Wavelength-primary fitting on the GPU: a band moved by multipliers renders
the chains of a scene rebuilt at the new wavelength, and a short fit driven
by the adjoint (and one driven by plain-tracer finite differences) lowers
the reconstruction loss."""

import dataclasses

import numpy as np
import pytest

from sky_cuda import GpuScene, RenderConfig, synthetic_scene
from sky_cuda import _abi
from sky_cuda.adjoint import AdjointRenderer, initial_layer_params
from sky_cuda.primaries import (BandModel, PrimaryFitConfig, evaluate, fit_adjoint, fit_finite_differences,
                                target_xyz)

pytestmark = pytest.mark.gpu


def test_moved_band_traces_the_rebuilt_scene(gpu, data_dir):
    import torch
    lam0 = np.array([450.0, 520.0, 570.0, 630.0])
    lam1 = lam0 + np.array([-7.3, 4.1, 12.6, -2.2])
    s0 = synthetic_scene(lam0, data_dir, sun_elevation_deg=10.0)
    s1 = synthetic_scene(lam1, data_dir, sun_elevation_deg=10.0)
    cfg = RenderConfig(width=32, height=16, spp=1, sample_offset=7, phase_sampling=_abi.PHASE_TABULATED,
                       tracking=_abi.TRACKING_RESIDUAL_CARRY, kernel=_abi.KERNEL_PLAIN)
    k = BandModel(data_dir, lam0).multipliers(torch.as_tensor(lam1, device="cuda")).contiguous()
    with GpuScene(s0) as g0, GpuScene(s1) as g1:
        got = AdjointRenderer(g0, cfg).forward(
            torch.as_tensor(initial_layer_params(s0, 0.76), device="cuda"), k)["cell_sum"].cpu().numpy()
        s = torch.zeros(cfg.pixels * 4, dtype=torch.float64, device="cuda")
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        g1.render_device(cfg, {"cell_sum": s.data_ptr(), "status": st.data_ptr()},
                         torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        want = s.cpu().numpy()
    close = np.abs(got - want) <= 1e-3 * np.maximum(np.abs(got), np.abs(want)) + 1e-30
    print("chain agreement", close.mean())
    assert close.mean() >= 0.98


def test_short_fits_lower_the_loss(gpu, data_dir):
    cfg = PrimaryFitConfig(elevation_count=4, width=32, height=16, fit_spp=16, target_spp=64,
                           target_wavelengths=(380.0, 780.0, 41), iterations=12, lr_nm=2.0, data_dir=str(data_dir))
    target, target_var = target_xyz(cfg)
    adj = fit_adjoint(cfg, target)
    print("adjoint", adj["loss"][0], adj["loss"][-1], adj["lambda_nm"])
    assert np.mean(adj["loss"][-3:]) < adj["loss"][0]
    assert not np.allclose(adj["lambda_nm"], cfg.primaries_nm)
    ev = evaluate(cfg, adj["lambda_nm"], adj["matrix"], target, target_var, spp=32)
    assert 0.0 < ev["relative_xyz_error"] < 0.5 and ev["oklab"]["score"] > 0.0
    assert 0.0 <= ev["relative_rms_error_debiased"] <= ev["relative_rms_error"]
    fd = fit_finite_differences(dataclasses.replace(cfg, iterations=3), target)
    assert len(fd["loss"]) == 3 and np.all(np.isfinite(fd["loss"]))
