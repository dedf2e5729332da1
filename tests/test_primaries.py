"""Wavelength-primary fitting on the GPU: a band moved by multipliers renders
the chains of a scene rebuilt at the new wavelength, and short fits driven by
the adjoint and by plain-tracer finite differences run end to end."""

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


def test_short_fits_run_end_to_end(gpu, data_dir):
    """Twelve adjoint steps and three finite-difference steps on a small image:
    the primaries move, every loss is finite and stays at its initial level, and
    the evaluation of the result is consistent.  At this size each step's loss
    is dominated by Monte Carlo noise (it varies by tens of percent between
    steps), so a short fit cannot show a decrease; the gradients themselves are
    checked against central differences in test_adjoint.py, and the full-size
    fit's reduction of the error is measured by the benchmark."""
    cfg = PrimaryFitConfig(primaries_nm=(410.0, 450.0, 490.0, 530.0), elevation_count=4, width=16, height=8,
                           fit_spp=256, target_spp=256, target_wavelengths=(380.0, 780.0, 41), iterations=12,
                           lr_nm=2.0, data_dir=str(data_dir))
    target, target_var = target_xyz(cfg)
    adj = fit_adjoint(cfg, target)
    print("adjoint", adj["loss"], adj["lambda_nm"])
    loss = np.asarray(adj["loss"])
    assert loss.shape == (12,) and np.all(np.isfinite(loss)) and np.all(loss > 0.0)
    assert np.mean(loss[-4:]) < 2.0 * np.mean(loss[:4])
    moved = np.abs(np.asarray(adj["lambda_nm"]) - np.asarray(cfg.primaries_nm))
    # an Adam step moves a parameter by at most lr (1 - beta1) / sqrt(1 - beta2) = 3.16 lr
    assert np.all(moved > 0.0) and np.all(moved <= 12 * cfg.lr_nm * 3.2)
    ev = evaluate(cfg, adj["lambda_nm"], adj["matrix"], target, target_var, spp=32)
    assert 0.0 < ev["relative_xyz_error"] < 0.5 and ev["oklab"]["score"] > 0.0
    assert 0.0 <= ev["relative_rms_error_debiased"] <= ev["relative_rms_error"]
    fd = fit_finite_differences(dataclasses.replace(cfg, iterations=3), target)
    assert len(fd["loss"]) == 3 and np.all(np.isfinite(fd["loss"]))
