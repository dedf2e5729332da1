"""The per-pixel epilogue against its definition, given the very sums it read.

One render_device call returns the FP64 cell sums together with the film,
XYZ, XYZ variance and linear sRGB that the epilogue formed from them, so the
outputs are checked against numpy on the same sums:
    film  = max(f32(sum / n), 0)                    (integrator.rs:306-310)
    XYZ   = sum_b (sum_b / n) w_b                   (spectrum.rs:232-241, FP64)
    var   = sum_b (sumsq_b - sum_b^2 / n) / (n - 1) / n  w_b^2
    sRGB  = f32(M XYZ), black unless finite         (spectrum.rs:132-165)
Shapes are chosen off the kernel's tiling: band counts that are not
multiples of its four lanes per pixel, pixel counts that leave its last
block partly empty, one sample per cell (zero variance), and an
accumulating second pass (n = sample_offset + spp), through both the
single-render epilogue (plain kernel) and the job-table one (wavefront).
"""

import numpy as np
import pytest

from sky_cuda import GpuScene, RenderConfig, synthetic_scene, wavelengths
from sky_cuda import _abi
from sky_cuda.colorimetry import SpectralRgbConverter

pytestmark = pytest.mark.gpu


def _render_all(gs, cfg):
    import torch
    B = gs.band_count
    cells, px = cfg.pixels * B, cfg.pixels
    t = {
        "cell_sum": torch.zeros(cells, dtype=torch.float64, device="cuda"),
        "cell_sumsq": torch.zeros(cells, dtype=torch.float64, device="cuda"),
        "film": torch.full((cells,), -1.0, dtype=torch.float32, device="cuda"),
        "xyz": torch.full((px * 3,), -1.0, dtype=torch.float64, device="cuda"),
        "xyz_var": torch.full((px * 3,), -1.0, dtype=torch.float64, device="cuda"),
        "rgb": torch.full((px * 3,), -1.0, dtype=torch.float32, device="cuda"),
        "status": torch.zeros(1, dtype=torch.int32, device="cuda"),
    }
    return t


def _run(gs, cfg, t):
    import torch
    gs.render_device(cfg, {k: v.data_ptr() for k, v in t.items()}, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert int(t["status"].item()) == 0
    B = gs.band_count
    out = {k: v.cpu().numpy() for k, v in t.items()}
    out["cell_sum"] = out["cell_sum"].reshape(-1, B)
    out["cell_sumsq"] = out["cell_sumsq"].reshape(-1, B)
    out["film"] = out["film"].reshape(-1, B)
    for k in ("xyz", "xyz_var", "rgb"):
        out[k] = out[k].reshape(-1, 3)
    return out


def _check(scene, out, n):
    s, q = out["cell_sum"], out["cell_sumsq"]
    mean = s / n
    film_want = np.maximum(mean.astype(np.float32), np.float32(0.0))
    np.testing.assert_allclose(out["film"], film_want, rtol=2e-7, atol=0)
    w = np.asarray(scene.band_xyz, dtype=np.float64)
    np.testing.assert_allclose(out["xyz"], mean @ w, rtol=1e-12, atol=1e-300)
    if n > 1:
        v = np.maximum(q - s * mean, 0.0) / (n - 1) / n
        var_want = v @ (w * w)
    else:
        var_want = np.zeros_like(out["xyz"])
    np.testing.assert_allclose(out["xyz_var"], var_want, rtol=1e-9, atol=1e-300)
    m = SpectralRgbConverter.for_scene(scene).rgb_from_xyz().astype(np.float64)
    rgb_want = (out["xyz"] @ m.T).astype(np.float32)
    scale = float(np.abs(rgb_want).max())
    np.testing.assert_allclose(out["rgb"], rgb_want, rtol=1e-5, atol=1e-7 * scale)


@pytest.fixture(scope="module")
def odd_band_scene(data_dir):
    # 37 bands: 9 full groups of four lanes and one lane left over
    return synthetic_scene(wavelengths(380.0, 780.0, 37), data_dir, sun_elevation_deg=7.0)


@pytest.mark.parametrize("kernel", [_abi.KERNEL_PLAIN, _abi.KERNEL_WAVEFRONT])
@pytest.mark.parametrize("shape,spp", [((13, 7), 5), ((67, 3), 1), ((9, 9), 3)])
def test_epilogue_matches_definition(gpu, odd_band_scene, ref_scene, kernel, shape, spp):
    for scene in (odd_band_scene, ref_scene):
        cfg = RenderConfig(width=shape[0], height=shape[1], spp=spp, kernel=kernel,
                           phase_sampling=_abi.PHASE_TABULATED, tracking=_abi.TRACKING_MERGED_LAYERS)
        with GpuScene(scene) as gs:
            out = _run(gs, cfg, _render_all(gs, cfg))
        assert np.all(out["xyz"] != -1.0) and np.all(out["film"] != -1.0)
        _check(scene, out, spp)


@pytest.mark.parametrize("kernel", [_abi.KERNEL_PLAIN, _abi.KERNEL_WAVEFRONT])
def test_epilogue_after_accumulating_pass(gpu, odd_band_scene, kernel):
    base = dict(width=11, height=6, kernel=kernel, phase_sampling=_abi.PHASE_TABULATED,
                tracking=_abi.TRACKING_MERGED_LAYERS)
    with GpuScene(odd_band_scene) as gs:
        t = _render_all(gs, RenderConfig(spp=3, **base))
        _run(gs, RenderConfig(spp=3, **base), t)
        out = _run(gs, RenderConfig(spp=4, sample_offset=3, flags=_abi.FLAG_ACCUMULATE, **base), t)
    _check(odd_band_scene, out, 7)
