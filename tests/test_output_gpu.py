"""The output stage on the GPU: the tracer's epilogue writes white-balanced
linear sRGB, and the sky-reference-render mirror writes band EXRs, the RGB
EXR/PNG and asset.json from one render."""

import json

import numpy as np
import pytest

from sky_cuda import GpuScene, RenderConfig
from sky_cuda import _abi
from sky_cuda.colorimetry import SpectralRgbConverter

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kernel", [_abi.KERNEL_PLAIN, _abi.KERNEL_WAVEFRONT])
def test_epilogue_rgb_matches_host_conversion(gpu, dome_scene, kernel):
    cfg = RenderConfig(width=16, height=8, spp=64, kernel=kernel, phase_sampling=_abi.PHASE_TABULATED,
                       tracking=_abi.TRACKING_MERGED_LAYERS)
    with GpuScene(dome_scene) as gs:
        film, rgb, _ = gs.render_rgb(cfg)
    want = SpectralRgbConverter.for_scene(dome_scene).to_linear_srgb(film.values.reshape(cfg.pixels, -1))
    scale = float(np.abs(want).max())
    np.testing.assert_allclose(rgb, want, rtol=2e-4, atol=1e-6 * scale)


def test_reference_render_cli_writes_every_output(gpu, tmp_path, data_dir):
    from sky_cuda.exr import read_exr, read_png_rgb8
    from sky_cuda.reference_render import main
    out = tmp_path / "out"
    assert main(["--width", "16", "--height", "8", "--spp", "8", "--out", str(out), "--data-dir", str(data_dir),
                 "--sun-elevation-deg", "10"]) == 0
    m = json.loads((out / "asset.json").read_text())
    assert m["kind"] == "spectral_panorama_v0" and m["dimensions"] == [16, 8] and m["spp"] == 8
    assert len(m["files"]["band_exrs"]) == len(m["band_centers_nm"]) == 41
    for name in m["files"]["band_exrs"]:
        ch = read_exr(out / name)
        assert ch["R"].shape == (8, 16) and np.all(np.isfinite(ch["R"])) and np.all(ch["R"] >= 0)
        np.testing.assert_array_equal(ch["R"], ch["G"])
    rgb = read_exr(out / "sky_rgb.exr")
    assert rgb["R"].shape == (8, 16) and np.all(np.isfinite(rgb["G"]))
    assert read_png_rgb8(out / "sky_rgb.png").shape == (8, 16, 3)
    # the rebuild path reproduces the RGB of the render from the band EXRs (host conversion vs epilogue)
    before = np.stack([rgb["R"], rgb["G"], rgb["B"]], axis=-1)
    assert main(["--out", str(out), "--data-dir", str(data_dir), "--rebuild-rgb-only"]) == 0
    after = read_exr(out / "sky_rgb.exr")
    after = np.stack([after["R"], after["G"], after["B"]], axis=-1)
    np.testing.assert_allclose(after, before, rtol=5e-3, atol=1e-4 * float(np.abs(before).max()))
