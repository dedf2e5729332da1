"""The output stage of sky-reference-render, host side (no GPU): OpenEXR and
PNG files, the solar-white-to-D65 colour conversion, the asset manifest and
the --rebuild-rgb-only path."""

import json
import struct
import zlib

import numpy as np
import pytest

from sky_cuda import colorimetry as cm
from sky_cuda.exr import (ZIP_COMPRESSION, ZIPS_COMPRESSION, read_exr, read_png_rgb8, write_exr_rgb,
                          write_png_rgb8)


def test_exr_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    img = rng.uniform(0, 50, (7, 13, 3)).astype(np.float32)
    write_exr_rgb(tmp_path / "a.exr", img)
    ch = read_exr(tmp_path / "a.exr")
    assert sorted(ch) == ["B", "G", "R"]
    np.testing.assert_array_equal(np.stack([ch["R"], ch["G"], ch["B"]], axis=-1), img)


def _zip_exr(path, img, compression):
    """A ZIP/ZIPS-compressed float RGB EXR built by the format's steps (split
    even/odd bytes, delta predictor, zlib), to exercise the reader."""
    h, w = img.shape[:2]
    per = 16 if compression == ZIP_COMPRESSION else 1
    def attr(name, kind, payload):
        return name.encode() + b"\0" + kind.encode() + b"\0" + struct.pack("<i", len(payload)) + payload
    chans = b"".join(c.encode() + b"\0" + struct.pack("<iB3xii", 2, 0, 1, 1) for c in "BGR") + b"\0"
    header = (attr("channels", "chlist", chans) + attr("compression", "compression", bytes([compression])) +
              attr("dataWindow", "box2i", struct.pack("<iiii", 0, 0, w - 1, h - 1)) +
              attr("displayWindow", "box2i", struct.pack("<iiii", 0, 0, w - 1, h - 1)) +
              attr("lineOrder", "lineOrder", b"\0") + attr("pixelAspectRatio", "float", struct.pack("<f", 1)) +
              attr("screenWindowCenter", "v2f", struct.pack("<ff", 0, 0)) +
              attr("screenWindowWidth", "float", struct.pack("<f", 1)) + b"\0")
    chunks = []
    for y0 in range(0, h, per):
        raw = b"".join(img[y, :, c].astype("<f4").tobytes() for y in range(y0, min(h, y0 + per)) for c in (2, 1, 0))
        b = np.frombuffer(raw, dtype=np.uint8)
        split = np.concatenate([b[0::2], b[1::2]]).astype(np.int32)
        pred = split.copy()
        pred[1:] = (split[1:] - split[:-1] + 128 + 256) % 256
        chunks.append((y0, zlib.compress(pred.astype(np.uint8).tobytes())))
    prefix = struct.pack("<ii", 20000630, 2) + header
    pos = len(prefix) + 8 * len(chunks)
    offs, body = [], b""
    for y0, data in chunks:
        offs.append(pos + len(body))
        body += struct.pack("<ii", y0, len(data)) + data
    path.write_bytes(prefix + struct.pack(f"<{len(offs)}Q", *offs) + body)


@pytest.mark.parametrize("compression", [ZIPS_COMPRESSION, ZIP_COMPRESSION])
def test_exr_reader_inflates_zip(tmp_path, compression):
    img = np.zeros((20, 9, 3), dtype=np.float32)
    img[..., 0] = np.arange(9)[None, :] * 1.5
    img[..., 1] = np.arange(20)[:, None] * 0.25
    img[..., 2] = 3.0
    _zip_exr(tmp_path / "z.exr", img, compression)
    ch = read_exr(tmp_path / "z.exr")
    np.testing.assert_array_equal(np.stack([ch["R"], ch["G"], ch["B"]], axis=-1), img)


def test_png_round_trip(tmp_path):
    img = np.random.default_rng(2).integers(0, 256, (5, 8, 3), dtype=np.uint8)
    write_png_rgb8(tmp_path / "a.png", img)
    assert (tmp_path / "a.png").read_bytes()[:8] == b"\x89PNG\r\n\x1a\n"
    np.testing.assert_array_equal(read_png_rgb8(tmp_path / "a.png"), img)


def test_white_balance_neutralises_the_solar_white():
    """spectrum.rs:408-452: the solar white maps to D65 and the matrix stays
    separate from the XYZ weights; a band-integrated value is not scaled by
    the band width (spectrum.rs:388-406)."""
    w = np.array([[0.3362, 0.038, 1.7721], [0.4334, 0.995, 0.0087]], dtype=np.float32)  # CIE at 450, 550 nm
    solar = np.array([2.0, 3.0], dtype=np.float32)
    conv = cm.SpectralRgbConverter(w, solar)
    xyz = cm.spectrum_to_xyz(w, solar[None, :])[0]
    wb = conv.white_balance["xyz_from_xyz"]
    bal = wb @ (xyz / xyz[1])
    np.testing.assert_allclose(bal, cm.D65_WHITE_XYZ_Y1, atol=1e-3)
    assert conv.white_balance["method"] == "Bradford solar-white-to-D65"
    # D65 white maps to (1, 1, 1) in linear sRGB, within the matrices' rounding
    np.testing.assert_allclose(cm.LINEAR_SRGB_FROM_XYZ_D65 @ cm.D65_WHITE_XYZ_Y1, [1, 1, 1], atol=2e-3)


def test_tonemap_and_srgb8():
    assert cm.to_srgb8(np.array([0.0, 1.0, 2.0], np.float32)).tolist() == [0, 255, 255]
    assert cm.to_srgb8(np.array([0.0031308], np.float32))[0] == int(0.0031308 * 12.92 * 255 + 0.5)
    np.testing.assert_allclose(cm.tonemap(np.array([-1.0, 20.0]), 0.05), [0.0, 1 - np.exp(-1.0)], rtol=1e-6)
    rgb = np.array([[np.nan, 1.0, 1.0], [0.5, 0.5, 0.5]], np.float32)
    conv = cm.SpectralRgbConverter(np.eye(3, dtype=np.float32), np.ones(3, np.float32))
    out = conv.to_linear_srgb(np.array([[np.inf, 0, 0], [1, 1, 1]], np.float32))
    assert np.all(out[0] == 0) and np.all(np.isfinite(out[1]))


def test_band_exr_names_follow_the_reference():
    from sky_cuda.reference_render import band_exr_name
    assert band_exr_name(380.0) == "bands/sky_380nm.exr"
    assert band_exr_name(42.0) == "bands/sky_042nm.exr"
    assert band_exr_name(552.5) == "bands/sky_552nm.exr"  # ties to even, as Rust's {:03.0}


def test_rebuild_rgb_only_from_band_exrs(tmp_path, data_dir):
    """--rebuild-rgb-only (main.rs:85-104): band EXRs -> film -> RGB EXR/PNG,
    colorimetry block refreshed; runs on the host."""
    from sky_cuda.reference_render import (asset_manifest, converter_for, main, parse_args, read_film_from_band_exrs,
                                           write_band_exrs)
    from sky_cuda.render import Film
    from sky_cuda.scene import load_bands
    centers = [float(c) for c in load_bands(data_dir / "bands.csv")["center_nm"]]
    rng = np.random.default_rng(5)
    w, h = 6, 4
    film = Film(w, h, len(centers), rng.uniform(0, 30, w * h * len(centers)).astype(np.float32))
    write_band_exrs(film, tmp_path, centers)
    back = read_film_from_band_exrs(tmp_path, centers)
    np.testing.assert_array_equal(back.values, film.values)
    args = parse_args(["--out", str(tmp_path), "--data-dir", str(data_dir), "--width", str(w), "--height", str(h)])
    from sky_cuda.render import RenderConfig
    conv = converter_for(data_dir, centers)
    manifest = asset_manifest(RenderConfig(width=w, height=h, spp=4), args, centers, conv)
    manifest["colorimetry"] = None
    (tmp_path / "asset.json").write_text(json.dumps(manifest))
    assert main(["--out", str(tmp_path), "--data-dir", str(data_dir), "--rebuild-rgb-only"]) == 0
    from sky_cuda.exr import read_exr, read_png_rgb8
    ch = read_exr(tmp_path / "sky_rgb.exr")
    rgb = np.stack([ch["R"], ch["G"], ch["B"]], axis=-1).reshape(-1, 3)
    np.testing.assert_allclose(rgb, conv.to_linear_srgb(film.values.reshape(-1, len(centers))), rtol=1e-6)
    png = read_png_rgb8(tmp_path / "sky_rgb.png")
    assert png.shape == (h, w, 3)
    m = json.loads((tmp_path / "asset.json").read_text())
    assert m["kind"] == "spectral_panorama_v0" and m["version"] == 0 and m["dimensions"] == [w, h]
    assert m["colorimetry"]["white_balance"]["method"] == "Bradford solar-white-to-D65"
    assert m["files"]["band_exrs"][0] == "bands/sky_380nm.exr" and len(m["band_centers_nm"]) == len(centers)
