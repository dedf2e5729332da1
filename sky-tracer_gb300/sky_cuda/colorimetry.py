"""Spectral film -> XYZ -> white-balanced linear sRGB -> 8-bit, restated from
sky-core and sky-reference-render for the host side of the output stage.

* band XYZ weights: CIE 1931 at the band centre, no width factor
  (band_xyz_weights / spectrum_to_xyz_with_weights, spectrum.rs:226-241);
* white balance: Bradford adaptation of the solar spectrum's white to D65
  (WhiteBalanceMatrix::bradford, SpectralRgbConverter::new_solar_d65,
  spectrum.rs:84-109, :132-147);
* XYZ -> linear sRGB (D65), black when any component is not finite
  (linear_srgb_from_xyz, spectrum.rs:221-224; Rgb::finite_or_black,
  math.rs:137-143);
* PNG tone map 1 - exp(-exposure * rgb) and the sRGB transfer curve
  (film_output.rs:158-175).

The matrices are the standard published ones.  Arithmetic is float32 in the
reference's operation order; the GPU epilogue applies the same matrices to
its FP64 XYZ (SkyDeviceOutputs.rgb).
"""

from __future__ import annotations

import numpy as np

f32 = np.float32

CIE_1931_2DEG_CMF_NAME = "CIE 1931 2 degree standard observer"
CIE_1931_2DEG_CMF_SOURCE = "data/CIE_xyz_1931_2deg.csv"
LINEAR_SRGB_D65_NAME = "linear sRGB D65"
BRADFORD_WHITE_BALANCE_NAME = "Bradford solar-white-to-D65"

D65_WHITE_XYZ_Y1 = np.array([0.9504559, 1.0, 1.0890578], dtype=f32)
LINEAR_SRGB_FROM_XYZ_D65 = np.array([[3.2404542, -1.5371385, -0.4985314],
                                     [-0.969266, 1.8760108, 0.041556],
                                     [0.0556434, -0.2040259, 1.0572252]], dtype=f32)
BRADFORD_LMS_FROM_XYZ = np.array([[0.8951, 0.2664, -0.1614],
                                  [-0.7502, 1.7135, 0.0367],
                                  [0.0389, -0.0685, 1.0296]], dtype=f32)
XYZ_FROM_BRADFORD_LMS = np.array([[0.9869929, -0.1470543, 0.1599627],
                                  [0.4323053, 0.5183603, 0.0492912],
                                  [-0.0085287, 0.0400428, 0.9684867]], dtype=f32)
F32_EPSILON = f32(1.1920929e-7)


def _mat3_vec(m, v):
    """Row sums left to right in float32 (mat3_mul_vec3)."""
    m = np.asarray(m, dtype=f32)
    v = np.asarray(v, dtype=f32)
    return np.array([f32(f32(m[r, 0] * v[0]) + f32(m[r, 1] * v[1])) + f32(m[r, 2] * v[2]) for r in range(3)],
                    dtype=f32)


def _mat3_mul(a, b):
    a = np.asarray(a, dtype=f32)
    b = np.asarray(b, dtype=f32)
    out = np.zeros((3, 3), dtype=f32)
    for r in range(3):
        for c in range(3):
            out[r, c] = f32(f32(a[r, 0] * b[0, c]) + f32(a[r, 1] * b[1, c])) + f32(a[r, 2] * b[2, c])
    return out


def normalized_to_y1(xyz) -> np.ndarray:
    x, y, z = (f32(v) for v in xyz)
    if abs(y) <= F32_EPSILON:
        return D65_WHITE_XYZ_Y1.copy()
    inv = f32(f32(1.0) / y)
    return np.array([x * inv, 1.0, z * inv], dtype=f32)


def spectrum_to_xyz(weights: np.ndarray, values: np.ndarray) -> np.ndarray:
    """XYZ of spectra [..., B] with band weights [B, 3], float32 accumulated
    band by band (spectrum_to_xyz_with_weights)."""
    w = np.asarray(weights, dtype=f32)
    v = np.asarray(values, dtype=f32)
    acc = np.zeros(v.shape[:-1] + (3,), dtype=f32)
    with np.errstate(invalid="ignore", over="ignore"):  # non-finite spectra give non-finite XYZ
        for b in range(w.shape[0]):
            acc = (acc + v[..., b:b + 1] * w[b]).astype(f32)
    return acc


def bradford(source_white_xyz, target_white_xyz) -> dict:
    """WhiteBalanceMatrix::bradford as a dict (method, whites, xyz_from_xyz)."""
    source = normalized_to_y1(source_white_xyz)
    target = normalized_to_y1(target_white_xyz)
    s_lms = _mat3_vec(BRADFORD_LMS_FROM_XYZ, source)
    t_lms = _mat3_vec(BRADFORD_LMS_FROM_XYZ, target)
    scale = np.diag([f32(t / s) if abs(s) > 1.0e-12 else f32(1.0) for t, s in zip(t_lms, s_lms)]).astype(f32)
    m = _mat3_mul(XYZ_FROM_BRADFORD_LMS, _mat3_mul(scale, BRADFORD_LMS_FROM_XYZ))
    return {"method": BRADFORD_WHITE_BALANCE_NAME, "source_white_xyz_y1": source, "target_white_xyz_y1": target,
            "xyz_from_xyz": m}


class SpectralRgbConverter:
    """SpectralRgbConverter::new_solar_d65 (spectrum.rs:132-165)."""

    def __init__(self, band_xyz_weights, solar_values):
        self.weights = np.asarray(band_xyz_weights, dtype=f32)
        white = spectrum_to_xyz(self.weights, np.asarray(solar_values, dtype=f32)[None, :])[0]
        self.white_balance = bradford(white, D65_WHITE_XYZ_Y1)

    @classmethod
    def for_scene(cls, scene) -> "SpectralRgbConverter":
        """Solar white from the scene's band solar radiances (irradiance per
        solid angle: the same chromaticity as the irradiance)."""
        return cls(scene.band_xyz, scene.bands["solar_radiance_w_m2_sr"])

    def rgb_from_xyz(self) -> np.ndarray:
        """The one matrix sRGB * white balance (what the GPU epilogue applies)."""
        return _mat3_mul(LINEAR_SRGB_FROM_XYZ_D65, self.white_balance["xyz_from_xyz"])

    def to_linear_srgb(self, film_values: np.ndarray) -> np.ndarray:
        """Linear sRGB [..., 3] of spectra [..., B]: XYZ, white balance, sRGB;
        black where any component is not finite."""
        xyz = spectrum_to_xyz(self.weights, film_values)
        wb = self.white_balance["xyz_from_xyz"]
        m = LINEAR_SRGB_FROM_XYZ_D65
        with np.errstate(invalid="ignore", over="ignore"):
            bal = np.stack([(xyz[..., 0] * wb[r, 0] + xyz[..., 1] * wb[r, 1]) + xyz[..., 2] * wb[r, 2]
                            for r in range(3)], axis=-1)
            rgb = np.stack([(bal[..., 0] * m[r, 0] + bal[..., 1] * m[r, 1]) + bal[..., 2] * m[r, 2]
                            for r in range(3)], axis=-1).astype(f32)
        bad = ~np.all(np.isfinite(rgb), axis=-1)
        rgb[bad] = 0.0
        return rgb


def tonemap(rgb: np.ndarray, exposure: float) -> np.ndarray:
    """1 - exp(-max(rgb, 0) exposure) (film_output.rs:158-163)."""
    return (f32(1.0) - np.exp(-np.maximum(np.asarray(rgb, dtype=f32), f32(0.0)) * f32(exposure))).astype(f32)


def to_srgb8(linear: np.ndarray) -> np.ndarray:
    """The sRGB transfer curve to 8 bits, (v * 255 + 0.5) truncated (film_output.rs:165-175)."""
    x = np.clip(np.asarray(linear, dtype=f32), f32(0.0), f32(1.0))
    srgb = np.where(x <= f32(0.0031308), f32(12.92) * x,
                    f32(1.055) * np.power(x, f32(1.0 / 2.4)).astype(f32) - f32(0.055)).astype(f32)
    return (np.clip(srgb, f32(0.0), f32(1.0)) * f32(255.0) + f32(0.5)).astype(np.uint8)


def colorimetry_manifest(converter: SpectralRgbConverter) -> dict:
    """The asset manifest's colorimetry block (main.rs:233-248, asset.rs:24-38)."""
    wb = converter.white_balance
    return {
        "cmf": CIE_1931_2DEG_CMF_NAME,
        "cmf_source": CIE_1931_2DEG_CMF_SOURCE,
        "rgb_color_space": LINEAR_SRGB_D65_NAME,
        "white_balance": {
            "method": wb["method"],
            "source_white_xyz_y1": [float(v) for v in wb["source_white_xyz_y1"]],
            "target_white_xyz_y1": [float(v) for v in wb["target_white_xyz_y1"]],
            "xyz_from_xyz": [[float(v) for v in row] for row in wb["xyz_from_xyz"]],
        },
    }
