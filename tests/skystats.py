"""Statistics shared by the parity tests.

Per-pixel CIE XYZ and its standard error are formed from per-(pixel, band)
sums and sums of squares over S samples:
    mean_b = sum_b / S,   var(mean_b) = (sumsq_b - sum_b mean_b) / (S - 1) / S
    XYZ_c  = sum_b w_bc mean_b,   var(XYZ_c) = sum_b w_bc^2 var(mean_b)
(bands are independent: each band has its own random stream).
"""

from __future__ import annotations

import numpy as np


def xyz_from_sums(cell_sum, cell_sumsq, spp: int, weights):
    s = np.asarray(cell_sum, dtype=np.float64)
    mean = s / spp
    var = np.maximum((np.asarray(cell_sumsq, dtype=np.float64) - s * mean) / max(spp - 1, 1), 0.0) / spp
    w = np.asarray(weights, dtype=np.float64)
    return mean @ w, var @ (w * w)


def zscores(xyz_a, var_a, xyz_b, var_b, floor=1e-30):
    return (xyz_a - xyz_b) / np.sqrt(np.maximum(var_a + var_b, floor))


def regular_pixels(xyz, var, factor=10.0):
    """Pixels whose relative standard error of Y is at most `factor` times the
    median: excludes the sun disc, where a rare hit of the 0.27-degree sun
    (radiance ~1e5 times the sky) dominates both the mean and the variance."""
    rel = np.sqrt(np.maximum(var[:, 1], 0)) / np.maximum(np.abs(xyz[:, 1]), 1e-30)
    return rel <= factor * np.median(rel)


def relative_bias(xyz_a, var_a, xyz_b, var_b):
    """Signed relative difference of the summed XYZ over regular pixels of
    both images, and its standard error."""
    keep = regular_pixels(xyz_a, var_a) & regular_pixels(xyz_b, var_b)
    d = (xyz_a[keep] - xyz_b[keep]).sum(axis=0)
    ref = xyz_b[keep].sum(axis=0)
    se = np.sqrt((var_a[keep] + var_b[keep]).sum(axis=0))
    return d / ref, se / np.abs(ref)


def parity_report(xyz_a, var_a, xyz_b, var_b, bright_fraction=1e-3):
    """z-scores on pixels whose Y is not below bright_fraction * p99(Y)
    (the exclusion rule of the 1 % error metric), and the mean relative
    error of XYZ over those pixels."""
    y = np.maximum(xyz_a[:, 1], xyz_b[:, 1])
    keep = y >= bright_fraction * np.percentile(y, 99)
    z = zscores(xyz_a[keep], var_a[keep], xyz_b[keep], var_b[keep])
    rel = np.abs(xyz_a[keep] - xyz_b[keep]) / np.maximum(np.abs(xyz_b[keep]), 1e-30)
    mean_rel = float(np.abs(xyz_a[keep] - xyz_b[keep]).sum() / np.abs(xyz_b[keep]).sum())
    bias, bias_se = relative_bias(xyz_a, var_a, xyz_b, var_b)
    # per pixel: mean over regular bright pixels and X, Y, Z of |a - b| / |b|,
    # and the value pure noise would give (E|N(0, s)| = 0.8 s per component)
    reg = keep & regular_pixels(xyz_a, var_a) & regular_pixels(xyz_b, var_b)
    rel_pp = np.abs(xyz_a[reg] - xyz_b[reg]) / np.maximum(np.abs(xyz_b[reg]), 1e-30)
    noise_pp = np.sqrt(2.0 / np.pi) * np.sqrt(np.maximum(var_a[reg] + var_b[reg], 0.0)) / \
        np.maximum(np.abs(xyz_b[reg]), 1e-30)
    return {
        "mean_rel_err_per_pixel": float(rel_pp.mean()) if rel_pp.size else 0.0,
        "noise_rel_err_per_pixel": float(noise_pp.mean()) if noise_pp.size else 0.0,
        "regular_pixels": int(reg.sum()),
        "bias_xyz": [float(v) for v in bias],
        "bias_se_xyz": [float(v) for v in bias_se],
        "pixels": int(keep.sum()),
        "frac_beyond_3se": float(np.mean(np.abs(z) > 3.0)),
        "max_abs_z": float(np.max(np.abs(z))) if z.size else 0.0,
        "mean_z": float(np.mean(z)) if z.size else 0.0,
        "mean_rel_err": mean_rel,
        "median_rel_err": float(np.median(rel)) if rel.size else 0.0,
    }
