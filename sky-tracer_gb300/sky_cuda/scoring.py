"""The wavelength optimizer's combination score, run by the GPU kernels of
sky_cuda_score_combos (sky-wavelength-optimizer/src/main.rs:414-488,
1121-1156): Oklab distances of rebuilt XYZ against a reference, their mean,
RMS and exact order statistics, score = rmse + 0.25 p95."""

from __future__ import annotations

import ctypes

import numpy as np

from . import _abi
from ._abi import SkyComboScore, check, load_library

FIELDS = ("mean", "rmse", "p50", "p90", "p95", "p99", "max", "score", "finite")


def reference_scale(ref_y: np.ndarray) -> float:
    """p99 of the reference Y over finite samples, element round((n-1) 0.99)
    (main.rs:343, percentile_sorted :1150-1156), at least 1e-12."""
    y = np.sort(np.asarray(ref_y, dtype=np.float64)[np.isfinite(ref_y)])
    if y.size == 0:
        return 1e-12
    return max(float(y[int(np.floor((y.size - 1) * 0.99 + 0.5))]), 1e-12)


def oklab(xyz: np.ndarray) -> np.ndarray:
    """Oklab of XYZ (float64, signed cube root; main.rs:1121-1130)."""
    m1 = np.array([[0.8189330101, 0.3618667424, -0.1288597137], [0.0329845436, 0.9293118715, 0.0361456387],
                   [0.0482003018, 0.2643662691, 0.6338517070]])
    m2 = np.array([[0.2104542553, 0.7936177850, -0.0040720468], [1.9779984951, -2.4285922050, 0.4505937099],
                   [0.0259040371, 0.7827717662, -0.8086757660]])
    return np.cbrt(np.asarray(xyz, dtype=np.float64) @ m1.T) @ m2.T


def score_combos(bands, ref_xyz: np.ndarray, combo_bands, combo_xyz, scale: float | None = None,
                 stream: int | None = None) -> list[dict]:
    """Scores of combinations c: XYZ[s] = sum_ch bands[combo_bands[c][ch]][s] * combo_xyz[c][ch].

    bands: CUDA float32 tensor [B, N]; ref_xyz: [N, 3] reference XYZ (host);
    combo_bands [C, K] ints, combo_xyz [C, K, 3]."""
    import torch
    lib = load_library()
    if not (bands.is_cuda and bands.dtype == torch.float32 and bands.dim() == 2):
        raise ValueError("bands must be a [B, N] float32 CUDA tensor")
    bands = bands.contiguous()
    n = bands.shape[1]
    ref_xyz = np.asarray(ref_xyz, dtype=np.float64).reshape(n, 3)
    scale = reference_scale(ref_xyz[:, 1]) if scale is None else float(scale)
    ref_lab = torch.as_tensor(oklab(ref_xyz / scale).astype(np.float32), device=bands.device).contiguous()
    cb = np.ascontiguousarray(combo_bands, dtype=np.uint32)
    cx = np.ascontiguousarray(combo_xyz, dtype=np.float32)
    c, k = cb.shape
    if cx.shape != (c, k, 3):
        raise ValueError("combo_xyz must be [C, K, 3] for combo_bands [C, K]")
    res = (SkyComboScore * c)()
    st = torch.cuda.current_stream().cuda_stream if stream is None else stream
    check(lib.sky_cuda_score_combos(ctypes.c_void_p(bands.data_ptr()), bands.shape[0], n,
                                    ctypes.c_void_p(ref_lab.data_ptr()), scale,
                                    cb.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                    cx.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), c, k, res,
                                    ctypes.c_void_p(st)), lib)
    return [{f: (int(getattr(r, f)) if f == "finite" else float(getattr(r, f))) for f in FIELDS} for r in res]


def score_xyz(xyz, xyz_ref) -> dict:
    """Score of one reconstruction XYZ [..., 3] (CUDA tensor) against its reference."""
    import torch
    x = xyz.reshape(-1, 3).to(torch.float32).T.contiguous()
    ref = xyz_ref.reshape(-1, 3).double().cpu().numpy() if hasattr(xyz_ref, "cpu") else np.asarray(xyz_ref)
    eye = np.eye(3, dtype=np.float32)[None]
    return score_combos(x, ref, np.array([[0, 1, 2]]), eye)[0]
