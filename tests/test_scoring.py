"""The optimizer's combination score on the GPU (sky_cuda_score_combos)
against a float64 numpy restatement of evaluate_combo (main.rs:414-488)."""

import numpy as np
import pytest

from sky_cuda.scoring import oklab, reference_scale

pytestmark = pytest.mark.gpu


def _numpy_score(bands, ref_xyz, idx, coeff, scale):
    xyz = sum(bands[i].astype(np.float64)[:, None] * coeff[k].astype(np.float64)[None, :] for k, i in enumerate(idx))
    d = np.linalg.norm(oklab(xyz / scale) - oklab(ref_xyz / scale), axis=1)
    d = np.sort(d[np.isfinite(d)])
    pick = lambda q: d[int(np.floor((d.size - 1) * q + 0.5))]  # noqa: E731
    rmse = float(np.sqrt(np.mean(d * d)))
    return {"mean": float(d.mean()), "rmse": rmse, "p50": pick(0.5), "p90": pick(0.9), "p95": pick(0.95),
            "p99": pick(0.99), "max": float(d[-1]), "score": rmse + 0.25 * pick(0.95), "finite": d.size}


def test_scores_match_numpy(gpu):
    import torch
    from sky_cuda.scoring import score_combos
    rng = np.random.default_rng(9)
    B, N = 12, 50_000
    bands = rng.gamma(2.0, 1.0, (B, N)).astype(np.float32)
    true_w = rng.uniform(0.0, 1.0, (B, 3)).astype(np.float32)
    ref_xyz = bands.astype(np.float64).T @ true_w
    scale = reference_scale(ref_xyz[:, 1])
    combos = np.array([rng.choice(B, 4, replace=False) for _ in range(37)])
    coeff = rng.uniform(0.5, 3.0, (37, 4, 3)).astype(np.float32)
    bands[3, :100] = np.nan  # non-finite samples are left out, as sorted_finite does
    got = score_combos(torch.as_tensor(bands, device="cuda"), ref_xyz, combos, coeff)
    for c in range(len(combos)):
        want = _numpy_score(bands, ref_xyz, combos[c], coeff[c], scale)
        assert got[c]["finite"] == want["finite"]
        for k in ("mean", "rmse", "p50", "p90", "p95", "p99", "max", "score"):
            assert got[c][k] == pytest.approx(want[k], rel=2e-4, abs=2e-6), (c, k)


def test_identity_reconstruction_scores_zero(gpu):
    import torch
    from sky_cuda.scoring import score_xyz
    xyz = torch.rand(1000, 3, device="cuda") + 0.1
    s = score_xyz(xyz, xyz.double().cpu().numpy())
    assert s["max"] < 1e-5 and s["finite"] == 1000
