"""Mie phase-table bake on the GPU (sky_cuda_bake_mie_phase) against the CPU
oracle's restatement of the published Mie series."""

import sys
import time
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "oracle"))

import mie_oracle as mo  # noqa: E402

pytestmark = pytest.mark.gpu


def test_single_sphere_known_answer(gpu):
    from sky_cuda.mie import MieDistribution, bake_phase
    # one radius: Bohren & Huffman's example sphere
    d = MieDistribution(0.525, 1.5, 0.525, 0.525, radii=1)
    phase, optics = bake_phase(d, [632.8], [1.55 + 0.0j], bins=512)
    area = np.pi * 0.525**2
    assert optics["sigma_sca_um2"][0] / area == pytest.approx(3.10543, abs=1e-5)
    assert optics["sigma_ext_um2"][0] / area == pytest.approx(3.10543, abs=1e-5)
    x = 2.0 * np.pi * 0.525 / 0.6328
    want = mo.unpolarized_phase(1.55 + 0.0j, x, mo.cube_root_mu_grid(512))
    np.testing.assert_allclose(phase[0], want, rtol=2e-5)
    assert optics["g"][0] == pytest.approx(mo.efficiencies(1.55 + 0.0j, x)[3], rel=1e-9)


@pytest.mark.parametrize("m", [1.53 + 0.008j, 1.75 + 0.44j, 1.33 + 0.0j])
def test_size_average_matches_oracle(gpu, m):
    from sky_cuda.mie import MieDistribution, bake_phase
    d = MieDistribution(0.0983, 2.03, 0.0073, 30.2, radii=40)
    lam_nm = np.array([380.0, 550.0, 780.0])
    phase, optics = bake_phase(d, lam_nm, [m] * 3, bins=256)
    mu = mo.cube_root_mu_grid(256)
    r, w = mo.lognormal_radii(d.r_mode_um, d.sigma_g, d.r_min_um, d.r_max_um, d.radii)
    for b, lam in enumerate(lam_nm):
        want, (sca, ext, g) = mo.size_dist_phase(m, lam * 1e-3, r, w, mu)
        # FP32 angular sums: the phase to 1e-4, the FP64 series to 1e-9
        np.testing.assert_allclose(phase[b], want, rtol=1e-4)
        assert optics["sigma_sca_um2"][b] == pytest.approx(sca, rel=1e-9)
        assert optics["sigma_ext_um2"][b] == pytest.approx(ext, rel=1e-9)
        assert optics["g"][b] == pytest.approx(g, rel=1e-9)


def test_reference_sized_bake_is_normalised_and_timed(gpu):
    from sky_cuda.mie import OPAC_SPECIES, bake_phase, cube_root_mu_grid
    lam_nm = np.linspace(380.0, 780.0, 41)
    u = (np.arange(1024) + 0.5) / 1024
    t0 = time.perf_counter()
    out = {name: bake_phase(d, lam_nm, [1.53 + 0.008j] * 41) for name, d in OPAC_SPECIES.items()}
    dt = time.perf_counter() - t0
    print(f"Mie bake, 4 species x 41 bands x 300 radii x 1024 bins: {dt:.2f} s")
    for name, (phase, optics) in out.items():
        assert np.all(np.isfinite(phase)) and np.all(phase > 0)
        norm = 2.0 * np.pi * np.sum(phase * 6.0 * u**2 / 1024, axis=1)
        np.testing.assert_allclose(norm, 1.0, atol=5e-3)
        assert np.all((optics["g"] > 0.0) & (optics["g"] < 1.0))
    assert cube_root_mu_grid(4)[0] > 0.99


def test_invalid_distribution_is_rejected(gpu):
    from sky_cuda._abi import SkyCudaError
    from sky_cuda.mie import MieDistribution, bake_phase
    with pytest.raises(SkyCudaError, match="size distribution"):
        bake_phase(MieDistribution(0.1, 1.0, 0.01, 1.0), [550.0], [1.5 + 0j])
    with pytest.raises(SkyCudaError, match="refractive index"):
        bake_phase(MieDistribution(0.1, 2.0, 0.01, 1.0), [550.0], [1.5 - 0.1j])
