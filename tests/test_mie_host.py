"""Mie phase-table bake, host side: the oracle pinned against published and
analytic answers, and the mie_phase.csv writer against the scene loader."""

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT / "oracle"))
sys.path.insert(0, str(ROOT / "sky-tracer_gb300"))

import mie_oracle as mo  # noqa: E402


def test_bohren_huffman_published_example():
    # BHMIE's example: sphere radius 0.525 um, wavelength 0.6328 um, m = 1.55:
    # Q_sca = Q_ext = 3.10543, Q_back = 2.92534 (Bohren & Huffman 1983, appendix A)
    x = 2.0 * np.pi * 0.525 / 0.6328
    qsca, qext, qback, g = mo.efficiencies(1.55 + 0.0j, x)
    assert abs(qsca - 3.10543) < 1e-5
    assert abs(qext - 3.10543) < 1e-5
    assert abs(qback - 2.92534) < 1e-5
    assert 0.6 < g < 0.7


def test_rayleigh_limit():
    m, x = 1.5 + 0.01j, 1e-2
    qsca, qext, _, g = mo.efficiencies(m, x)
    k = (m * m - 1) / (m * m + 2)
    assert qsca == pytest.approx(8.0 / 3.0 * x**4 * abs(k) ** 2, rel=1e-3)
    assert qext == pytest.approx(4.0 * x * k.imag, rel=1e-2)  # absorption dominates
    assert abs(g) < 1e-3
    mu = mo.cube_root_mu_grid(128)
    p = mo.unpolarized_phase(m, x, mu)
    np.testing.assert_allclose(p, 3.0 / (16.0 * np.pi) * (1.0 + mu**2), rtol=1e-3)


@pytest.mark.parametrize("x", [0.3, 4.0, 40.0])
def test_energy_conservation_and_normalisation(x):
    qsca, qext, _, _ = mo.efficiencies(1.33 + 0.0j, x)
    assert qsca == pytest.approx(qext, rel=1e-10)
    # the phase integrates to 1 over the sphere (midpoint rule in u, mu = 1 - 2 u^3)
    bins = 4096
    u = (np.arange(bins) + 0.5) / bins
    p = mo.unpolarized_phase(1.33 + 0.0j, x, mo.cube_root_mu_grid(bins))
    assert 2.0 * np.pi * np.sum(p * 6.0 * u**2 / bins) == pytest.approx(1.0, abs=2e-3)


def test_size_average_is_normalised():
    mu = mo.cube_root_mu_grid(1024)
    u = (np.arange(1024) + 0.5) / 1024
    r, w = mo.lognormal_radii(0.0983, 2.03, 0.0073, 30.2, 60)
    assert w.sum() == pytest.approx(1.0)
    p, (sca, ext, g) = mo.size_dist_phase(1.43 + 1e-3j, 0.55, r, w, mu)
    assert 2.0 * np.pi * np.sum(p * 6.0 * u**2 / 1024) == pytest.approx(1.0, abs=1e-3)
    assert ext > sca > 0 and 0.0 < g < 1.0


def test_csv_writer_round_trip(tmp_path):
    from sky_cuda.mie import OPAC_SPECIES, write_mie_phase_csv
    from sky_cuda.scene import SPECIES_NAMES, load_mie_phase
    assert tuple(OPAC_SPECIES) == SPECIES_NAMES
    rng = np.random.default_rng(7)
    tables = {name: rng.uniform(0.01, 30.0, size=(3, 16)) for name in SPECIES_NAMES}
    path = tmp_path / "mie_phase.csv"
    write_mie_phase_csv(path, tables)
    back = load_mie_phase(path, 3, bins=16)
    for s, name in enumerate(SPECIES_NAMES):
        np.testing.assert_allclose(back[s], tables[name], rtol=1e-7)
