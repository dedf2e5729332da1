"""Mie phase-table bake (scripts/bake_opac_data.py:99-121, :192-204) on the GPU.

The reference bakes data/mie_phase.csv from OPAC refractive indices and
lognormal size distributions with miepython; that file, the OPAC data and
miepython are all absent here.  `bake_phase` runs the same computation for
caller-supplied refractive indices through sky_cuda_bake_mie_phase (the
sphere's Mie series in FP64, the angular sums in FP32), and
`write_mie_phase_csv` writes the reference's file format, which
`load_scene_data` reads back.
"""

from __future__ import annotations

import ctypes
from dataclasses import dataclass
from pathlib import Path

import numpy as np

from ._abi import SkyMieBand, SkyMieDistribution, check, load_library

PHASE_BINS = 1024
RADII = 300


@dataclass(frozen=True)
class MieDistribution:
    """Lognormal size distribution: mode radius, geometric standard deviation
    and the radius range sampled by `radii` geometric points."""

    r_mode_um: float
    sigma_g: float
    r_min_um: float
    r_max_um: float
    radii: int = RADII

    def to_c(self) -> SkyMieDistribution:
        return SkyMieDistribution(self.r_mode_um, self.sigma_g, self.r_min_um, self.r_max_um, self.radii, 0)


# The OPAC species of the reference bake (name: mode radius um, sigma_g, radius range um),
# bake_opac_data.py:20-53, in the species order of the scene tables.
OPAC_SPECIES = {
    "inso": MieDistribution(0.471, 2.51, 0.005, 20.0),
    "waso": MieDistribution(0.0262, 2.24, 0.006, 25.0),
    "soot": MieDistribution(0.0118, 2.0, 0.005, 20.0),
    "suso": MieDistribution(0.0983, 2.03, 0.0073, 30.2),
}


def cube_root_mu_grid(bins: int = PHASE_BINS) -> np.ndarray:
    u = (np.arange(bins, dtype=np.float64) + 0.5) / bins
    return 1.0 - 2.0 * u**3


def bake_phase(dist: MieDistribution, wavelength_nm, refractive_index, bins: int = PHASE_BINS):
    """Size-averaged phase function [bands, bins] (normalised to 1 over the
    sphere) and per-band optics {"sigma_sca_um2", "sigma_ext_um2", "g"}.

    refractive_index: complex per band, n + i k with k >= 0 for absorption."""
    lam = np.ascontiguousarray(np.asarray(wavelength_nm, dtype=np.float64) * 1e-3)
    m = np.asarray(refractive_index, dtype=np.complex128).reshape(-1)
    if m.size == 1:
        m = np.full(lam.shape, m[0])
    if m.shape != lam.shape:
        raise ValueError("one refractive index per wavelength")
    re = np.ascontiguousarray(m.real)
    im = np.ascontiguousarray(m.imag)
    n_bands = lam.size
    phase = np.zeros((n_bands, bins), dtype=np.float64)
    bands = (SkyMieBand * n_bands)()
    lib = load_library()
    dp = ctypes.POINTER(ctypes.c_double)
    d = dist.to_c()
    check(lib.sky_cuda_bake_mie_phase(ctypes.byref(d), lam.ctypes.data_as(dp), re.ctypes.data_as(dp),
                                      im.ctypes.data_as(dp), n_bands, bins, phase.ctypes.data_as(dp), bands), lib)
    optics = {k: np.array([getattr(b, k) for b in bands]) for k in ("sigma_sca_um2", "sigma_ext_um2", "g")}
    return phase, optics


def write_mie_phase_csv(path, tables: dict) -> None:
    """data/mie_phase.csv rows `species, band, bin, value` (bake_opac_data.py:196-204);
    `tables` maps species name -> [bands, bins] phase values."""
    lines = []
    for name, values in tables.items():
        values = np.asarray(values)
        for b in range(values.shape[0]):
            for k in range(values.shape[1]):
                lines.append(f"{name},{b},{k},{float(values[b, k]):.8e}")
    p = Path(path)
    p.parent.mkdir(parents=True, exist_ok=True)
    p.write_text("\n".join(lines) + "\n")
