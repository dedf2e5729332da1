"""CPU oracle of the Mie phase-table bake.

TEST INFRASTRUCTURE ONLY: imported by tests/, never by the sky_cuda package.

Restates, in float64 numpy:
* the Mie series of a homogeneous sphere as published by Bohren & Huffman,
  "Absorption and Scattering of Light by Small Particles" (1983), appendix A
  (BHMIE): the logarithmic derivative D_n(mx) by downward recurrence, the
  Riccati-Bessel functions by upward recurrence, a_n, b_n, Q_sca, Q_ext,
  Q_back, the asymmetry parameter and the amplitude functions S1, S2 through
  the angular functions pi_n, tau_n; series length x + 4.05 x^(1/3) + 2 + 1
  (Wiscombe, Appl. Opt. 19, 1505, 1980);
* the reference's size averaging (scripts/bake_opac_data.py:99-121):
  geometric radii with lognormal weights, and the scattering-cross-section
  weighted average of each sphere's unpolarised phase function normalised to
  1 over the sphere (miepython.i_unpolarized(..., norm="one")).

The reference calls miepython, which is not vendored and whose version the
reference does not pin; the published series above is what miepython
implements.  Pinned in tests/test_mie_host.py against Bohren & Huffman's
published example (m = 1.55, x = 5.213: Q_sca = Q_ext = 3.10543,
Q_back = 2.92534), the Rayleigh limit and energy conservation.
"""

from __future__ import annotations

import numpy as np


def mie_terms(x: float) -> int:
    return int(x + 4.05 * np.cbrt(x) + 2.0) + 1


def mie_ab(m: complex, x: float):
    """Mie coefficients a_n, b_n (n = 1..N) of a sphere, BHMIE's recurrences."""
    n_terms = mie_terms(x)
    mx = m * x
    nmx = int(max(n_terms, abs(mx))) + 16
    d = np.zeros(nmx + 1, dtype=complex)
    for n in range(nmx, 0, -1):
        t = n / mx
        d[n - 1] = t - 1.0 / (d[n] + t)
    psi0, psi1 = np.cos(x), np.sin(x)
    chi0, chi1 = -np.sin(x), np.cos(x)
    xi1 = complex(psi1, -chi1)
    a = np.zeros(n_terms, dtype=complex)
    b = np.zeros(n_terms, dtype=complex)
    for n in range(1, n_terms + 1):
        psi = (2.0 * n - 1.0) * psi1 / x - psi0
        chi = (2.0 * n - 1.0) * chi1 / x - chi0
        xi = complex(psi, -chi)
        ta = d[n] / m + n / x
        tb = m * d[n] + n / x
        a[n - 1] = (ta * psi - psi1) / (ta * xi - xi1)
        b[n - 1] = (tb * psi - psi1) / (tb * xi - xi1)
        psi0, psi1 = psi1, psi
        chi0, chi1 = chi1, chi
        xi1 = complex(psi1, -chi1)
    return a, b


def efficiencies(m: complex, x: float):
    """(Q_sca, Q_ext, Q_back, g) of a sphere."""
    a, b = mie_ab(m, x)
    n = np.arange(1, len(a) + 1, dtype=float)
    qsca = 2.0 / x**2 * np.sum((2 * n + 1) * (np.abs(a) ** 2 + np.abs(b) ** 2))
    qext = 2.0 / x**2 * np.sum((2 * n + 1) * (a.real + b.real))
    qback = np.abs(np.sum((2 * n + 1) * (-1.0) ** n * (a - b))) ** 2 / x**2
    nn = n[:-1]
    gsum = np.sum(nn * (nn + 2) / (nn + 1) * (a[:-1] * np.conj(a[1:]) + b[:-1] * np.conj(b[1:])).real)
    gsum += np.sum((2 * n + 1) / (n * (n + 1)) * (a * np.conj(b)).real)
    g = 4.0 / (x**2 * qsca) * gsum
    return qsca, qext, qback, g


def amplitudes(a, b, mu: np.ndarray):
    """S1(mu), S2(mu) from the coefficients (BHMIE's pi_n / tau_n recurrence)."""
    mu = np.asarray(mu, dtype=float)
    pi0 = np.zeros_like(mu)
    pi1 = np.ones_like(mu)
    s1 = np.zeros(mu.shape, dtype=complex)
    s2 = np.zeros(mu.shape, dtype=complex)
    for n in range(1, len(a) + 1):
        pi = pi1
        tau = n * mu * pi - (n + 1) * pi0
        fn = (2.0 * n + 1.0) / (n * (n + 1.0))
        s1 += fn * (a[n - 1] * pi + b[n - 1] * tau)
        s2 += fn * (a[n - 1] * tau + b[n - 1] * pi)
        pi1 = ((2.0 * n + 1.0) * mu * pi - (n + 1.0) * pi0) / n
        pi0 = pi
    return s1, s2


def unpolarized_phase(m: complex, x: float, mu: np.ndarray) -> np.ndarray:
    """(|S1|^2 + |S2|^2) / 2 normalised to 1 over the sphere."""
    a, b = mie_ab(m, x)
    s1, s2 = amplitudes(a, b, mu)
    qsca = efficiencies(m, x)[0]
    return (np.abs(s1) ** 2 + np.abs(s2) ** 2) / 2.0 / (np.pi * x**2 * qsca)


def cube_root_mu_grid(bins: int) -> np.ndarray:
    """bake_opac_data.py:99-101."""
    u = (np.arange(bins, dtype=np.float64) + 0.5) / bins
    return 1.0 - 2.0 * u**3


def lognormal_radii(r_mode_um: float, sigma_g: float, r_min_um: float, r_max_um: float, count: int):
    """bake_opac_data.py:103-109."""
    r = np.geomspace(r_min_um, r_max_um, count)
    ls = np.log(sigma_g)
    w = np.exp(-(np.log(r / r_mode_um)) ** 2 / (2.0 * ls**2))
    return r, w / np.sum(w)


def size_dist_phase(m: complex, lam_um: float, r_um, weights, mu):
    """bake_opac_data.py:112-121; also returns (sigma_sca, sigma_ext, g) of the average."""
    p_acc = np.zeros_like(mu)
    sca = ext = g_acc = 0.0
    for r_i, w_i in zip(r_um, weights):
        x = 2.0 * np.pi * r_i / lam_um
        qsca, qext, _qback, g = efficiencies(m, x)
        sigma_sca = np.pi * r_i**2 * qsca
        p_acc += w_i * sigma_sca * unpolarized_phase(m, x, mu)
        sca += w_i * sigma_sca
        ext += w_i * np.pi * r_i**2 * qext
        g_acc += w_i * sigma_sca * g
    return p_acc / sca, (sca, ext, g_acc / sca)
