"""Independent numerical answers used to pin the oracle and the GPU tracer.

  * sky-view LUT camera directions, restated in float64 from
    sky_trace.wgsl:625-681 (no jitter, so each pixel is one direction);
  * single-scattering radiance along a view ray: the exact integral of the
    piecewise-linear medium with numerically integrated view and sun
    transmittances (what the tracer estimates when paths are cut after one
    scattering order);
  * the vacuum ground radiance  albedo/pi * L_sun * Omega * (n.s)(1+cos_max)/2.
"""

from __future__ import annotations

import math

import numpy as np


def lut_direction(width, height, x, y, observer_alt, ground_radius, sun):
    def unit(u, res):
        return 0.5 if res <= 1 else (u - 0.5 / res) * (res / (res - 1.0))

    u = (x + 0.5) / width
    v = (y + 0.5) / height
    ux = min(max(unit(u, width), 0.0), 1.0)
    uy = min(max(unit(v, height), 0.0), 1.0)
    vh = ground_radius + max(observer_alt, 0.0)
    v_h = math.sqrt(max(vh * vh - ground_radius ** 2, 0.0))
    beta = math.acos(min(max(v_h / vh, 0.0), 1.0))
    zha = math.pi - beta
    if uy < 0.75:
        c = 1.0 - (1.0 - uy / 0.75) ** 2
        vzc = math.cos(zha * c)
    else:
        c = ((uy - 0.75) / 0.25) ** 2
        vzc = math.cos(zha + beta * c)
    lvc = -((ux * ux) * 2.0 - 1.0)
    s = np.asarray(sun, dtype=np.float64)
    sh = np.array([s[0], 0.0, s[2]])
    fwd = sh / np.linalg.norm(sh) if np.linalg.norm(sh) > 1e-5 else np.array([1.0, 0.0, 0.0])
    side = np.array([fwd[2], 0.0, -fwd[0]])
    side /= np.linalg.norm(side)
    sin_view = math.sqrt(max(1.0 - vzc * vzc, 0.0))
    ss = math.sqrt(max(1.0 - lvc * lvc, 0.0))
    d = np.array([0.0, vzc, 0.0]) + sin_view * (fwd * lvc + side * ss)
    return d / np.linalg.norm(d)


def knot_tables(scene):
    """Union-knot piecewise-linear coefficient tables, float64:
    z [K], rayleigh [B,K], mie_sca [B,4,K], extinction [B,K]."""
    top = scene.top_altitude_km
    atm, aer = scene.atmosphere, scene.aerosol
    z = np.unique(np.concatenate([[0.0, top], atm["altitude_km"][(atm["altitude_km"] > 0) & (atm["altitude_km"] < top)],
                                  aer["altitude_km"][(aer["altitude_km"] > 0) & (aer["altitude_km"] < top)]]))
    za = atm["altitude_km"].astype(np.float64)
    air = np.interp(z, za, atm["air_cm3"].astype(np.float64))
    oz = np.interp(z, za, atm["ozone_cm3"].astype(np.float64))
    zr = aer["altitude_km"].astype(np.float64)
    mass = np.stack([np.interp(z, zr, aer["mass_g_m3"][:, i].astype(np.float64)) for i in range(4)])
    b = scene.bands
    ray = air[None, :] * b["rayleigh_cross_section_m2"].astype(np.float64)[:, None] * 1e9
    ozone = oz[None, :] * b["ozone_cross_section_cm2"].astype(np.float64)[:, None] * 1e5
    opt = scene.aerosol_optics.reshape(scene.band_count, 4)
    sca = mass[None, :, :] * opt["scattering_km_inv_per_g_m3"].astype(np.float64)[:, :, None]
    ab = mass[None, :, :] * opt["absorption_km_inv_per_g_m3"].astype(np.float64)[:, :, None]
    ext = ray + ozone + sca.sum(1) + ab.sum(1)
    return z, ray, sca, ext


def _interp_alt(z, vals, alt, top):
    out = np.interp(alt, z, vals)
    return np.where((alt >= 0.0) & (alt <= top), out, 0.0)


def _sphere_exit(o, d, radius):
    b = np.sum(o * d, axis=-1)
    c = np.sum(o * o, axis=-1) - radius * radius
    disc = b * b - c
    return -b + np.sqrt(np.maximum(disc, 0.0)), disc


def single_scatter(scene, band, direction, mie_phase_fn, observer_alt=0.2, n_view=6000, n_sun=1200,
                   cos_max=None):
    """Single-scattering radiance (one order, NEE to the sun) along a sky ray."""
    rg, rt, top = scene.ground_radius_km, scene.atmosphere_radius_km, scene.top_altitude_km
    z, ray, sca, ext = knot_tables(scene)
    s = np.asarray(scene.sun_direction, dtype=np.float64)
    s /= np.linalg.norm(s)
    d = np.asarray(direction, dtype=np.float64)
    o = np.array([0.0, rg + observer_alt, 0.0])
    t_exit, _ = _sphere_exit(o, d, rt)
    t = np.linspace(0.0, float(t_exit), n_view)
    p = o[None, :] + t[:, None] * d[None, :]
    alt = np.linalg.norm(p, axis=1) - rg
    sig_t = _interp_alt(z, ext[band], alt, top)
    tau_view = np.concatenate([[0.0], np.cumsum(0.5 * (sig_t[1:] + sig_t[:-1]) * np.diff(t))])
    # sun transmittance from every point
    ts_exit, _ = _sphere_exit(p, np.broadcast_to(s, p.shape), rt)
    bs = p @ s
    cg = np.sum(p * p, axis=1) - rg * rg
    disc_g = bs * bs - cg
    blocked = (disc_g > 0) & ((-bs - np.sqrt(np.maximum(disc_g, 0))) > 0)
    u = np.linspace(0.0, 1.0, n_sun)
    tau_sun = np.zeros(len(t))
    for i0 in range(0, len(t), 500):
        sl = slice(i0, min(len(t), i0 + 500))
        du = ts_exit[sl, None] * u[None, :]
        q = p[sl, None, :] + du[..., None] * s[None, None, :]
        a = np.linalg.norm(q, axis=2) - rg
        st = _interp_alt(z, ext[band], a, top)
        tau_sun[sl] = np.trapezoid(st, du, axis=1)
    t_sun = np.where(blocked, 0.0, np.exp(-tau_sun))
    mu = float(d @ s)
    p_r = 3.0 / (16.0 * math.pi) * (1.0 + mu * mu)
    scat_phase = _interp_alt(z, ray[band], alt, top) * p_r
    for i in range(4):
        si = _interp_alt(z, sca[band, i], alt, top)
        if np.any(si > 0):
            scat_phase = scat_phase + si * float(mie_phase_fn(i, band, mu))
    integrand = scat_phase * np.exp(-tau_view) * t_sun
    l_sun = float(scene.bands["solar_radiance_w_m2_sr"][band])
    if cos_max is None:
        cos_max = float(np.float32(math.cos(float(np.float32(scene.sun_angular_radius_rad)))))
    omega = float(np.float32(2.0 * math.pi) * (np.float32(1.0) - np.float32(cos_max)))
    return float(np.trapezoid(integrand, t)) * l_sun * omega


def vacuum_ground(scene, band, direction, observer_alt=0.2):
    """Radiance of a ground-hitting ray in vacuum: one NEE to the sun cone."""
    rg = scene.ground_radius_km
    o = np.array([0.0, rg + observer_alt, 0.0])
    d = np.asarray(direction, dtype=np.float64)
    b = o @ d
    c = o @ o - rg * rg
    t = -b - math.sqrt(b * b - c)
    n = o + t * d
    n /= np.linalg.norm(n)
    s = np.asarray(scene.sun_direction, dtype=np.float64)
    s /= np.linalg.norm(s)
    cos_max = float(np.float32(math.cos(float(np.float32(scene.sun_angular_radius_rad)))))
    omega = float(np.float32(2.0 * math.pi) * (np.float32(1.0) - np.float32(cos_max)))
    l_sun = float(scene.bands["solar_radiance_w_m2_sr"][band])
    return scene.ground_albedo / math.pi * l_sun * omega * float(n @ s) * (1.0 + cos_max) / 2.0
