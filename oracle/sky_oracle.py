"""ctypes binding of the CPU oracle (oracle/sky_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline legs, never by the sky_cuda package.  See the header
of sky_oracle.cpp for what the oracle restates and how it is pinned.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libsky_oracle.so"

_lib = None


def build() -> Path:
    """Compile the oracle with its Makefile (g++, -ffp-contract=off)."""
    res = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    return LIB


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not LIB.exists() or LIB.stat().st_mtime < (HERE / "sky_oracle.cpp").stat().st_mtime:
        build()
    lib = ctypes.CDLL(str(LIB))
    vp, fp, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_double)
    u32p, u64p = ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint64)
    lib.oracle_render.argtypes = [vp, vp, ctypes.c_uint32, ctypes.c_uint32, dp, dp, u64p, u32p, ctypes.c_int]
    lib.oracle_render.restype = ctypes.c_int
    lib.oracle_pcg4d.argtypes = [u32p, u32p]
    lib.oracle_rng_stream.argtypes = [ctypes.c_uint32] * 3 + [ctypes.c_uint64, ctypes.c_uint32, u32p, fp]
    lib.oracle_next_boundary.argtypes = [ctypes.c_float, ctypes.c_float, fp, fp, fp, u32p]
    lib.oracle_next_boundary.restype = ctypes.c_int
    lib.oracle_coefficients.argtypes = [vp, ctypes.c_float, ctypes.c_uint32, fp]
    lib.oracle_mie_phase.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32, fp, ctypes.c_uint32, fp]
    lib.oracle_sample_mu_pdf.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32, fp, ctypes.c_uint32, fp, fp]
    lib.oracle_sampling_pdf.argtypes = [vp, ctypes.c_uint32, ctypes.c_uint32, fp, ctypes.c_uint32, fp]
    lib.oracle_invert_rayleigh_cdf.argtypes = [ctypes.c_float]
    lib.oracle_invert_rayleigh_cdf.restype = ctypes.c_float
    lib.oracle_bake_majorant_grid.argtypes = [vp, ctypes.c_uint32, fp, fp]
    lib.oracle_cpu_extinction.argtypes = [vp, ctypes.c_float, ctypes.c_uint32]
    lib.oracle_cpu_extinction.restype = ctypes.c_float
    lib.oracle_merge_groups.argtypes = [fp, ctypes.c_uint32, ctypes.c_float, u32p]
    lib.oracle_merge_groups.restype = ctypes.c_uint32
    lib.oracle_transmittance.argtypes = [vp, ctypes.c_uint32, fp, fp, ctypes.c_uint32, ctypes.c_uint32]
    lib.oracle_transmittance.restype = ctypes.c_double
    _lib = lib
    return lib


def _f(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def render(scene, config, row_begin: int = 0, row_step: int = 1, threads: int = 0):
    """Per-cell FP64 (sum, sumsq) [pixels, bands], event counters and the
    watchdog flag for the rows row_begin, row_begin + row_step, ..."""
    lib = load()
    desc = scene.desc()
    cfg = config.to_c()
    cells = config.width * config.height * scene.band_count
    s = np.zeros(cells, dtype=np.float64)
    sq = np.zeros(cells, dtype=np.float64)
    counters = np.zeros(8, dtype=np.uint64)
    wd = ctypes.c_uint32(0)
    if threads <= 0:
        threads = os.cpu_count() or 1
    st = lib.oracle_render(ctypes.byref(desc), ctypes.byref(cfg), row_begin, row_step,
                           s.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                           sq.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                           counters.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), ctypes.byref(wd), threads)
    if st != 0:
        raise ValueError(f"oracle_render rejected the scene/config (status {st})")
    shape = (config.width * config.height, scene.band_count)
    return s.reshape(shape), sq.reshape(shape), counters, int(wd.value)


def pcg4d(v):
    lib = load()
    a = (ctypes.c_uint32 * 4)(*[int(x) & 0xFFFFFFFF for x in v])
    o = (ctypes.c_uint32 * 4)()
    lib.oracle_pcg4d(a, o)
    return tuple(o)


def rng_stream(pixel: int, sample: int, band: int, seed: int, n: int):
    lib = load()
    u = np.zeros(n, dtype=np.uint32)
    f = np.zeros(n, dtype=np.float32)
    lib.oracle_rng_stream(pixel, sample, band, seed, n, u.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), _f(f))
    return u, f


def next_boundary(ground_radius, atmosphere_radius, origin, direction):
    lib = load()
    o = np.asarray(origin, dtype=np.float32)
    d = np.asarray(direction, dtype=np.float32)
    t = ctypes.c_float()
    k = ctypes.c_uint32()
    hit = lib.oracle_next_boundary(ground_radius, atmosphere_radius, _f(o), _f(d), ctypes.byref(t), ctypes.byref(k))
    return bool(hit), float(t.value), int(k.value)


def coefficients(scene, altitude_km: float, band: int) -> np.ndarray:
    """[rayleigh, sca0..3, abs0..3, ozone, scattering_total, extinction_total]."""
    lib = load()
    out = np.zeros(12, dtype=np.float32)
    desc = scene.desc()
    lib.oracle_coefficients(ctypes.byref(desc), altitude_km, band, _f(out))
    return out


def mie_phase(scene, species: int, band: int, mu) -> np.ndarray:
    lib = load()
    mu = np.ascontiguousarray(mu, dtype=np.float32)
    out = np.zeros_like(mu)
    desc = scene.desc()
    lib.oracle_mie_phase(ctypes.byref(desc), species, band, _f(mu), mu.size, _f(out))
    return out


def sample_mu_pdf(scene, species: int, band: int, xi):
    lib = load()
    xi = np.ascontiguousarray(xi, dtype=np.float32)
    mu = np.zeros_like(xi)
    pdf = np.zeros_like(xi)
    desc = scene.desc()
    lib.oracle_sample_mu_pdf(ctypes.byref(desc), species, band, _f(xi), xi.size, _f(mu), _f(pdf))
    return mu, pdf


def sampling_pdf(scene, species: int, band: int, mu) -> np.ndarray:
    lib = load()
    mu = np.ascontiguousarray(mu, dtype=np.float32)
    out = np.zeros_like(mu)
    desc = scene.desc()
    lib.oracle_sampling_pdf(ctypes.byref(desc), species, band, _f(mu), mu.size, _f(out))
    return out


def invert_rayleigh_cdf(xi: float) -> float:
    return float(load().oracle_invert_rayleigh_cdf(xi))


def bake_majorant_grid(scene, layers: int):
    lib = load()
    maj = np.zeros(scene.band_count * layers, dtype=np.float32)
    mino = np.zeros_like(maj)
    desc = scene.desc()
    lib.oracle_bake_majorant_grid(ctypes.byref(desc), layers, _f(maj), _f(mino))
    return maj.reshape(scene.band_count, layers), mino.reshape(scene.band_count, layers)


def transmittance(scene, tracking: int, origin, direction, band: int, n: int) -> float:
    """Mean of the binary transmittance estimator along one ray to its boundary."""
    desc = scene.desc()
    o = np.ascontiguousarray(origin, dtype=np.float32)
    d = np.ascontiguousarray(direction, dtype=np.float32)
    return float(load().oracle_transmittance(ctypes.byref(desc), tracking, _f(o), _f(d), band, n))


def merge_groups(majorants, layer_dz: float) -> list[int]:
    """First uniform layer of each merged group of tracking mode 2."""
    maj = np.ascontiguousarray(majorants, dtype=np.float32)
    starts = np.zeros(len(maj), dtype=np.uint32)
    n = load().oracle_merge_groups(_f(maj), len(maj), layer_dz, starts.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
    return [int(v) for v in starts[:n]]


def cpu_extinction(scene, altitude_km: float, band: int) -> float:
    desc = scene.desc()
    return float(load().oracle_cpu_extinction(ctypes.byref(desc), altitude_km, band))
