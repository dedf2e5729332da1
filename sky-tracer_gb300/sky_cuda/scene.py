"""Scene model: the sky-core inputs of the tracer, as numpy tables.

Host-side restatement of the reference's scene preparation:
  * CSV loading             crates/sky-core/src/data.rs:15-167
  * Sun from degrees        crates/sky-core/src/atmosphere.rs:19-37
  * Rayleigh cross section  crates/sky-core/src/medium.rs:104-106
  * majorant-grid bake      crates/sky-core/src/medium.rs:63-159
  * CIE 1931 weights        crates/sky-core/src/spectrum.rs:196-241
plus synthetic scenes with the shapes of the benchmark workloads (exponential
Rayleigh / Mie, tent ozone, Henyey-Greenstein phase tables), which stand in
for the reference's absent mie_phase.csv and for datasets that are not here.

All arithmetic that feeds the tracer is float32, in the reference's order.
"""

from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from ._abi import (AEROSOL_DTYPE, ATMOSPHERE_DTYPE, BAND_DTYPE, OPTICS_DTYPE, SPECIES_COUNT, SkySceneDesc)

f32 = np.float32

SPECIES_NAMES = ("inso", "waso", "soot", "suso")        # atmosphere.rs:8
PHASE_BINS = 1024                                      # atmosphere.rs:7
GROUND_ALBEDO = 0.18                                   # atmosphere.rs:9
SOLAR_ANGULAR_RADIUS_RAD = 0.00465047                  # atmosphere.rs:10
GROUND_RADIUS_KM = 6360.0                              # geometry.rs:12-17
ATMOSPHERE_RADIUS_KM = 6480.0
BAND_COUNT = 41                                        # spectrum.rs:5
MAJORANT_LAYERS = 64                                   # data.rs:48
_PI = f32(math.pi)
_TAU = f32(2.0 * math.pi)
_DEG2RAD = f32(_PI / f32(180.0))


class SceneError(ValueError):
    """Scene data that cannot be loaded (the reference's Box<dyn Error> from data.rs)."""


@dataclass
class Scene:
    """The tables of SceneData (atmosphere.rs:121-133) that the tracer reads."""

    bands: np.ndarray                  # BAND_DTYPE [B]
    atmosphere: np.ndarray             # ATMOSPHERE_DTYPE [Na], ascending
    aerosol: np.ndarray                # AEROSOL_DTYPE [Nr], ascending
    aerosol_optics: np.ndarray         # OPTICS_DTYPE [B * 4], band-major
    phase_values: np.ndarray           # f32 [4, B, bins]
    majorants: np.ndarray | None = None    # f32 [B, L]
    minorants: np.ndarray | None = None    # f32 [B, L]
    band_xyz: np.ndarray | None = None     # f32 [B, 3]
    ground_radius_km: float = GROUND_RADIUS_KM
    atmosphere_radius_km: float = ATMOSPHERE_RADIUS_KM
    top_altitude_km: float = ATMOSPHERE_RADIUS_KM - GROUND_RADIUS_KM
    sun_direction: tuple = (0.0, 0.0, 1.0)
    sun_angular_radius_rad: float = SOLAR_ANGULAR_RADIUS_RAD
    sun_solid_angle_sr: float = 0.0
    ground_albedo: float = GROUND_ALBEDO
    _keep: list = field(default_factory=list, repr=False)

    @property
    def band_count(self) -> int:
        return int(self.bands.shape[0])

    @property
    def phase_bins(self) -> int:
        return int(self.phase_values.shape[2])

    @property
    def layer_count(self) -> int:
        return int(self.majorants.shape[1])

    def with_sun(self, elevation_deg: float, azimuth_deg: float = 0.0) -> "Scene":
        """Copy with the sun moved; radiances keep the band irradiance."""
        direction, radius, solid = sun_from_degrees(elevation_deg, azimuth_deg, self.sun_angular_radius_rad)
        out = Scene(**{k: v for k, v in self.__dict__.items() if k != "_keep"})
        out.sun_direction = direction
        out.sun_angular_radius_rad = radius
        if solid != self.sun_solid_angle_sr:
            bands = self.bands.copy()
            bands["solar_radiance_w_m2_sr"] = (bands["solar_radiance_w_m2_sr"] * f32(self.sun_solid_angle_sr)
                                               / f32(solid)).astype(f32)
            out.bands = bands
        out.sun_solid_angle_sr = solid
        return out

    def desc(self) -> SkySceneDesc:
        """A SkySceneDesc viewing this scene's arrays (kept alive by the scene)."""
        if self.majorants is None:
            raise SceneError("scene has no majorant grid; call bake_majorants()")
        arrays = {
            "bands": np.ascontiguousarray(self.bands, dtype=BAND_DTYPE),
            "atmosphere": np.ascontiguousarray(self.atmosphere, dtype=ATMOSPHERE_DTYPE),
            "aerosol": np.ascontiguousarray(self.aerosol, dtype=AEROSOL_DTYPE),
            "aerosol_optics": np.ascontiguousarray(self.aerosol_optics, dtype=OPTICS_DTYPE),
            "majorants_km_inv": np.ascontiguousarray(self.majorants, dtype=f32),
            "phase_values": np.ascontiguousarray(self.phase_values, dtype=f32),
        }
        if self.band_xyz is not None:
            arrays["band_xyz_weights"] = np.ascontiguousarray(self.band_xyz, dtype=f32)
        d = SkySceneDesc()
        d.band_count = self.band_count
        d.atmosphere_len = len(self.atmosphere)
        d.aerosol_len = len(self.aerosol)
        d.majorant_layers = self.majorants.shape[1]
        d.phase_bins = self.phase_bins
        d.ground_radius_km = self.ground_radius_km
        d.atmosphere_radius_km = self.atmosphere_radius_km
        d.top_altitude_km = self.top_altitude_km
        d.sun_direction = (ctypes.c_float * 3)(*self.sun_direction)
        d.sun_angular_radius_rad = self.sun_angular_radius_rad
        d.sun_solid_angle_sr = self.sun_solid_angle_sr
        d.ground_albedo = self.ground_albedo
        for name, arr in arrays.items():
            setattr(d, name, arr.ctypes.data)
        self._keep = list(arrays.values())
        return d

    def bake_majorants(self, layers: int = MAJORANT_LAYERS) -> "Scene":
        self.majorants, self.minorants = compute_majorant_grid(self, layers)
        self.top_altitude_km = float(f32(self.atmosphere_radius_km) - f32(self.ground_radius_km))
        return self


# ---- sky-core helpers -----------------------------------------------------------


def _cosf(x) -> np.float32:
    """Correctly rounded float32 cosine (what glibc's cosf returns)."""
    return f32(math.cos(float(f32(x))))


def _sinf(x) -> np.float32:
    return f32(math.sin(float(f32(x))))


def sun_from_degrees(elevation_deg: float, azimuth_deg: float,
                     angular_radius_rad: float = SOLAR_ANGULAR_RADIUS_RAD):
    """Sun::from_degrees (atmosphere.rs:20-36): direction, radius, solid angle."""
    e = f32(elevation_deg) * _DEG2RAD
    a = f32(azimuth_deg) * _DEG2RAD
    cos_e = _cosf(e)
    v = np.array([cos_e * _sinf(a), _sinf(e), cos_e * _cosf(a)], dtype=f32)
    length = np.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2], dtype=f32)
    v = v / length if length > 0 else np.array([0, 1, 0], dtype=f32)
    r = f32(angular_radius_rad)
    solid = _TAU * (f32(1.0) - _cosf(r))
    return tuple(float(x) for x in v), float(r), float(solid)


def rayleigh_cross_section_m2(wavelength_nm):
    """5.8e-31 (550/lambda)^4 m^2 (medium.rs:104-106), float32 powi."""
    x = (f32(550.0) / np.asarray(wavelength_nm, dtype=f32)).astype(f32)
    x2 = x * x
    return (f32(5.8e-31) * (x2 * x2)).astype(f32)


def load_cie_1931(path) -> np.ndarray:
    """CIE 1931 2-degree table rows (lambda, x, y, z) (spectrum.rs:255-300)."""
    rows = _csv_rows(Path(path))
    table = np.array([[float(c) for c in r] for r in rows], dtype=f32)
    if table.ndim != 2 or table.shape[1] != 4 or len(table) == 0:
        raise SceneError(f"{path}: expected 4 columns")
    return table


def cie_1931_2deg(table: np.ndarray, wavelength_nm) -> np.ndarray:
    """cie_1931_2deg (spectrum.rs:196-219): lerp of the 1-nm table, clamped."""
    lam = np.atleast_1d(np.asarray(wavelength_nm, dtype=f32))
    out = np.empty((len(lam), 3), dtype=f32)
    keys = table[:, 0]
    for i, l in enumerate(lam):
        if l <= keys[0]:
            out[i] = table[0, 1:]
            continue
        if l >= keys[-1]:
            out[i] = table[-1, 1:]
            continue
        j = int(np.searchsorted(keys, l, side="left"))
        if keys[j] == l:
            out[i] = table[j, 1:]
            continue
        a, b = table[j - 1], table[j]
        t = (l - a[0]) / (b[0] - a[0])
        out[i] = a[1:] + (b[1:] - a[1:]) * t  # spectrum.rs:336-338 lerp
    return out


def band_xyz_weights(cie_table: np.ndarray, centers_nm) -> np.ndarray:
    """band_xyz_weights (spectrum.rs:226-231): CIE at the band centre, no width."""
    return cie_1931_2deg(cie_table, centers_nm)


def hg_phase_values(g: float, bins: int) -> np.ndarray:
    """Henyey-Greenstein phase sampled at the cube-root mu bin centres
    (bake_opac_data.py:98-100 grid), normalised to 1 over the sphere."""
    u = (np.arange(bins, dtype=np.float64) + 0.5) / bins
    mu = 1.0 - 2.0 * u ** 3
    p = (1.0 - g * g) / (4.0 * math.pi * (1.0 + g * g - 2.0 * g * mu) ** 1.5)
    return p.astype(f32)


# ---- majorant bake: medium.rs:28-159 ---------------------------------------------


def _bracket(keys: np.ndarray, x: np.ndarray):
    """bracket (medium.rs:130-155) vectorised over x."""
    n = len(keys)
    hi = np.searchsorted(keys, x, side="left")
    lo = np.clip(hi - 1, 0, n - 1)
    hic = np.clip(hi, 0, n - 1)
    klo, khi = keys[lo], keys[hic]
    with np.errstate(divide="ignore", invalid="ignore"):
        t = np.where(khi > klo, (x - klo) / np.where(khi > klo, khi - klo, f32(1)), f32(0)).astype(f32)
    t = np.clip(t, f32(0), f32(1)).astype(f32)
    below = hi == 0
    above = hi >= n
    lo = np.where(below, 0, np.where(above, n - 1, lo))
    hic = np.where(below, 0, np.where(above, n - 1, hic))
    t = np.where(below | above, f32(0), t).astype(f32)
    return lo, hic, t


def _lerp(a, b, t):
    return (a * (f32(1) - t) + b * t).astype(f32)


def cpu_extinction(scene: Scene, altitudes: np.ndarray) -> np.ndarray:
    """CPU coefficients_at(...).extinction_total() (medium.rs:28-55, :17-25) at
    positions (0, Rg + altitude, 0); returns [B, n] float32."""
    rg = f32(scene.ground_radius_km)
    y = (rg + np.asarray(altitudes, dtype=f32)).astype(f32)
    alt = (np.sqrt((f32(0) * f32(0) + y * y) + f32(0) * f32(0), dtype=f32) - rg).astype(f32)
    top = f32(scene.atmosphere_radius_km) - rg
    inside = (alt >= 0) & (alt <= top)
    atm, aer = scene.atmosphere, scene.aerosol
    lo, hi, t = _bracket(atm["altitude_km"], alt)
    air = _lerp(atm["air_cm3"][lo], atm["air_cm3"][hi], t)
    oz = _lerp(atm["ozone_cm3"][lo], atm["ozone_cm3"][hi], t)
    lo, hi, t = _bracket(aer["altitude_km"], alt)
    mass = np.maximum(_lerp(aer["mass_g_m3"][lo], aer["mass_g_m3"][hi], t[:, None]), f32(0))  # [n, 4]
    B = scene.band_count
    ray_xs = scene.bands["rayleigh_cross_section_m2"].astype(f32)[:, None]
    oz_xs = scene.bands["ozone_cross_section_cm2"].astype(f32)[:, None]
    rayleigh = np.maximum((air[None, :] * ray_xs) * f32(1.0e9), f32(0)).astype(f32)
    ozone = np.maximum((oz[None, :] * oz_xs) * f32(1.0e5), f32(0)).astype(f32)
    optics = scene.aerosol_optics.reshape(B, SPECIES_COUNT)
    sca_sum = np.zeros((B, len(alt)), dtype=f32)
    abs_sum = np.zeros((B, len(alt)), dtype=f32)
    for s in range(SPECIES_COUNT):
        sca = (mass[None, :, s] * optics["scattering_km_inv_per_g_m3"][:, s:s + 1]).astype(f32)
        ab = (mass[None, :, s] * optics["absorption_km_inv_per_g_m3"][:, s:s + 1]).astype(f32)
        sca_sum = (sca_sum + sca).astype(f32)
        abs_sum = (abs_sum + ab).astype(f32)
    ext = ((rayleigh + sca_sum).astype(f32) + (ozone + abs_sum).astype(f32)).astype(f32)
    return np.where(inside[None, :], ext, f32(0)).astype(f32)


def compute_majorant_grid(scene: Scene, layer_count: int = MAJORANT_LAYERS):
    """compute_majorant_grid (medium.rs:63-83) with the probes of :85-102.
    Returns (majorants, minorants), each float32 [B, layer_count]."""
    top = f32(scene.atmosphere_radius_km) - f32(scene.ground_radius_km)
    dz = top / f32(layer_count)
    B = scene.band_count
    maj = np.zeros((B, layer_count), dtype=f32)
    mino = np.zeros((B, layer_count), dtype=f32)
    knots = np.concatenate([scene.atmosphere["altitude_km"], scene.aerosol["altitude_km"]]).astype(f32)
    for layer in range(layer_count):
        lo = f32(layer) * dz
        hi = f32(layer + 1) * dz
        probes = [lo, hi, f32(0.5) * (lo + hi)] + [z for z in knots if lo < z < hi]
        ext = cpu_extinction(scene, np.array(probes, dtype=f32))
        max_ext = np.maximum(ext.max(axis=1), f32(0))
        min_ext = ext.min(axis=1)
        majorant = np.maximum(max_ext * f32(1.05), f32(1.0e-8)).astype(f32)
        minorant = np.minimum(np.maximum(min_ext, f32(0)) * f32(0.99), majorant).astype(f32)
        mn = np.clip(minorant, f32(0), np.maximum(majorant, f32(0)))  # set_bounds, atmosphere.rs:102-106
        maj[:, layer] = np.maximum(majorant, mn)
        mino[:, layer] = mn
    return maj, mino


# ---- CSV loading: data.rs:15-167 ---------------------------------------------------


def _csv_rows(path: Path):
    if not path.exists():
        raise FileNotFoundError(f"{path}: No such file or directory")
    rows = []
    for line in path.read_text().splitlines():
        t = line.strip()
        if not t or t.startswith("#"):
            continue
        rows.append([c.strip() for c in t.split(",")])
    return rows


def _parse(v: str, path: Path) -> float:
    try:
        return float(v)
    except ValueError as e:
        raise SceneError(f"{path}: cannot parse {v!r}") from e


def _parse_index(v: str, path: Path, limit: int, what: str) -> int:
    """A table index: a non-negative integer (the reference parses usize,
    data.rs:123, :142-143) below `limit` (where the reference would index out of
    bounds)."""
    try:
        i = int(v)
    except ValueError as e:
        raise SceneError(f"{path}: cannot parse {what} {v!r}") from e
    if not 0 <= i < limit:
        raise SceneError(f"{path}: {what} {i} out of range [0, {limit})")
    return i


def load_bands(path: Path) -> np.ndarray:
    rows = _csv_rows(path)
    out = np.zeros(len(rows), dtype=[("index", "<i4"), ("center_nm", "<f4"), ("lower_nm", "<f4"),
                                     ("upper_nm", "<f4"), ("solar_irradiance_w_m2", "<f4"),
                                     ("ozone_cross_section_cm2", "<f4")])
    for i, r in enumerate(rows):
        if len(r) != 6:
            raise SceneError(f"{path}: expected 6 columns")
        out[i] = tuple(_parse(c, path) for c in r)
    return out


def load_atmospheric_profile(path: Path) -> np.ndarray:
    rows = _csv_rows(path)
    out = np.zeros(len(rows), dtype=ATMOSPHERE_DTYPE)
    for i, r in enumerate(rows):
        if len(r) != 4:
            raise SceneError(f"{path}: expected 4 columns")
        out[i] = tuple(_parse(c, path) for c in r)
    return out[np.argsort(out["altitude_km"], kind="stable")]


def load_aerosol_profile(path: Path) -> np.ndarray:
    rows = _csv_rows(path)
    out = np.zeros(len(rows), dtype=AEROSOL_DTYPE)
    for i, r in enumerate(rows):
        if len(r) != 1 + SPECIES_COUNT:
            raise SceneError(f"{path}: expected {1 + SPECIES_COUNT} columns")
        out["altitude_km"][i] = _parse(r[0], path)
        out["mass_g_m3"][i] = [_parse(c, path) for c in r[1:]]
    return out[np.argsort(out["altitude_km"], kind="stable")]


def _species_index(name: str) -> int:
    if name not in SPECIES_NAMES:
        raise SceneError(f"unknown species {name}")
    return SPECIES_NAMES.index(name)


def load_aerosol_optics(path: Path, band_count: int) -> np.ndarray:
    out = np.zeros(band_count * SPECIES_COUNT, dtype=OPTICS_DTYPE)
    seen = np.zeros(band_count * SPECIES_COUNT, dtype=bool)
    for r in _csv_rows(path):
        if len(r) != 4:
            raise SceneError(f"{path}: expected 4 columns")
        s = _species_index(r[0])
        b = _parse_index(r[1], path, band_count, "band")
        out[b * SPECIES_COUNT + s] = (_parse(r[2], path), _parse(r[3], path))
        seen[b * SPECIES_COUNT + s] = True
    if not seen.all():
        i = int(np.argmin(seen))
        raise SceneError(f"{path}: missing optics for band {i // SPECIES_COUNT}, "
                         f"species {SPECIES_NAMES[i % SPECIES_COUNT]}")
    return out


def load_mie_phase(path: Path, band_count: int, bins: int = PHASE_BINS) -> np.ndarray:
    values = np.zeros((SPECIES_COUNT, band_count, bins), dtype=f32)
    seen = np.zeros(values.shape, dtype=bool)
    for r in _csv_rows(path):
        if len(r) != 4:
            raise SceneError(f"{path}: expected 4 columns")
        s = _species_index(r[0])
        b = _parse_index(r[1], path, band_count, "band")
        k = _parse_index(r[2], path, bins, "bin")
        values[s, b, k] = _parse(r[3], path)
        seen[s, b, k] = True
    if not seen.all():
        raise SceneError(f"{path}: missing phase entry index {int(np.argmin(seen.ravel()))}")
    return values


def load_scene_data(data_dir, sun_elevation_deg: float, sun_azimuth_deg: float, *,
                    synthesize_missing_mie_g: float | None = None,
                    cie_path=None) -> Scene:
    """load_scene_data (data.rs:15-51).

    The reference requires data/mie_phase.csv; when it is absent and
    `synthesize_missing_mie_g` is given, every (species, band) gets a
    Henyey-Greenstein table with that asymmetry on the 1024-bin grid.
    """
    d = Path(data_dir)
    raw = load_bands(d / "bands.csv")
    if len(raw) != BAND_COUNT:
        raise SceneError(f"expected {BAND_COUNT} bands, found {len(raw)}")
    atmosphere = load_atmospheric_profile(d / "atmosphere_profile.csv")
    aerosol = load_aerosol_profile(d / "aerosol_profile.csv")
    optics = load_aerosol_optics(d / "aerosol_optics.csv", len(raw))
    mie_path = d / "mie_phase.csv"
    if mie_path.exists() or synthesize_missing_mie_g is None:
        phase = load_mie_phase(mie_path, len(raw))
    else:
        phase = np.broadcast_to(hg_phase_values(synthesize_missing_mie_g, PHASE_BINS),
                                (SPECIES_COUNT, len(raw), PHASE_BINS)).astype(f32).copy()
    direction, radius, solid = sun_from_degrees(sun_elevation_deg, sun_azimuth_deg)
    bands = np.zeros(len(raw), dtype=BAND_DTYPE)
    for name in ("center_nm", "lower_nm", "upper_nm", "ozone_cross_section_cm2"):
        bands[name] = raw[name]
    bands["rayleigh_cross_section_m2"] = rayleigh_cross_section_m2(raw["center_nm"])
    bands["solar_radiance_w_m2_sr"] = (raw["solar_irradiance_w_m2"] / f32(solid)).astype(f32)
    scene = Scene(bands=bands, atmosphere=atmosphere, aerosol=aerosol, aerosol_optics=optics, phase_values=phase,
                  sun_direction=direction, sun_angular_radius_rad=radius, sun_solid_angle_sr=solid)
    cie = Path(cie_path) if cie_path else d / "CIE_xyz_1931_2deg.csv"
    if cie.exists():
        scene.band_xyz = band_xyz_weights(load_cie_1931(cie), bands["center_nm"])
    return scene.bake_majorants(MAJORANT_LAYERS)


# ---- synthetic benchmark atmospheres ---------------------------------------------------


@dataclass
class SyntheticAtmosphere:
    """Analytic atmosphere tabulated on uniform altitude knots.

    Rayleigh: exponential density (scale height 8 km) with the lambda^-4 cross
    section of medium.rs:104-106 scaled to `rayleigh_ext_km` at
    `rayleigh_ref_nm`; Mie: one species, exponential (1.2 km), extinction
    `mie_ext_km`, albedo `mie_albedo`, HG asymmetry `mie_g`; ozone: tent
    centred at 25 km, 30 km wide, absorption `ozone_peak_km` at 600 nm with the
    spectral shape of bands.csv's cross sections.
    """

    ground_radius_km: float = 6360.0
    top_km: float = 100.0
    layers: int = 64
    rayleigh_scale_km: float = 8.0
    rayleigh_ext_km: float = 5.8e-3
    rayleigh_ref_nm: float = 680.0
    mie_scale_km: float = 1.2
    mie_ext_km: float = 4.0e-3
    mie_albedo: float = 0.9
    mie_g: float = 0.76
    ozone_center_km: float = 25.0
    ozone_width_km: float = 30.0
    ozone_peak_km: float = 6.5e-4
    ozone_ref_nm: float = 600.0
    ground_albedo: float = 0.3
    sun_angular_radius_rad: float = math.radians(0.27)
    phase_bins: int = 256


def _lerp_table(x_tab, y_tab, x):
    return np.interp(np.asarray(x, dtype=np.float64), np.asarray(x_tab, np.float64), np.asarray(y_tab, np.float64))


def synthetic_scene(wavelengths_nm, data_dir, *, sun_elevation_deg: float, sun_azimuth_deg: float = 0.0,
                    atmosphere: SyntheticAtmosphere | None = None, layer_scales=None) -> Scene:
    """A scene with the benchmark atmosphere at arbitrary wavelengths.

    `data_dir` supplies bands.csv (solar irradiance and ozone cross-section
    shapes, lerped to each wavelength) and CIE_xyz_1931_2deg.csv.
    `layer_scales` optionally multiplies the Rayleigh, Mie and ozone densities
    per majorant layer ([layers, 3], piecewise constant in altitude).
    """
    a = atmosphere or SyntheticAtmosphere()
    d = Path(data_dir)
    lam = np.asarray(wavelengths_nm, dtype=np.float64)
    raw = load_bands(d / "bands.csv")
    irr = _lerp_table(raw["center_nm"], raw["solar_irradiance_w_m2"], lam)
    o3_shape = _lerp_table(raw["center_nm"], raw["ozone_cross_section_cm2"], lam)
    o3_ref = float(_lerp_table(raw["center_nm"], raw["ozone_cross_section_cm2"], [a.ozone_ref_nm])[0])
    B = len(lam)
    spacing = np.diff(lam).mean() if B > 1 else 10.0
    # knots: uniform layer edges (plus the ozone tent vertices)
    z = np.linspace(0.0, a.top_km, a.layers + 1)
    tent = [a.ozone_center_km - a.ozone_width_km / 2, a.ozone_center_km, a.ozone_center_km + a.ozone_width_km / 2]
    z = np.unique(np.concatenate([z, [t for t in tent if 0 < t < a.top_km]]))
    scale = np.ones((a.layers, 3))
    if layer_scales is not None:
        scale = np.asarray(layer_scales, dtype=np.float64).reshape(a.layers, 3)
    dz = a.top_km / a.layers
    layer_of = np.minimum((z / dz).astype(int), a.layers - 1)
    ray_xs_ref = float(rayleigh_cross_section_m2(a.rayleigh_ref_nm))
    air0 = a.rayleigh_ext_km / (ray_xs_ref * 1.0e9)
    air = air0 * np.exp(-z / a.rayleigh_scale_km) * scale[layer_of, 0]
    tent_v = np.maximum(0.0, 1.0 - np.abs(z - a.ozone_center_km) / (a.ozone_width_km / 2))
    oz0 = a.ozone_peak_km / (o3_ref * 1.0e5) if o3_ref > 0 else 0.0
    ozone = oz0 * tent_v * scale[layer_of, 2]
    mass = np.exp(-z / a.mie_scale_km) * scale[layer_of, 1]
    atm = np.zeros(len(z), dtype=ATMOSPHERE_DTYPE)
    atm["altitude_km"] = z
    atm["temperature_k"] = 288.0
    atm["air_cm3"] = air
    atm["ozone_cm3"] = ozone
    aer = np.zeros(len(z), dtype=AEROSOL_DTYPE)
    aer["altitude_km"] = z
    aer["mass_g_m3"][:, 0] = mass
    optics = np.zeros(B * SPECIES_COUNT, dtype=OPTICS_DTYPE)
    optics["scattering_km_inv_per_g_m3"][0::SPECIES_COUNT] = a.mie_ext_km * a.mie_albedo
    optics["absorption_km_inv_per_g_m3"][0::SPECIES_COUNT] = a.mie_ext_km * (1.0 - a.mie_albedo)
    direction, radius, solid = sun_from_degrees(sun_elevation_deg, sun_azimuth_deg, a.sun_angular_radius_rad)
    bands = np.zeros(B, dtype=BAND_DTYPE)
    bands["center_nm"] = lam
    bands["lower_nm"] = lam - spacing / 2
    bands["upper_nm"] = lam + spacing / 2
    bands["ozone_cross_section_cm2"] = o3_shape
    bands["rayleigh_cross_section_m2"] = rayleigh_cross_section_m2(lam.astype(f32))
    bands["solar_radiance_w_m2_sr"] = (irr.astype(f32) / f32(solid)).astype(f32)
    phase = np.zeros((SPECIES_COUNT, B, a.phase_bins), dtype=f32)
    phase[0] = hg_phase_values(a.mie_g, a.phase_bins)[None, :]
    scene = Scene(bands=bands, atmosphere=atm, aerosol=aer, aerosol_optics=optics, phase_values=phase,
                  ground_radius_km=a.ground_radius_km, atmosphere_radius_km=a.ground_radius_km + a.top_km,
                  sun_direction=direction, sun_angular_radius_rad=radius, sun_solid_angle_sr=solid,
                  ground_albedo=a.ground_albedo)
    cie = d / "CIE_xyz_1931_2deg.csv"
    if cie.exists():
        scene.band_xyz = band_xyz_weights(load_cie_1931(cie), bands["center_nm"])
    return scene.bake_majorants(a.layers)


def wavelengths(start_nm: float, end_nm: float, count: int) -> np.ndarray:
    return np.linspace(start_nm, end_nm, count).astype(np.float64)
