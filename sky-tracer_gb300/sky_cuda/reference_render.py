"""sky-reference-render on the GB300 tracer: the reference's offline render
command (crates/sky-reference-render/src/main.rs) with its flags, defaults,
outputs and messages, rendering through this library.

    python -m sky_cuda.reference_render --spp 256 --sun-elevation-deg 10 --out out

Outputs (film_output.rs:12-124, main.rs:156-213):
    out/bands/sky_{center:03.0f}nm.exr   one float RGB EXR per band (v, v, v)
    out/sky_rgb.exr                      white-balanced linear sRGB
    out/sky_rgb.png                      the same, tone-mapped (1 - exp(-exposure x)), sRGB 8-bit
    out/asset.json                       spectral asset manifest v0 with its colorimetry block
--rebuild-rgb-only rebuilds the RGB files and the colorimetry block from the
band EXRs on the host (main.rs:85-104).  The linear sRGB of a render comes
from the tracer's epilogue (SkyDeviceOutputs.rgb); the rebuild path computes
it on the host with the same conversion.
"""

from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

from . import _abi
from .colorimetry import SpectralRgbConverter, colorimetry_manifest, to_srgb8, tonemap
from .exr import read_exr, write_exr_rgb, write_png_rgb8
from .render import DEFAULT_SEED, Film, GpuScene, RenderConfig
from .scene import band_xyz_weights, load_bands, load_cie_1931, load_scene_data

PANORAMA_DEFAULT = (2048, 1024)      # main.rs:55-56
SKY_VIEW_LUT_DEFAULT = (256, 256)    # main.rs:57-58
SPECTRAL_PANORAMA_KIND = "spectral_panorama_v0"        # asset.rs:3
SPECTRAL_SKY_VIEW_LUT_KIND = "spectral_sky_view_lut_v0"  # asset.rs:4


def parse_args(argv=None):
    p = argparse.ArgumentParser(prog="sky-reference-render",
                                description="Offline spectral OPAC atmosphere path tracer (GB300)")
    p.add_argument("--width", type=int)
    p.add_argument("--height", type=int)
    p.add_argument("--spp", type=int, default=1024)
    p.add_argument("--seed", type=int, default=DEFAULT_SEED)
    p.add_argument("--out", type=Path, default=Path("out"))
    p.add_argument("--data-dir", type=Path, default=Path("data"))
    p.add_argument("--sun-elevation-deg", type=float, default=0.0)
    p.add_argument("--sun-azimuth-deg", type=float, default=0.0)
    p.add_argument("--observer-altitude-km", type=float, default=0.2)
    p.add_argument("--direct-light-samples", type=int, default=1)
    p.add_argument("--png-exposure", type=float, default=0.05)
    p.add_argument("--sky-view-lut", action="store_true")
    p.add_argument("--rebuild-rgb-only", action="store_true")
    # flags the reference CLI does not have (its behaviour when left at their defaults)
    p.add_argument("--mie-g", type=float, default=0.76,
                   help="HG asymmetry of the phase tables used when data/mie_phase.csv is absent")
    p.add_argument("--phase-sampling", choices=("isotropic", "tabulated"), default="isotropic")
    p.add_argument("--tracking", choices=("segment-restart", "residual-carry", "merged-layers"),
                   default="segment-restart")
    return p.parse_args(argv)


def resolve_dimensions(width, height, sky_view_lut):
    dw, dh = SKY_VIEW_LUT_DEFAULT if sky_view_lut else PANORAMA_DEFAULT
    return (width or dw, height or dh)


def band_exr_name(center_nm: float) -> str:
    """bands/sky_{:03.0}nm.exr (film_output.rs:86, main.rs:161): Rust's {:03.0}
    rounds half to even and pads to 3 digits."""
    return f"bands/sky_{round(float(np.float32(center_nm))):03d}nm.exr"


def converter_for(data_dir: Path, centers_nm) -> SpectralRgbConverter:
    """SpectralRgbConverter::new_solar_d65 of the data's bands: CIE weights at
    the band centres, solar irradiance of bands.csv."""
    raw = load_bands(Path(data_dir) / "bands.csv")
    cie = load_cie_1931(Path(data_dir) / "CIE_xyz_1931_2deg.csv")
    return SpectralRgbConverter(band_xyz_weights(cie, centers_nm), raw["solar_irradiance_w_m2"])


def write_band_exrs(film: Film, out_dir: Path, centers_nm) -> None:
    (out_dir / "bands").mkdir(parents=True, exist_ok=True)
    img = film.as_array()
    for b, c in enumerate(centers_nm):
        v = img[:, :, b]
        write_exr_rgb(out_dir / band_exr_name(c), np.stack([v, v, v], axis=-1))


def write_rgb_outputs(rgb_linear: np.ndarray, width: int, height: int, out_dir: Path, exposure: float) -> None:
    out_dir.mkdir(parents=True, exist_ok=True)
    rgb = np.asarray(rgb_linear, dtype=np.float32).reshape(height, width, 3)
    write_exr_rgb(out_dir / "sky_rgb.exr", rgb)
    write_png_rgb8(out_dir / "sky_rgb.png", to_srgb8(tonemap(rgb, exposure)))


def read_film_from_band_exrs(out_dir: Path, centers_nm) -> Film:
    """read_film_from_band_exrs (film_output.rs:36-78): the R channel of each band EXR."""
    if len(centers_nm) == 0:
        raise ValueError("no spectral bands to rebuild")
    planes = []
    for c in centers_nm:
        path = out_dir / band_exr_name(c)
        r = read_exr(path)["R"]
        if planes and r.shape != planes[0].shape:
            raise ValueError(f"band EXR {path} has dimensions {r.shape[1]}x{r.shape[0]}, "
                             f"expected {planes[0].shape[1]}x{planes[0].shape[0]}")
        planes.append(r)
    h, w = planes[0].shape
    values = np.stack(planes, axis=-1).reshape(-1).astype(np.float32)
    return Film(w, h, len(centers_nm), values)


def asset_manifest(cfg: RenderConfig, args, centers_nm, converter) -> dict:
    """SpectralAssetManifest v0 (asset.rs:6-98, main.rs:156-200)."""
    return {
        "version": 0,
        "kind": SPECTRAL_SKY_VIEW_LUT_KIND if args.sky_view_lut else SPECTRAL_PANORAMA_KIND,
        "dimensions": [cfg.width, cfg.height],
        "spp": cfg.spp,
        "seed": cfg.seed,
        "sun_elevation_deg": float(np.float32(cfg.sun_elevation_deg)),
        "sun_azimuth_deg": float(np.float32(cfg.sun_azimuth_deg)),
        "observer_altitude_km": float(np.float32(cfg.observer_altitude_km)),
        "band_centers_nm": [float(np.float32(c)) for c in centers_nm],
        "data_hash": None,
        "colorimetry": colorimetry_manifest(converter),
        "files": {"rgb_exr": "sky_rgb.exr", "rgb_png": "sky_rgb.png",
                  "band_exrs": [band_exr_name(c) for c in centers_nm]},
    }


def format_duration(seconds: float) -> str:
    """format_duration (main.rs:250-262)."""
    if seconds < 1.0:
        return f"{seconds * 1000.0:.1f}ms"
    if seconds < 60.0:
        return f"{seconds:.2f}s"
    minutes = int(seconds // 60)
    return f"{minutes}m{seconds - minutes * 60:.1f}s"


def main(argv=None) -> int:
    t_total = time.perf_counter()
    args = parse_args(argv)
    width, height = resolve_dimensions(args.width, args.height, args.sky_view_lut)
    out_dir = args.out
    cfg = RenderConfig(width=width, height=height, spp=args.spp, seed=args.seed,
                       sun_elevation_deg=args.sun_elevation_deg, sun_azimuth_deg=args.sun_azimuth_deg,
                       observer_altitude_km=args.observer_altitude_km,
                       direct_light_samples=args.direct_light_samples,
                       output_projection=_abi.PROJECTION_SKY_VIEW_LUT if args.sky_view_lut else _abi.PROJECTION_PANORAMA,
                       phase_sampling=_abi.PHASE_TABULATED if args.phase_sampling == "tabulated" else _abi.PHASE_ISOTROPIC,
                       tracking=("segment-restart", "residual-carry", "merged-layers").index(args.tracking))
    t0 = time.perf_counter()
    scene = load_scene_data(args.data_dir, args.sun_elevation_deg, args.sun_azimuth_deg,
                            synthesize_missing_mie_g=args.mie_g)
    centers = [float(c) for c in scene.bands["center_nm"]]
    converter = converter_for(args.data_dir, centers)
    t_load = time.perf_counter() - t0

    if args.rebuild_rgb_only:
        t0 = time.perf_counter()
        film = read_film_from_band_exrs(out_dir, centers)
        rgb = converter.to_linear_srgb(film.values.reshape(-1, film.band_count))
        write_rgb_outputs(rgb, film.width, film.height, out_dir, args.png_exposure)
        manifest_path = out_dir / "asset.json"
        if manifest_path.exists():  # update_asset_colorimetry (main.rs:202-213)
            manifest = json.loads(manifest_path.read_text())
            manifest["colorimetry"] = colorimetry_manifest(converter)
            manifest_path.write_text(json.dumps(manifest, indent=2))
        t_out = time.perf_counter() - t0
        print(f"rebuilt rgb outputs from {len(centers)} band EXRs in {out_dir}")
        print(f"timing: load={format_duration(t_load)} output={format_duration(t_out)} "
              f"total={format_duration(time.perf_counter() - t_total)}")
        return 0

    label = "sky-view LUT" if args.sky_view_lut else "panorama"  # OutputProjection::label (config.rs:30-35)
    print(f"config: gpu-integrator output={label} direct-light-samples={args.direct_light_samples}")
    t0 = time.perf_counter()
    with GpuScene(scene) as gs:
        film, rgb, _ = gs.render_rgb(cfg)
    t_render = time.perf_counter() - t0
    t0 = time.perf_counter()
    write_band_exrs(film, out_dir, centers)
    write_rgb_outputs(rgb, width, height, out_dir, args.png_exposure)
    (out_dir / "asset.json").write_text(json.dumps(asset_manifest(cfg, args, centers, converter), indent=2))
    t_out = time.perf_counter() - t0
    print(f"wrote {width}x{height} {label} with {cfg.spp} spp to {out_dir}")
    print(f"timing: load={format_duration(t_load)} render={format_duration(t_render)} "
          f"output={format_duration(t_out)} total={format_duration(time.perf_counter() - t_total)}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
