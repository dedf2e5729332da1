"""The sky-cuda Rust crate's calls, made from C (tests/c_abi_harness.c and,
for its differentiable-render pair, tests/c_adjoint_harness.c).

No Rust toolchain is installed (cargo and rustc are absent on the x86 build
host and on the aarch64 GPU host), so the crate's FFI sequence is exercised by a C program
that makes the same calls with the same structs: sky_cuda_render_desc (the
crate's `render`), sky_cuda_scene_create / sky_cuda_render /
sky_cuda_scene_destroy (its `GpuScene`), and the error path through
sky_cuda_last_error (its RenderError mapping).  On the CPU the harness is
compiled and linked against libsky_cuda.so; on the GPU it renders the
reference's own data/ scene and its film must equal the Python one-shot
render of the same scene and config.  The adjoint harness makes the crate's
Adjoint calls (sky_cuda_adjoint_forward with a chain-radiance buffer, then
sky_cuda_adjoint_backward reading it) on device buffers of its own; its film
and gradients must equal the Python AdjointRenderer's on the same inputs.
"""

import os
import struct
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from sky_cuda import RenderConfig, render

ROOT = Path(__file__).resolve().parents[1]
HARNESS = ROOT / "tests" / "c_abi_harness.c"
LIB_DIR = ROOT / "sky-tracer_gb300" / "_build"


def build_harness(out_dir: Path) -> Path:
    exe = out_dir / "c_abi_harness"
    cmd = ["gcc", "-std=c11", "-O2", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"), str(HARNESS),
           "-L", str(LIB_DIR), "-lsky_cuda", f"-Wl,-rpath,{LIB_DIR}", "-o", str(exe)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return exe


ADJOINT_HARNESS = ROOT / "tests" / "c_adjoint_harness.c"
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def build_adjoint_harness(out_dir: Path) -> Path:
    exe = out_dir / "c_adjoint_harness"
    cmd = ["gcc", "-std=c11", "-O2", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"),
           "-I", str(CUDA_HOME / "include"), str(ADJOINT_HARNESS), "-L", str(LIB_DIR), "-lsky_cuda",
           f"-Wl,-rpath,{LIB_DIR}", "-L", str(CUDA_HOME / "lib64"), "-lcudart",
           f"-Wl,-rpath,{CUDA_HOME / 'lib64'}", "-o", str(exe)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    return exe


def write_scene(scene, path: Path) -> None:
    """The harness's scene file: counts, scalars, then the table rows."""
    with open(path, "wb") as f:
        f.write(b"SKYT")
        f.write(struct.pack("<5I", scene.band_count, len(scene.atmosphere), len(scene.aerosol), scene.layer_count,
                            scene.phase_bins))
        f.write(struct.pack("<11f", scene.ground_radius_km, scene.atmosphere_radius_km, scene.top_altitude_km,
                            *scene.sun_direction, scene.sun_angular_radius_rad, scene.sun_solid_angle_sr,
                            scene.ground_albedo, 0.0, 0.0))
        for table in (scene.bands, scene.atmosphere, scene.aerosol, scene.aerosol_optics,
                      np.ascontiguousarray(scene.majorants, dtype=np.float32),
                      np.ascontiguousarray(scene.phase_values, dtype=np.float32)):
            f.write(np.ascontiguousarray(table).tobytes())


def test_harness_compiles_and_links_against_the_library(lib_built, tmp_path):
    exe = build_harness(tmp_path)
    assert exe.exists()
    # the dynamic symbols the harness binds resolve in the library
    res = subprocess.run(["nm", "-D", "--undefined-only", str(exe)], capture_output=True, text=True)
    for sym in ("sky_cuda_render_desc", "sky_cuda_scene_create", "sky_cuda_render", "sky_cuda_last_error",
                "sky_cuda_scene_destroy", "sky_cuda_version"):
        assert sym in res.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("projection", [0, 1])
def test_harness_film_equals_the_python_render(gpu, ref_scene, tmp_path, projection):
    exe = build_harness(tmp_path)
    scene_file, film_file = tmp_path / "scene.bin", tmp_path / "film.bin"
    write_scene(ref_scene, scene_file)
    cfg = RenderConfig(width=24, height=12, spp=8, seed=0x5EC7_2026_0430, output_projection=projection)
    res = subprocess.run([str(exe), str(scene_file), "24", "12", "8", str(cfg.seed), str(projection),
                          str(film_file)], capture_output=True, text=True, timeout=300,
                         env={**os.environ, "LD_LIBRARY_PATH": str(LIB_DIR)})
    assert res.returncode == 0, res.stdout + res.stderr
    film_c = np.fromfile(film_file, dtype=np.float32)
    film_py = render(ref_scene, cfg).values
    assert film_c.shape == film_py.shape == (24 * 12 * ref_scene.band_count,)
    # the same one-shot call on the same inputs: equal up to the order of the FP64 cell sums
    np.testing.assert_allclose(film_c, film_py, rtol=1e-6, atol=0)
    assert np.all(np.isfinite(film_c)) and np.all(film_c >= 0) and np.any(film_c > 0)


def test_adjoint_harness_compiles_and_links_against_the_library(lib_built, tmp_path):
    if not (CUDA_HOME / "include" / "cuda_runtime.h").exists():
        pytest.skip("no CUDA runtime headers")
    exe = build_adjoint_harness(tmp_path)
    res = subprocess.run(["nm", "-D", "--undefined-only", str(exe)], capture_output=True, text=True)
    for sym in ("sky_cuda_scene_create", "sky_cuda_adjoint_param_count", "sky_cuda_adjoint_forward",
                "sky_cuda_adjoint_backward", "sky_cuda_last_error", "sky_cuda_scene_destroy"):
        assert sym in res.stdout


@pytest.mark.gpu
def test_adjoint_harness_matches_the_python_renderer(gpu, dome_scene, tmp_path):
    """The crate's Adjoint forward/backward and forward_batch/backward_batch
    from C against AdjointRenderer on the same scene, parameters, config and
    dLoss/dfilm: the films to the order of the FP64 cell sums, the gradients
    to the rounding of the per-warp FP32 gradient sums."""
    import torch

    from sky_cuda import GpuScene, _abi
    from sky_cuda.adjoint import BAND_PARAMS, AdjointRenderer, initial_layer_params

    exe = build_adjoint_harness(tmp_path)
    scene_file = tmp_path / "scene.bin"
    write_scene(dome_scene, scene_file)
    w, h, spp, seed = 16, 8, 16, 0x5EC7_2026_0430
    theta = initial_layer_params(dome_scene, 0.76)
    theta[:3 * dome_scene.layer_count] *= np.float32(1.02)
    (tmp_path / "params.bin").write_bytes(theta.astype(np.float32).tobytes())
    dloss = np.random.default_rng(7).normal(size=w * h * dome_scene.band_count).astype(np.float32)
    (tmp_path / "dloss.bin").write_bytes(dloss.tobytes())
    prefix = tmp_path / "out"
    res = subprocess.run([str(exe), str(scene_file), str(w), str(h), str(spp), str(seed), str(tmp_path / "params.bin"),
                          str(tmp_path / "dloss.bin"), str(prefix)], capture_output=True, text=True, timeout=300,
                         env={**os.environ, "LD_LIBRARY_PATH": str(LIB_DIR)})
    assert res.returncode == 0, res.stdout + res.stderr
    film_c = np.fromfile(str(prefix) + ".film", dtype=np.float32)
    lg_c = np.fromfile(str(prefix) + ".layer_grad", dtype=np.float64)
    bg_c = np.fromfile(str(prefix) + ".band_grad", dtype=np.float64)
    batch_films = [np.fromfile(str(prefix) + f".batch_film{i}", dtype=np.float32) for i in range(2)]
    batch_lg = np.fromfile(str(prefix) + ".batch_layer_grad", dtype=np.float64)
    batch_bg = np.fromfile(str(prefix) + ".batch_band_grad", dtype=np.float64)
    high_sun = (0.0, 0.5, 0.8660254)  # the harness's second render

    cfg = RenderConfig(width=w, height=h, spp=spp, seed=seed, observer_altitude_km=0.2,
                       phase_sampling=_abi.PHASE_TABULATED, tracking=_abi.TRACKING_MERGED_LAYERS)
    with GpuScene(dome_scene) as gs:
        r = AdjointRenderer(gs, cfg)
        th = torch.as_tensor(theta, device="cuda").contiguous()
        band = torch.ones(dome_scene.band_count * BAND_PARAMS, dtype=torch.float32, device="cuda")
        chains = r.new_chain_buffer()
        film_py = r.forward(th, band, chains=chains)["film"].cpu().numpy()
        d = torch.as_tensor(dloss, device="cuda")
        lg, bg = r.backward(th, band, d, chains=chains)
        film_high = r.forward(th, band, sun=high_sun)["film"].cpu().numpy()
        lg_high, bg_high = r.backward(th, band, d, sun=high_sun)
    np.testing.assert_allclose(film_c, film_py, rtol=1e-6, atol=0)
    np.testing.assert_allclose(batch_films[0], film_py, rtol=1e-6, atol=0)
    np.testing.assert_allclose(batch_films[1], film_high, rtol=1e-6, atol=0)
    assert not np.array_equal(batch_films[0], batch_films[1])
    lg, bg = lg.cpu().numpy(), bg.cpu().numpy()
    for a, b in ((lg_c, lg), (bg_c, bg), (batch_lg, lg + lg_high.cpu().numpy()),
                 (batch_bg, bg + bg_high.cpu().numpy())):
        assert a.shape == b.shape and np.any(b != 0.0)
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-4 * np.abs(b).max())


if __name__ == "__main__":
    sys.exit(pytest.main([__file__, "-q"]))
