import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "sky-tracer_gb300"
for p in (str(PKG), str(ROOT), str(ROOT / "oracle"), str(Path(__file__).resolve().parent)):
    if p not in sys.path:
        sys.path.insert(0, p)

DATA_DIR = ROOT / "tests" / "golden" / "data"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")
    config.addinivalue_line("markers", "slow: longer statistical checks")


@pytest.fixture(scope="session")
def data_dir():
    return DATA_DIR


@pytest.fixture(scope="session")
def ref_scene():
    """The reference's data/ tables with the sun at 0 deg (as its tests load
    them), the missing mie_phase.csv replaced by HG g=0.76 tables."""
    from sky_cuda import load_scene_data
    return load_scene_data(DATA_DIR, 0.0, 0.0, synthesize_missing_mie_g=0.76)


@pytest.fixture(scope="session")
def dome_scene():
    """The CPU-runnable benchmark scene: 32 wavelengths 380-780 nm, sun 10 deg."""
    from sky_cuda import synthetic_scene, wavelengths
    return synthetic_scene(wavelengths(380.0, 780.0, 32), DATA_DIR, sun_elevation_deg=10.0)


@pytest.fixture(scope="session")
def lib_built():
    """libsky_cuda.so, built here if needed (nvcc cross-compiles without a GPU)."""
    sys.path.insert(0, str(PKG))
    import build as skybuild
    return skybuild.build()


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu(lib_built):
    if not gpu_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    return True
