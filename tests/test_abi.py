"""CPU checks of the C ABI: the library builds and exports every declared
symbol, the ctypes mirror matches the C header byte for byte, and calls
without a usable device fail with the NoAdapter-equivalent status."""

import ctypes
import re
import subprocess
from pathlib import Path

import pytest

from sky_cuda import _abi

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "sky_cuda.h"


def _declared_functions(header: Path):
    text = header.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sky_cuda_\w+)\s*\(", text)))


def test_header_and_ctypes_agree_on_functions():
    assert _declared_functions(HEADER) == sorted(_abi.declared_symbols())


def test_header_flags_match_the_mirrors():
    """SKY_FLAG_* of the header = the Python and Rust constants."""
    flags = dict((k, int(v)) for k, v in re.findall(r"#define SKY_FLAG_(\w+) (\d+)u", HEADER.read_text()))
    assert flags == {"ACCUMULATE": _abi.FLAG_ACCUMULATE, "COUNT_EVENTS": _abi.FLAG_COUNT_EVENTS}
    rust = (ROOT / "sky-tracer_gb300" / "rust" / "sky-cuda" / "src" / "ffi.rs").read_text()
    assert dict((k, int(v)) for k, v in re.findall(r"pub const SKY_FLAG_(\w+): u32 = (\d+);", rust)) == flags


def test_library_exports_every_declared_symbol(lib_built):
    out = subprocess.run(["nm", "-D", "--defined-only", str(lib_built)], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [s for s in _declared_functions(HEADER) if s not in exported]
    assert not missing, missing
    lib = ctypes.CDLL(str(lib_built))
    for s in _declared_functions(HEADER):
        assert getattr(lib, s)


def test_struct_layouts_match_header(tmp_path):
    structs = {
        "SkyBand": _abi.BAND_DTYPE, "SkyAtmospherePoint": _abi.ATMOSPHERE_DTYPE,
        "SkyAerosolPoint": _abi.AEROSOL_DTYPE, "SkyAerosolOptics": _abi.OPTICS_DTYPE,
    }
    ctypes_structs = {
        "SkySceneDesc": _abi.SkySceneDesc, "SkyRenderConfig": _abi.SkyRenderConfig,
        "SkyRenderStats": _abi.SkyRenderStats, "SkyDeviceOutputs": _abi.SkyDeviceOutputs,
        "SkyTuning": _abi.SkyTuning, "SkyBatchJob": _abi.SkyBatchJob,
        "SkyAdjointParams": _abi.SkyAdjointParams, "SkyAdjointGrads": _abi.SkyAdjointGrads,
        "SkyComboScore": _abi.SkyComboScore, "SkyMieDistribution": _abi.SkyMieDistribution,
        "SkyMieBand": _abi.SkyMieBand,
    }
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HEADER}"', "int main(void){"]
    for name, dt in structs.items():
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for field in dt.names:
            if field.startswith("_"):
                continue
            lines.append(f'printf("{name}.{field} %zu\\n", offsetof({name}, {field}));')
    for name, st in ctypes_structs.items():
        lines.append(f'printf("{name} %zu\\n", sizeof({name}));')
        for field, _ in st._fields_:
            if field.startswith("_"):
                continue
            lines.append(f'printf("{name}.{field} %zu\\n", offsetof({name}, {field}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-o", str(exe), str(src)], check=True)
    c_layout = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], capture_output=True, text=True,
                                                                    check=True).stdout.splitlines())
    for name, dt in structs.items():
        assert int(c_layout[name]) == dt.itemsize, name
        for field in dt.names:
            if not field.startswith("_"):
                assert int(c_layout[f"{name}.{field}"]) == dt.fields[field][1], (name, field)
    for name, st in ctypes_structs.items():
        assert int(c_layout[name]) == ctypes.sizeof(st), name
        for field, _ in st._fields_:
            if not field.startswith("_"):
                assert int(c_layout[f"{name}.{field}"]) == getattr(st, field).offset, (name, field)


def test_version_string(lib_built):
    lib = _abi.load_library()
    assert b"sky_cuda" in lib.sky_cuda_version()


def test_invalid_arguments_are_rejected_without_a_device(lib_built, dome_scene):
    """Argument errors map to InvalidConfig before any device work; with no
    usable device, scene creation reports the NoAdapter-equivalent status."""
    from conftest import gpu_available
    lib = _abi.load_library()
    handle = ctypes.c_void_p()
    assert lib.sky_cuda_scene_create(None, ctypes.byref(handle)) in (_abi.SKY_ERR_INVALID_CONFIG,
                                                                     _abi.SKY_ERR_NO_DEVICE)
    cfg = _abi.SkyRenderConfig()
    film = (ctypes.c_float * 4)()
    assert lib.sky_cuda_render(None, ctypes.byref(cfg), film, 4, None) == _abi.SKY_ERR_INVALID_CONFIG
    assert "scene" in _abi.last_error(lib)
    if not gpu_available():
        desc = dome_scene.desc()
        st = lib.sky_cuda_scene_create(ctypes.byref(desc), ctypes.byref(handle))
        assert st == _abi.SKY_ERR_NO_DEVICE
        with pytest.raises(_abi.SkyCudaError) as e:
            _abi.check(st, lib)
        assert e.value.status == _abi.SKY_ERR_NO_DEVICE
