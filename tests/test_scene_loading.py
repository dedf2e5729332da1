"""Host-side loading of the reference's `data/` tables (data.rs:15-152): the
repository's tables load, and malformed tables raise SceneError (the
reference's Box<dyn Error>) instead of loading wrong values."""

import shutil

import numpy as np
import pytest

from sky_cuda.scene import PHASE_BINS, SceneError, hg_phase_values, load_mie_phase, load_scene_data


@pytest.fixture
def data_copy(tmp_path, data_dir):
    d = tmp_path / "data"
    shutil.copytree(data_dir, d)
    return d


def _edit(path, old, new):
    text = path.read_text()
    assert old in text
    path.write_text(text.replace(old, new, 1))


def test_repository_tables_load(data_copy):
    s = load_scene_data(data_copy, 10.0, 0.0, synthesize_missing_mie_g=0.76)
    assert s.band_count == 41 and np.all(np.isfinite(s.phase_values))
    assert np.all(np.diff(s.atmosphere["altitude_km"]) > 0)


def test_missing_mie_table_is_an_error_unless_synthesized(data_copy):
    with pytest.raises(FileNotFoundError):
        load_scene_data(data_copy, 10.0, 0.0)


@pytest.mark.parametrize("old,new,match", [
    ("inso,0,", "inso,-1,", "band -1 out of range"),       # usize in the reference: no wrap-around
    ("inso,0,", "inso,41,", "band 41 out of range"),
    ("inso,0,", "inso,zero,", "cannot parse band"),
    ("inso,0,", "dust,0,", "unknown species"),
    ("inso,0,1.57930891e+02", "inso,0,abc", "cannot parse"),
])
def test_malformed_optics_rows_raise(data_copy, old, new, match):
    _edit(data_copy / "aerosol_optics.csv", old, new)
    with pytest.raises(SceneError, match=match):
        load_scene_data(data_copy, 10.0, 0.0, synthesize_missing_mie_g=0.76)


def test_missing_optics_entry_raises(data_copy):
    p = data_copy / "aerosol_optics.csv"
    p.write_text("\n".join(l for l in p.read_text().splitlines() if not l.startswith("suso,7,")) + "\n")
    with pytest.raises(SceneError, match="missing optics"):
        load_scene_data(data_copy, 10.0, 0.0, synthesize_missing_mie_g=0.76)


def test_wrong_column_count_raises(data_copy):
    p = data_copy / "bands.csv"
    lines = p.read_text().splitlines()
    i = next(k for k, l in enumerate(lines) if l.strip() and not l.startswith("#") and l[0].isdigit())
    lines[i] = lines[i] + ",1.0"
    p.write_text("\n".join(lines) + "\n")
    with pytest.raises(SceneError, match="expected 6 columns"):
        load_scene_data(data_copy, 10.0, 0.0, synthesize_missing_mie_g=0.76)


def test_mie_phase_table_indices_checked(tmp_path):
    """A full table loads; a negative or out-of-range bin, or a missing entry, raises."""
    p = tmp_path / "mie_phase.csv"
    hg = hg_phase_values(0.5, PHASE_BINS)
    rows = [f"{sp},{b},{k},{hg[k]:.8e}" for sp in ("inso", "waso", "soot", "suso") for b in range(2)
            for k in range(PHASE_BINS)]
    p.write_text("\n".join(rows) + "\n")
    v = load_mie_phase(p, 2)
    assert v.shape == (4, 2, PHASE_BINS) and np.allclose(v[3, 1], hg, rtol=1e-6)
    for bad, match in ((f"inso,0,-1,{hg[0]:.8e}", "bin -1 out of range"),
                       (f"inso,0,{PHASE_BINS},{hg[0]:.8e}", f"bin {PHASE_BINS} out of range"),
                       (f"inso,2,0,{hg[0]:.8e}", "band 2 out of range")):
        p.write_text("\n".join(rows + [bad]) + "\n")
        with pytest.raises(SceneError, match=match):
            load_mie_phase(p, 2)
    p.write_text("\n".join(rows[:-1]) + "\n")
    with pytest.raises(SceneError, match="missing phase entry"):
        load_mie_phase(p, 2)
