"""Host logic of the launch-shape autotuner (no GPU): it times every point of
the search space on a reduced-sample probe of the caller's render, keeps the
fastest on the scene (or restores the scene's shape when asked not to apply),
and reports every trial."""

from dataclasses import replace

import pytest

from sky_cuda import RenderConfig
from sky_cuda import autotune as at


class FakeScene:
    """Stands in for GpuScene: holds a tuning dict like sky_cuda_scene_{get,set}_tuning."""

    def __init__(self):
        self.tuning = {"variant": 2, "max_blocks_per_sm": 0, "crossing_cost": 0.1}
        self.sets = []

    def get_tuning(self):
        return dict(self.tuning)

    def set_tuning(self, **kw):
        self.tuning.update(kw)
        self.sets.append(dict(self.tuning))


def _cost(t):  # a synthetic timing surface with its minimum at variant 0, cost 0.5
    return 10.0 + abs(t["variant"] - 0) * 3.0 + abs(t["crossing_cost"] - 0.5) * 2.0


@pytest.fixture
def fake_timing(monkeypatch):
    probes = []

    def fake_time(gs, cfg, repeats):
        probes.append(cfg)
        return _cost(gs.get_tuning())

    monkeypatch.setattr(at, "_time_render", fake_time)
    return probes


def test_autotune_keeps_the_fastest(fake_timing):
    gs = FakeScene()
    cfg = RenderConfig(width=64, height=32, spp=256, sample_offset=17, flags=1)
    best, trials = at.autotune(gs, cfg)
    n = len(at.DEFAULT_SPACE["variant"]) * len(at.DEFAULT_SPACE["crossing_cost"])
    assert len(trials) == n and len(fake_timing) == n
    assert best["variant"] == 0 and best["crossing_cost"] == 0.5
    assert gs.get_tuning() == best
    assert sorted(ms for _, ms in trials)[0] == _cost(best)
    # the probe is the caller's image at spp / 8 (at least 64) from sample 0, without flags
    assert all(p.spp == 64 and p.sample_offset == 0 and p.flags == 0 and p.width == 64 for p in fake_timing)


def test_autotune_restores_the_shape_when_not_applying(fake_timing):
    gs = FakeScene()
    before = gs.get_tuning()
    best, trials = at.autotune(gs, RenderConfig(width=8, height=8, spp=16), space={"crossing_cost": (0.25, 1.0)},
                               apply=False)
    assert best["crossing_cost"] == 0.25 and best["variant"] == before["variant"]
    assert gs.get_tuning() == before
    assert [t["crossing_cost"] for t, _ in trials] == [0.25, 1.0]
    # below 64 spp the probe is the whole render
    assert all(p.spp == 16 for p in fake_timing)


def test_autotune_probe_spp_override(fake_timing):
    gs = FakeScene()
    at.autotune(gs, replace(RenderConfig(width=8, height=8, spp=1024)), space={"variant": (1,)}, probe_spp=7)
    assert [p.spp for p in fake_timing] == [7]
