"""World-size-2 gloo ranks on CPU: one render split into pixel-row slabs
(SkyRenderConfig.row_begin / row_count), gathered to rank 0 and joined there,
equals the whole render; a sweep splits into contiguous blocks of whole
elevations; the max-over-ranks timing reduction.

The renderer of each rank is a stand-in that needs no GPU: a fake renderer
whose value is a function of the image pixel, and the oracle (test
infrastructure) rendering the slab's rows.  Both index pixels the way the
tracer does (image pixel in the random stream, slab pixel in the output), so
a wrong slab offset shows up as a mismatch."""

import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def fake_slab(cfg, bands):
    """[slab pixels, bands]: a hash of (image pixel, band), like a render whose
    random stream is keyed by the image pixel."""
    rows = cfg.row_count or cfg.height
    y = np.arange(cfg.row_begin, cfg.row_begin + rows)[:, None]
    x = np.arange(cfg.width)[None, :]
    pixel = (y * cfg.width + x).reshape(-1, 1).astype(np.uint64)
    band = np.arange(bands, dtype=np.uint64)[None, :]
    h = (pixel * np.uint64(2654435761) + band * np.uint64(40503) + np.uint64(cfg.seed)) % np.uint64(1000003)
    return h.astype(np.float64)


def oracle_slab(scene, cfg):
    """The oracle's per-cell sums of the slab's rows ([slab pixels, bands])."""
    import sky_oracle
    from dataclasses import replace
    whole = replace(cfg, row_begin=0, row_count=0)
    s, _, _, _ = sky_oracle.render(scene, whole, row_begin=cfg.row_begin, row_step=1, threads=1)
    rows = cfg.row_count or cfg.height
    return s[cfg.row_begin * cfg.width:(cfg.row_begin + rows) * cfg.width]


def _scene_and_config():
    from sky_cuda import RenderConfig, synthetic_scene, wavelengths
    from sky_cuda import _abi
    data = os.path.join(os.path.dirname(__file__), "golden", "data")
    scene = synthetic_scene(wavelengths(380.0, 780.0, 4), data, sun_elevation_deg=10.0)
    cfg = RenderConfig(width=6, height=5, spp=4, seed=21, max_orders=4, phase_sampling=_abi.PHASE_TABULATED,
                       tracking=_abi.TRACKING_MERGED_LAYERS)
    return scene, cfg


def _worker(rank, world, port, q):
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    for p in (os.path.join(here, "..", "sky-tracer_gb300"), os.path.join(here, "..", "oracle"), here):
        sys.path.insert(0, p)
    import torch.distributed as dist
    from sky_cuda.parallel import (balanced_row_slabs, broadcast_slabs, elevation_shard, gather_to_rank0,
                                   max_over_ranks, render_split)
    from sky_cuda.sweep import elevation_schedule
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    scene, cfg = _scene_and_config()
    fake = render_split(lambda c: fake_slab(c, 3), cfg, rank, world, 3)
    # cost-balanced slabs: rank 0 alone knows the row costs (its pilot) and broadcasts the cut
    slabs = balanced_row_slabs([5.0, 1.0, 1.0, 1.0, 1.0], world) if rank == 0 else None
    slabs = broadcast_slabs(slabs)
    orc = render_split(lambda c: oracle_slab(scene, c), cfg, rank, world, scene.band_count, slabs=slabs)
    elev = elevation_schedule(32)
    mine = [float(elev[i]) for i in elevation_shard(len(elev), rank, world)]
    sweep = gather_to_rank0(mine)
    t = max_over_ranks(1.0 + rank)
    if rank == 0:
        q.put((t, fake, orc, sweep, slabs))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_row_split_equals_whole_render():
    import sky_oracle
    import torch.multiprocessing as mp
    sky_oracle.load()  # built before the ranks start
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
        assert p.exitcode == 0
    t, fake, orc, sweep, slabs = q.get()
    assert t == 2.0
    assert slabs == [(0, 1), (1, 4)]  # the costly first row alone on rank 0
    scene, cfg = _scene_and_config()
    np.testing.assert_array_equal(fake, fake_slab(cfg, 3))
    whole, _, _, _ = sky_oracle.render(scene, cfg, threads=1)
    np.testing.assert_array_equal(orc, whole)
    assert orc.shape == (cfg.pixels, scene.band_count) and np.any(orc > 0)
    # whole elevations, contiguous blocks in rank order, covering the sweep once
    from sky_cuda.sweep import elevation_schedule
    assert [e for part in sweep for e in part] == [float(e) for e in elevation_schedule(32)]


def test_row_slabs_partition_the_image():
    from sky_cuda import RenderConfig
    from sky_cuda.parallel import elevation_shard, row_slabs, slab_config
    for height, world in [(256, 8), (256, 3), (5, 5), (7, 2), (1, 1)]:
        slabs = row_slabs(height, world)
        assert len(slabs) == world and slabs[0][0] == 0
        assert all(b1 == b0 + n0 for (b0, n0), (b1, _) in zip(slabs, slabs[1:]))
        assert sum(n for _, n in slabs) == height and max(n for _, n in slabs) - min(n for _, n in slabs) <= 1
    with pytest.raises(ValueError):
        row_slabs(3, 4)
    cfg = slab_config(RenderConfig(width=4, height=10, spp=1), 2, 3)
    assert (cfg.row_begin, cfg.row_count, cfg.pixels) == (7, 3, 12)
    with pytest.raises(ValueError):
        slab_config(cfg, 0, 2)  # already a slab
    assert [list(elevation_shard(5, r, 2)) for r in range(2)] == [[0, 1, 2], [3, 4]]
    with pytest.raises(ValueError):
        elevation_shard(5, 2, 2)


def test_balanced_slabs_minimise_the_largest_slab():
    import itertools
    from sky_cuda import RenderConfig
    from sky_cuda.parallel import balanced_row_slabs, slab_config
    rng = np.random.default_rng(3)
    for trial in range(60):
        height = int(rng.integers(1, 11))
        world = int(rng.integers(1, height + 1))
        cost = rng.choice([0.0, 0.5, 1.0, 3.0, 10.0], size=height)
        slabs = balanced_row_slabs(cost, world)
        assert len(slabs) == world and slabs[0][0] == 0 and all(n >= 1 for _, n in slabs)
        assert all(b1 == b0 + n0 for (b0, n0), (b1, _) in zip(slabs, slabs[1:]))
        assert sum(n for _, n in slabs) == height
        got = max(cost[b:b + n].sum() for b, n in slabs)
        best = min(max(cost[a:b].sum() for a, b in zip((0,) + cuts, cuts + (height,)))
                   for cuts in itertools.combinations(range(1, height), world - 1))
        assert got <= best * (1 + 1e-9) + 1e-12, (cost, world, slabs)
    # the panorama's profile: the ground rows cost ~2.6x the sky rows
    cost = np.repeat([1.0, 2.6], 128)
    slabs = balanced_row_slabs(cost, 4)
    parts = [cost[b:b + n].sum() for b, n in slabs]
    assert max(parts) / (cost.sum() / 4) < 1.01
    for bad in ([1.0, -1.0], [np.nan, 1.0]):
        with pytest.raises(ValueError):
            balanced_row_slabs(bad, 1)
    with pytest.raises(ValueError):
        balanced_row_slabs([1.0], 2)
    cfg = RenderConfig(width=4, height=10, spp=1)
    assert slab_config(cfg, 1, 2, [(0, 3), (3, 7)]).row_begin == 3
    for bad in ([(0, 3), (4, 6)], [(0, 3)], [(0, 0), (0, 10)], [(1, 3), (4, 6)]):
        with pytest.raises(ValueError):
            slab_config(cfg, 0, len(bad), bad)


def test_balanced_shards_deal_whole_elevations():
    from sky_cuda.parallel import balanced_shards
    # the sweep's pilot budgets: twilight elevations need up to 16x the samples
    budgets = [992, 1024, 1024, 1024, 1024, 1024, 1024, 672, 352, 192, 160, 128, 96, 96, 96, 96] + [64] * 16
    for world in (1, 2, 4, 8, 32, 40):
        shards = balanced_shards(budgets, world)
        assert len(shards) == world
        assert sorted(i for sh in shards for i in sh) == list(range(len(budgets)))
        assert all(sh == sorted(sh) for sh in shards)
        loads = [sum(budgets[i] for i in sh) for sh in shards]
        # LPT: within 4/3 of the lower bound on the optimum
        assert max(loads) <= 4.0 / 3.0 * max(max(budgets), sum(budgets) / world) + 1e-9
    loads8 = [sum(budgets[i] for i in sh) for sh in balanced_shards(budgets, 8)]
    assert sum(budgets) / (8 * max(loads8)) > 0.95
    with pytest.raises(ValueError):
        balanced_shards([1.0, -2.0], 2)
