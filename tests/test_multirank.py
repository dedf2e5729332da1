"""World-size-2 gloo ranks on CPU: sharding of sweep jobs across ranks, the
max-over-ranks timing reduction and the gather of per-rank results."""

import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "sky-tracer_gb300"))
    import torch.distributed as dist
    from sky_cuda.parallel import gather_to_rank0, max_over_ranks, shard
    from sky_cuda.sweep import elevation_schedule
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    mine = shard(list(elevation_schedule(32)), rank, world)
    t = max_over_ranks(1.0 + rank)
    got = gather_to_rank0(mine)
    if rank == 0:
        q.put((t, got))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sharding_and_timing():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    t, got = q.get()
    assert t == 2.0
    from sky_cuda.sweep import elevation_schedule
    flat = sorted(x for part in got for x in part)
    assert flat == sorted(elevation_schedule(32))
    assert not set(got[0]) & set(got[1])


def test_shard_rejects_bad_ranks():
    from sky_cuda.parallel import shard
    assert shard(range(5), 1, 2) == [1, 3]
    with pytest.raises(ValueError):
        shard(range(5), 2, 2)
