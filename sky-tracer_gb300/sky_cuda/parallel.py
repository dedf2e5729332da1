"""Multi-GPU split of one render into pixel-row slabs, and of a sweep into
whole elevations.

Every chain is independent, so the tracer has no exchange step.  The
reference dispatches workgroups over (x, y, band) of one image
(integrator.rs:252-283); here one render is cut into contiguous pixel-row
slabs, one per rank (SkyRenderConfig.row_begin / row_count).  Each rank
writes a disjoint slab of the film, and rank 0 concatenates the slabs in row
order.  Pixels keep their whole-image index in the random-number counter, so
the concatenation is the whole render: bit-identical with the plain kernel,
equal to FP64 rounding of the cell sums with the wavefront kernel.  The
reference's sweep is a loop over elevations
(scripts/bake_skyview_elevations.ps1:16-35); a sweep is dealt out in whole
elevations, by sample budget (balanced_shards), or in contiguous blocks
(elevation_shard).

Rows do not cost the same: on a panorama the rows below the horizon (camera
rays that reach the ground, then ground NEE and continuations) cost about 2.6
times the sky rows, so equal-row slabs leave the sky ranks idle.
balanced_row_slabs() cuts the rows into contiguous slabs of equal estimated
cost instead, from per-row costs that pilot_row_costs() times on one GPU with
a short render; rank 0 runs the pilot and broadcasts the slabs
(broadcast_slabs), so every rank uses the same partition.

The only collectives are the slab broadcast, the timing barrier, a
max-reduction of elapsed time and the final gather of slabs to rank 0: none on
the data path.  Any torch.distributed backend works (NCCL on GPUs, gloo on
CPU).
"""

from __future__ import annotations

from dataclasses import replace

import numpy as np


def row_slabs(height: int, world: int) -> list[tuple[int, int]]:
    """Contiguous (row_begin, row_count) of every rank: the rows split as
    evenly as possible, the first height % world ranks one row more."""
    if world < 1:
        raise ValueError(f"world size must be positive, got {world}")
    if height < world:
        raise ValueError(f"{height} rows cannot give each of {world} ranks a row")
    base, extra = divmod(height, world)
    slabs, begin = [], 0
    for r in range(world):
        n = base + (1 if r < extra else 0)
        slabs.append((begin, n))
        begin += n
    return slabs


def balanced_row_slabs(row_cost, world: int) -> list[tuple[int, int]]:
    """Contiguous (row_begin, row_count) of every rank, each at least one row,
    that minimise the largest slab cost (the sum of its rows' costs): the
    bottleneck is bisected with a greedy packing, then slabs are split (the
    longest first) until there is one per rank."""
    c = np.asarray(row_cost, dtype=np.float64).reshape(-1)
    height = c.size
    if world < 1:
        raise ValueError(f"world size must be positive, got {world}")
    if height < world:
        raise ValueError(f"{height} rows cannot give each of {world} ranks a row")
    if not np.all(np.isfinite(c)) or np.any(c < 0.0):
        raise ValueError("row costs must be finite and non-negative")

    def pack(limit):
        slabs, begin, acc = [], 0, 0.0
        for y in range(height):
            if y > begin and acc + c[y] > limit:
                slabs.append((begin, y - begin))
                begin, acc = y, 0.0
            acc += c[y]
        slabs.append((begin, height - begin))
        return slabs

    lo, hi = max(float(c.max()), float(c.sum()) / world), float(c.sum())
    for _ in range(100):
        if hi - lo <= 1e-12 * max(hi, 1e-300):
            break
        mid = 0.5 * (lo + hi)
        if len(pack(mid)) <= world:
            hi = mid
        else:
            lo = mid
    slabs = pack(hi)
    while len(slabs) < world:  # splitting a slab never raises the largest cost
        i = max(range(len(slabs)), key=lambda k: slabs[k][1])
        b, n = slabs[i]
        slabs[i:i + 1] = [(b, n // 2), (b + n // 2, n - n // 2)]
    return slabs


def slab_config(cfg, rank: int, world: int, slabs=None):
    """The rows of `cfg` (a RenderConfig of the whole image) that `rank`
    renders: slab `rank` of `slabs` (e.g. balanced_row_slabs()), or of the
    equal-row split."""
    if not 0 <= rank < world:
        raise ValueError(f"bad rank {rank} of {world}")
    if cfg.row_count or cfg.row_begin:
        raise ValueError("slab_config splits a whole-image config")
    slabs = row_slabs(cfg.height, world) if slabs is None else [tuple(map(int, t)) for t in slabs]
    if len(slabs) != world or slabs[0][0] != 0 or sum(n for _, n in slabs) != cfg.height or \
            any(n < 1 for _, n in slabs) or any(b1 != b0 + n0 for (b0, n0), (b1, _) in zip(slabs, slabs[1:])):
        raise ValueError("slabs must be one contiguous, non-empty row range per rank covering the image")
    begin, count = slabs[rank]
    return replace(cfg, row_begin=begin, row_count=count)


def pilot_row_costs(gs, cfg, blocks: int = 16, spp: int = 32, stream=None) -> np.ndarray:
    """Per-row cost of `cfg` on this GPU: blocks of rows rendered at `spp`
    samples, each timed with CUDA events on `stream` (after one untimed
    render of the first block), its time spread evenly over its rows."""
    import torch
    stream = stream or torch.cuda.current_stream()
    pilot = replace(cfg, spp=spp, row_begin=0, row_count=0, flags=0, sample_offset=0)
    parts = row_slabs(cfg.height, min(blocks, cfg.height))
    most = max(n for _, n in parts) * cfg.width * gs.band_count
    s = torch.zeros(most, dtype=torch.float64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    outs = {"cell_sum": s.data_ptr(), "status": status.data_ptr()}
    gs.render_device(replace(pilot, row_begin=parts[0][0], row_count=parts[0][1]), outs, stream.cuda_stream)
    cost = np.empty(cfg.height)
    for b, n in parts:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        gs.render_device(replace(pilot, row_begin=b, row_count=n), outs, stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
        cost[b:b + n] = e0.elapsed_time(e1) / n
    if int(status.item()):
        raise RuntimeError("the pilot render tripped the path watchdog")
    return cost


def broadcast_object(obj):
    """Rank 0's `obj` on every rank (unchanged without a process group)."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return obj
    box = [obj if dist.get_rank() == 0 else None]
    dist.broadcast_object_list(box, src=0)
    return box[0]


def broadcast_slabs(slabs):
    """Rank 0's slabs, [(row_begin, row_count), ...], on every rank."""
    out = broadcast_object(slabs)
    return None if out is None else [tuple(int(v) for v in t) for t in out]


def elevation_shard(count: int, rank: int, world: int) -> range:
    """Contiguous block of whole elevations (indices into a sweep's list) of `rank`."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"bad rank {rank} of {world}")
    base, extra = divmod(count, world)
    begin = rank * base + min(rank, extra)
    return range(begin, begin + base + (1 if rank < extra else 0))


def balanced_shards(costs, world: int) -> list[list[int]]:
    """Whole items (e.g. a sweep's elevations) of the given costs dealt to
    `world` ranks, largest first to the least loaded rank (the LPT rule: the
    largest load is at most 4/3 of the optimum); each rank's indices in
    ascending order."""
    c = np.asarray(costs, dtype=np.float64).reshape(-1)
    if world < 1:
        raise ValueError(f"world size must be positive, got {world}")
    if not np.all(np.isfinite(c)) or np.any(c < 0.0):
        raise ValueError("costs must be finite and non-negative")
    load = [0.0] * world
    shards = [[] for _ in range(world)]
    for i in sorted(range(c.size), key=lambda k: (-c[k], k)):
        r = min(range(world), key=lambda k: (load[k], k))
        shards[r].append(i)
        load[r] += c[i]
    return [sorted(sh) for sh in shards]


def concat_slabs(slabs, width: int, channels: int) -> np.ndarray:
    """Join per-rank slabs (each [rows * width * channels] or [rows * width,
    channels], pixel-major from its first row) in rank order into the whole
    image's [pixels, channels] array."""
    parts = [np.asarray(s).reshape(-1, channels) for s in slabs]
    for p in parts:
        if p.shape[0] % width:
            raise ValueError("a slab does not hold whole rows")
    return np.concatenate(parts, axis=0)


def max_over_ranks(value: float, device=None) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_to_rank0(obj):
    """All ranks' objects on rank 0 (list in rank order), None elsewhere."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return [obj]
    out = [None] * dist.get_world_size() if dist.get_rank() == 0 else None
    dist.gather_object(obj, out, dst=0)
    return out


def render_split(render_slab, cfg, rank: int, world: int, channels: int, slabs=None):
    """Render rank's slab of `cfg` with render_slab(slab_cfg) -> array of the
    slab ([slab pixels, channels] or flat) and join all slabs on rank 0.
    Returns the whole image's [pixels, channels] on rank 0, None elsewhere."""
    part = np.asarray(render_slab(slab_config(cfg, rank, world, slabs)))
    parts = gather_to_rank0(part)
    if parts is None:
        return None
    return concat_slabs(parts, cfg.width, channels)
