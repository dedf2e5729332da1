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
(scripts/bake_skyview_elevations.ps1:16-35); a sweep is cut into contiguous
blocks of whole elevations.

The only collectives are the timing barrier, a max-reduction of elapsed time
and the final gather of slabs to rank 0: none on the data path.  Any
torch.distributed backend works (NCCL on GPUs, gloo on CPU).
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


def slab_config(cfg, rank: int, world: int):
    """The rows of `cfg` (a RenderConfig of the whole image) that `rank` renders."""
    if not 0 <= rank < world:
        raise ValueError(f"bad rank {rank} of {world}")
    if cfg.row_count or cfg.row_begin:
        raise ValueError("slab_config splits a whole-image config")
    begin, count = row_slabs(cfg.height, world)[rank]
    return replace(cfg, row_begin=begin, row_count=count)


def elevation_shard(count: int, rank: int, world: int) -> range:
    """Contiguous block of whole elevations (indices into a sweep's list) of `rank`."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"bad rank {rank} of {world}")
    base, extra = divmod(count, world)
    begin = rank * base + min(rank, extra)
    return range(begin, begin + base + (1 if rank < extra else 0))


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


def render_split(render_slab, cfg, rank: int, world: int, channels: int):
    """Render rank's slab of `cfg` with render_slab(slab_cfg) -> array of the
    slab ([slab pixels, channels] or flat) and join all slabs on rank 0.
    Returns the whole image's [pixels, channels] on rank 0, None elsewhere."""
    part = np.asarray(render_slab(slab_config(cfg, rank, world)))
    parts = gather_to_rank0(part)
    if parts is None:
        return None
    return concat_slabs(parts, cfg.width, channels)
