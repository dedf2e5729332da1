"""Multi-GPU helpers: independent frames or sweep jobs per rank.

The tracer has no exchange step (every chain is independent), so N GPUs run
N disjoint shards; the only collectives are a barrier and a max-reduction of
elapsed times for timing, and an optional gather of per-rank results to rank
0.  Works with any torch.distributed backend (NCCL on GPUs, gloo on CPU).
"""

from __future__ import annotations


def shard(items, rank: int, world: int) -> list:
    """Round-robin shard of `items` for `rank` of `world` (disjoint, covering)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"bad rank {rank} of {world}")
    return list(items)[rank::world]


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
