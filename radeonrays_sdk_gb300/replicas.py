"""Replica sharding for more than one GPU.

Rays are independent, so N GPUs each hold a full copy of the BVH and trace a
contiguous shard of the rays; hits are written in place and need no exchange.
The helpers below define the shard of a rank and (for callers that want all
hits on one rank) gather the shards back in ray order.
"""
from __future__ import annotations


def shard(n: int, rank: int, world: int) -> tuple[int, int]:
    """[begin, end) of rank's contiguous shard of n units (sizes differ by at most one)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    q, r = divmod(n, world)
    begin = rank * q + min(rank, r)
    return begin, begin + q + (1 if rank < r else 0)


def gather_shards(local, n: int, rank: int, world: int, group=None):
    """All-gather per-rank hit arrays (torch tensors, first dim = rays of the
    shard) into one tensor in ray order; every rank receives the result."""
    import torch
    import torch.distributed as dist

    sizes = [shard(n, r, world)[1] - shard(n, r, world)[0] for r in range(world)]
    width = max(sizes)
    pad = torch.zeros((width,) + tuple(local.shape[1:]), dtype=local.dtype, device=local.device)
    pad[: local.shape[0]] = local
    parts = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad, group=group)
    return torch.cat([p[:s] for p, s in zip(parts, sizes)], dim=0)
