"""One process per GPU: partitioning of independent work and rank reductions.

The hot path has no data exchange: FFA searches of different series and
pruning runs from different reference segments (``prune.py:855-930``) are
independent. Ranks therefore only split the work and, for timing, agree on
the slowest rank. Works with any torch.distributed backend (NCCL on GPUs,
gloo on CPUs).
"""

from __future__ import annotations

import torch


def shard(items: list, rank: int, world: int) -> list:
    """Round-robin share of ``items`` for ``rank`` of ``world`` (every item
    goes to exactly one rank; shares differ in size by at most one)."""
    if world < 1 or not 0 <= rank < world:
        msg = f"bad rank {rank} of world {world}"
        raise ValueError(msg)
    return list(items[rank::world])


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """The maximum of ``value`` over all ranks (the value itself without a
    process group)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, dist=None, device=None) -> float:
    """The sum of ``value`` over all ranks (e.g. leaves or trials processed)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
