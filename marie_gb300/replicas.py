"""Replica-parallel host logic for several GPUs.

The J-VIE path shards over independent units (bodies, excitations,
frequencies) with no exchange inside a solve, so N GPUs run N replicas: each
rank takes its share of the units, solves them on its own GPU, and the host
only gathers results and times.  No collective touches the data path.
"""
from __future__ import annotations

import os
from typing import Callable, List, Sequence


def dist_env():
    """(world, rank, local_rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard(n_units: int, rank: int, world: int) -> List[int]:
    """Contiguous, balanced block of unit indices owned by `rank`."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(n_units, world)
    start = rank * base + min(rank, extra)
    return list(range(start, start + base + (1 if rank < extra else 0)))


def max_over_ranks(value: float, world: int, device=None) -> float:
    """Maximum of a per-rank float (a timing) over all ranks."""
    if world == 1:
        return value
    import torch
    import torch.distributed as dist

    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_results(local: Sequence, world: int) -> list:
    """All ranks' result lists, concatenated in rank order (host objects)."""
    if world == 1:
        return list(local)
    import torch.distributed as dist

    out = [None] * world
    dist.all_gather_object(out, list(local))
    return [x for part in out for x in part]


def run_sharded(units: Sequence, solve: Callable, rank: int, world: int) -> list:
    """Solve this rank's share of `units` with `solve(unit)`; gather all results."""
    mine = [solve(units[i]) for i in shard(len(units), rank, world)]
    return gather_results(mine, world)
