"""Replica-parallel host logic for several GPUs.

The J-VIE path shards over independent units (bodies, excitations,
frequencies) with no exchange inside a solve, so N GPUs run N replicas: each
rank takes its share of the units, solves them on its own GPU, and the host
only gathers results and times.  No collective touches the data path.
"""
from __future__ import annotations

import os
import socket
import subprocess
import sys
from typing import Callable, List, Sequence


def dist_env():
    """(world, rank, local_rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def under_launcher() -> bool:
    """True inside a process started by torch.distributed.run."""
    return "WORLD_SIZE" in os.environ and "RANK" in os.environ


def free_port() -> int:
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def relaunch(nproc: int, script: str, argv: Sequence[str], env=None) -> int:
    """Runs `script argv` as nproc processes of one node under
    torch.distributed.run (rendezvous on 127.0.0.1), waits for them and returns
    the launcher's exit code.  Rank r sees RANK / LOCAL_RANK = r and
    WORLD_SIZE = nproc, so it takes GPU r and its share of the units."""
    if nproc < 1:
        raise ValueError("nproc must be >= 1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={nproc}",
           "--master-addr=127.0.0.1", f"--master-port={free_port()}", str(script), *argv]
    return subprocess.call(cmd, env=env)


def init(backend: str) -> tuple:
    """Joins the process group of a launched run ('nccl' on GPUs, 'gloo' on the
    host); returns (world, rank, local_rank).  A single process needs none."""
    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        if not dist.is_initialized():
            dist.init_process_group(backend)
    return world, rank, local


def finish(world: int) -> None:
    if world > 1:
        import torch.distributed as dist

        if dist.is_initialized():
            dist.destroy_process_group()


def barrier(world: int) -> None:
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


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
