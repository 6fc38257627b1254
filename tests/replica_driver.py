"""Test driver for the replica launcher that bench.py uses (no GPU): run with
--gpus N, it re-runs itself as N processes under torch.distributed.run
(replicas.relaunch), each rank joins a gloo group (replicas.init), solves its
shard of 16 excitations and 3 bodies with a host stand-in for the solve, and
rank 0 prints one JSON line with the gathered units and the maximum time over
ranks, as bench.py's c3 path reports them."""
import argparse
import json
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

from marie_gb300 import replicas  # noqa: E402


def host_solve(unit):
    """Stand-in for one excitation solve: a deterministic function of the unit."""
    kind, i = unit
    t0 = time.perf_counter()
    acc = sum((i + 1) * k for k in range(1000))
    return {"kind": kind, "unit": i, "value": acc, "seconds": time.perf_counter() - t0}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    args = ap.parse_args()
    if args.gpus > 1 and not replicas.under_launcher():
        sys.exit(replicas.relaunch(args.gpus, __file__, sys.argv[1:]))
    world, rank, _ = replicas.init("gloo")
    units = [("excitation", e) for e in range(16)] + [("body", b) for b in range(3)]
    t0 = time.perf_counter()
    results = replicas.run_sharded(units, host_solve, rank, world)
    elapsed = replicas.max_over_ranks(time.perf_counter() - t0, world)
    owners = replicas.gather_results([(u, rank) for u in replicas.shard(len(units), rank, world)], world)
    if rank == 0:
        print(json.dumps({"n_gpus": world, "seconds_max": elapsed, "results": results,
                          "owners": [[u, r] for u, r in owners]}))
    replicas.finish(world)


if __name__ == "__main__":
    main()
