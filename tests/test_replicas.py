"""Multi-process (gloo, world size 2) tests of the replica sharding used for N
GPUs: every unit is solved exactly once, results come back in order, and the
timing reduction takes the maximum over ranks.  No GPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from marie_gb300 import replicas


def test_shard_covers_every_unit_once():
    for n in (0, 1, 5, 16, 17):
        for world in (1, 2, 3, 8):
            got = [i for r in range(world) for i in replicas.shard(n, r, world)]
            assert got == list(range(n))
            sizes = [len(replicas.shard(n, r, world)) for r in range(world)]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        replicas.shard(4, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        units = [(e, 0.1 * e) for e in range(7)]  # (excitation id, payload)
        res = replicas.run_sharded(units, lambda u: (u[0], u[1] * 2.0, rank), rank, world)
        t = replicas.max_over_ranks(1.0 + rank, world)
        q.put((rank, res, t))
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo_sharding():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, res, t in out:
        assert [u for u, _, _ in res] == list(range(7))
        assert all(abs(v - 0.2 * u) < 1e-12 for u, v, _ in res)
        owners = [r for _, _, r in res]
        assert owners == [0, 0, 0, 0, 1, 1, 1]
        assert t == 2.0


def test_launcher_runs_two_gloo_ranks_end_to_end():
    """The launcher bench.py uses (--gpus 2 outside torchrun re-runs the script
    as two ranks): every unit solved exactly once, results in unit order, the
    work split between the two ranks, n_gpus reported as 2."""
    import json
    import subprocess
    import sys
    from pathlib import Path

    drv = Path(__file__).resolve().parent / "replica_driver.py"
    env = dict(os.environ, OMP_NUM_THREADS="1")
    p = subprocess.run([sys.executable, str(drv), "--gpus", "2"], capture_output=True, text=True, timeout=300,
                       env=env)
    assert p.returncode == 0, p.stderr[-2000:]
    line = [l for l in p.stdout.splitlines() if l.startswith("{")][-1]
    out = json.loads(line)
    assert out["n_gpus"] == 2
    got = [(r["kind"], r["unit"]) for r in out["results"]]
    want = [("excitation", e) for e in range(16)] + [("body", b) for b in range(3)]
    assert got == want
    assert all(r["value"] == (r["unit"] + 1) * 499500 for r in out["results"])
    owners = [r for _, r in out["owners"]]
    assert sorted(set(owners)) == [0, 1] and abs(owners.count(0) - owners.count(1)) <= 1
    assert out["seconds_max"] >= 0
