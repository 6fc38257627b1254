"""Host side of the solve log, the JSON run records and the on-disk caches
(CPU only: formats, file handling, cache keys and misses)."""
import json

import numpy as np
import pytest

from marie_gb300 import opcache, solvelog
from oracle import vie_oracle as vo

FIELDS = dict(L=16, M=12, N=8, dx=5e-3, n_scat=100, freq=298.2e6, fN_bytes=32 * 24 * 16 * 6 * 16, solver="G",
              precond="", inner_it=50, ritz=5, solvert=1.234, resvec=[1.0, 0.5, 1e-7], flag=0, relres=9.5e-7,
              elapsed=2.5)


def test_solve_log_lines_follow_the_reference_formats():
    text = solvelog.format_solve_log(**FIELDS)
    lines = text.split("\n")
    assert " Domain:                16x12x8 voxels" in lines
    assert " Resolution:            5.00mm" in lines
    assert " # DOFS:                %d" % (3 * 16 * 12 * 8) in lines
    assert " # DOFS in Scatterer:   300" in lines
    assert " Operating Frequency:   298.20 MHz" in lines
    assert " Estimated MVP Peak Memory %.3f MB." % (4 * FIELDS["fN_bytes"] / 1048576) in lines
    assert (" GPU GMRES solver (50 restart), wo/ preconditioner Time  = 1.23 [sec] for 3 iterations, flag 0, "
            "residue 1e-07, relative residue 9.5e-07 ") in lines
    assert " VIE Solve finished. Elapsed Time  = 2.50 [sec] " in lines


@pytest.mark.parametrize("solver,precond,expect", [
    ("G", "R", " GPU GMRES solver (50 restart), w/ Right preconditioner"),
    ("G", "L", " GPU GMRES solver (50 restart), w/ Left preconditioner"),
    ("D", "", " GPU GMRES solver (50 restart, deflated 5), wo/ preconditioner "),
    ("D", "R", " GPU GMRES solver (50 restart, deflated 5), w/ Right preconditioner "),
    ("B", "", " GPU BICGSTAB solver, wo/ preconditioner"),
    ("B", "L", " GPU BICGSTAB solver, w/ preconditioner"),
])
def test_solver_line_per_solver(solver, precond, expect):
    text = solvelog.format_solve_log(**dict(FIELDS, solver=solver, precond=precond))
    assert any(line.startswith(expect) for line in text.split("\n"))


def test_log_destinations(tmp_path, capsys):
    log = tmp_path / "solve.log"
    solvelog.write_solve_log(str(log), **FIELDS)
    solvelog.write_solve_log(str(log), **FIELDS)
    assert log.read_text() == 2 * solvelog.format_solve_log(**FIELDS)  # appended, as fopen(logfile, 'a')
    solvelog.write_solve_log(None, **FIELDS)
    assert capsys.readouterr().out == ""
    solvelog.write_solve_log(1, **FIELDS)
    assert capsys.readouterr().out == solvelog.format_solve_log(**FIELDS)
    solvelog.write_solve_log(str(tmp_path), **FIELDS)  # a directory cannot be opened: falls back to fid 1
    assert "Domain:" in capsys.readouterr().out
    solvelog.write_overall_log(str(log), 3.0)
    assert "Overall Scattering Problem:      \tElapsed time  = 3.00 [sec]" in log.read_text()


def test_run_records_are_json_lines(tmp_path):
    path = tmp_path / "runs.jsonl"
    rec = solvelog.run_record(16, 12, 8, 5e-3, 100, 298e6, "G", "", "mixed", 1e-6, 50, 200, 1000, 0, 9.5e-7,
                              [12, 2], [1.0, 0.5, 1e-7], 0.2, 0.3)
    solvelog.write_run_record(str(path), rec)
    solvelog.write_run_record(str(path), dict(rec, flag=1))
    solvelog.write_run_record(None, rec)
    rows = [json.loads(line) for line in path.read_text().splitlines()]
    assert len(rows) == 2 and rows[0] == rec and rows[1]["flag"] == 1
    assert rows[0]["dofs"] == 3 * 16 * 12 * 8 and rows[0]["dofs_scatterer"] == 300 and rows[0]["iter"] == [12, 2]
    assert rows[0]["precond"] is None
    assert solvelog.run_record(4, 4, 4, 1e-3, 1, 1e8, "B", "L", "fp64", 1e-3, 50, 200, 1000, 0, 1e-4, 3.5, [1.0],
                               0.1, 0.1)["iter"] == 3.5


def test_operator_cache_round_trip_and_misses(tmp_path):
    cache = opcache.OperatorCache(str(tmp_path / "ops"))
    key = opcache.operator_key(3, 2, 2, 5e-3, 298e6)
    rng = np.random.default_rng(0)
    arr = np.asfortranarray(rng.standard_normal((6, 4, 4, 6)) + 1j * rng.standard_normal((6, 4, 4, 6)))
    assert cache.load(key) is None
    cache.store(key, arr)
    back = cache.load(key)
    assert back.flags.f_contiguous and np.array_equal(back, arr)
    # a different frequency, dx, singular method or operator is another entry
    assert cache.load(opcache.operator_key(3, 2, 2, 5e-3, 298e6 + 1)) is None
    assert cache.load(opcache.operator_key(3, 2, 2, 5e-3 * (1 + 1e-15), 298e6)) is None
    assert cache.load(opcache.operator_key(3, 2, 2, 5e-3, 298e6, singular="other")) is None
    assert cache.load(opcache.operator_key(3, 2, 2, 5e-3, 298e6, op="K")) is None
    with pytest.raises(ValueError):
        cache.store(key, arr[:, :, :, :3])
    with pytest.raises(ValueError):
        opcache.operator_key(3, 2, 2, 5e-3, 298e6, op="L")
    # a damaged array or key file reads as a miss
    arr_path, key_path = cache._paths(key)
    with open(arr_path, "r+b") as fh:
        fh.truncate(100)
    assert cache.load(key) is None
    cache.store(key, arr)
    with open(key_path, "w") as fh:
        fh.write('{"op": "N"}')
    assert cache.load(key) is None
    assert not [p for p in (tmp_path / "ops").iterdir() if p.name.startswith(".tmp-")]


def test_cached_getOPERATORS_hit_reads_the_disk(tmp_path):
    # a hit never reaches the device: the entry stored here is what comes back
    r = vo.grid(4, 4, 4, 5e-3)
    rng = np.random.default_rng(1)
    fN = np.asfortranarray(rng.standard_normal((8, 8, 8, 6)) + 1j * rng.standard_normal((8, 8, 8, 6)))
    cache = opcache.OperatorCache(str(tmp_path))
    cache.store(opcache.operator_key(4, 4, 4, float(r[1, 0, 0, 0] - r[0, 0, 0, 0]), 298e6), fN)
    out = cache.getOPERATORS(r, 298e6)
    assert np.array_equal(out, fN)


class _FakeOperator:
    def __init__(self, L, M, N):
        self.L, self.M, self.N = L, M, N
        self.calls = []

    def autotune(self):
        self.calls.append("autotune")
        return (1, 0, 2), [(1, 0, 2, 0.5)]

    def set_schedule(self, fuse, fvar, zvar):
        self.calls.append(("set", fuse, fvar, zvar))
        return self


def test_schedule_cache_tunes_once_per_device_and_grid(tmp_path):
    cache = opcache.ScheduleCache(str(tmp_path / "sched" / "schedules.json"))
    a = _FakeOperator(64, 64, 64)
    assert cache.apply(a, device="GPU-A") == ((1, 0, 2), True) and a.calls == ["autotune"]
    b = _FakeOperator(64, 64, 64)
    assert cache.apply(b, device="GPU-A") == ((1, 0, 2), False) and b.calls == [("set", 1, 0, 2)]
    c = _FakeOperator(64, 64, 64)
    assert cache.apply(c, device="GPU-B")[1] is True
    d = _FakeOperator(64, 64, 32)
    assert cache.apply(d, device="GPU-A")[1] is True
    data = json.loads((tmp_path / "sched" / "schedules.json").read_text())
    assert set(data) == {"GPU-A|128x128x128", "GPU-B|128x128x128", "GPU-A|128x128x64"}
    e = _FakeOperator(32, 32, 32)
    e.autotune = lambda: ((0, 0, 0), [])  # an FP64-only plan: nothing timed, nothing cached
    assert cache.apply(e, device="GPU-A") == (None, False)
    assert "GPU-A|64x64x64" not in json.loads((tmp_path / "sched" / "schedules.json").read_text())
    (tmp_path / "sched" / "schedules.json").write_text("not json")
    assert cache.get("GPU-A|128x128x128") is None
