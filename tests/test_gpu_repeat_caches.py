"""Run-to-run determinism of the device path (every reduction is two-stage in
a fixed order, no floating-point atomics), and the on-device side of the
operator cache, the schedule cache and the solve log."""
import json

import numpy as np
import pytest

from oracle import vie_oracle as vo

pytestmark = pytest.mark.gpu
FREQ = 298e6
L, DX = 32, 4e-3


def sphere(L=L, dx=DX, radius=0.05):
    r = vo.grid(L, L, L, dx)
    er = np.ones((L, L, L), complex)
    er[np.sum(r * r, axis=3) < radius**2] = 60.0 - 1j * 0.7 / (vo.EPS0 * 2 * np.pi * FREQ)
    em = vo.EMconstants(FREQ)
    E, _ = vo.PlaneWave_Excitation(r, [0, 0, em["ko"]], em["omega_mu"], [1, 0, 0])
    return r, np.asfortranarray(er), np.asfortranarray(E)


def test_assembly_and_matvecs_repeat_bitwise(cuda):
    import marie_gb300 as mg

    a = mg.Operator.assemble(L, L, L, DX, FREQ, precision="mixed")
    b = mg.Operator.assemble(L, L, L, DX, FREQ, precision="mixed")
    assert np.array_equal(a.to_array(), b.to_array())
    r, er, _ = sphere()
    V = L**3
    idxS = np.flatnonzero(np.abs(er.reshape(-1, order="F") - 1) > 1e-12)
    idx = (np.concatenate([idxS, V + idxS, 2 * V + idxS]) + 1).astype(np.int64)
    Mr = np.asfortranarray(er / er)
    Mc = np.asfortranarray((er - 1) / er)
    rng = np.random.default_rng(5)
    J = rng.standard_normal(idx.size) + 1j * rng.standard_normal(idx.size)
    for prec in ("fp64", "fp32"):
        y1 = mg.mv_AN(J, a, Mr, Mc, DX**3, "notransp", idx, precision=prec)
        y2 = mg.mv_AN(J, a, Mr, Mc, DX**3, "notransp", idx, precision=prec)
        y3 = mg.mv_AN(J, b, Mr, Mc, DX**3, "notransp", idx, precision=prec)
        assert np.array_equal(y1, y2) and np.array_equal(y1, y3)
    a.close()
    b.close()


@pytest.mark.parametrize("precision,solver", [("fp64", "G"), ("fp64", "B"), ("mixed", "G"), ("fp64", "D")])
def test_solves_repeat_bitwise(cuda, precision, solver):
    import marie_gb300 as mg

    r, er, E = sphere()
    op = mg.Operator.assemble(L, L, L, DX, FREQ, precision=precision)
    runs = [mg.JVIE_Solver(E, er, r, FREQ, op, tol=1e-6, solver=solver) for _ in range(2)]
    (J1, f1, rr1, it1, rv1, _), (J2, f2, rr2, it2, rv2, _) = runs
    assert f1 == f2 == 0
    assert it1 == it2 and rr1 == rr2
    assert np.array_equal(rv1, rv2) and np.array_equal(J1, J2)
    op.close()


def test_operator_cache_serves_the_assembled_operator(cuda, tmp_path):
    import marie_gb300 as mg

    r, er, E = sphere()
    dx = float(r[1, 0, 0, 0] - r[0, 0, 0, 0])  # the spacing getOPERATORS reads from r
    cache = mg.OperatorCache(str(tmp_path))
    miss = cache.operator(L, L, L, dx, FREQ, precision="mixed")
    assert len(list(tmp_path.glob("fN_32x32x32_*.npy"))) == 1
    hit = cache.operator(L, L, L, dx, FREQ, precision="mixed")
    assert np.array_equal(miss.to_array(), hit.to_array())
    a = mg.JVIE_Solver(E, er, r, FREQ, miss, tol=1e-6, solver="G")
    b = mg.JVIE_Solver(E, er, r, FREQ, hit, tol=1e-6, solver="G")
    assert a[3] == b[3] and np.array_equal(a[0], b[0])
    # getOPERATORS through the same cache: the stored entry, no new one
    assert np.array_equal(cache.getOPERATORS(r, FREQ), miss.to_array())
    assert len(list(tmp_path.glob("fN_*.npy"))) == 1
    miss.close()
    hit.close()


def test_schedule_cache_tunes_then_pins(cuda, tmp_path):
    import marie_gb300 as mg

    path = tmp_path / "schedules.json"
    op = mg.Operator.assemble(L, L, L, DX, FREQ, precision="mixed")
    s, tuned = mg.ScheduleCache(str(path)).apply(op)
    assert tuned and s is not None
    op2 = mg.Operator.assemble(L, L, L, DX, FREQ, precision="mixed")
    s2, tuned2 = mg.ScheduleCache(str(path)).apply(op2)
    assert s2 == s and not tuned2
    data = json.loads(path.read_text())
    assert list(data.values()) == [list(s)] and list(data)[0].endswith("|64x64x64")
    # an FP64-only plan has no FP32 schedule to tune: nothing is cached
    op3 = mg.Operator.assemble(8, 8, 8, DX, FREQ, precision="fp64")
    assert mg.ScheduleCache(str(path)).apply(op3) == (None, False)
    for o in (op, op2, op3):
        o.close()


def test_solve_log_and_run_record(cuda, tmp_path):
    import marie_gb300 as mg

    r, er, E = sphere()
    op = mg.Operator.assemble(L, L, L, DX, FREQ, precision="mixed")
    log, runs = tmp_path / "solve.log", tmp_path / "runs.jsonl"
    Je, flag, relres, it, resvec, t = mg.JVIE_Solver(E, er, r, FREQ, op, tol=1e-6, solver="G", logfile=str(log),
                                                    runlog=str(runs))
    text = log.read_text()
    ns = int(np.count_nonzero(np.abs(er - 1) > 1e-12))
    assert " Domain:                32x32x32 voxels" in text
    assert " # DOFS in Scatterer:   %d" % (3 * ns) in text
    assert (" GPU GMRES solver (50 restart), wo/ preconditioner Time  = %.2f [sec] for %d iterations, flag 0, "
            % (t, len(resvec))) in text
    rec = json.loads(runs.read_text())
    assert rec["flag"] == flag == 0 and rec["iter"] == it and rec["precision"] == "mixed"
    assert rec["relres"] == relres and rec["resvec_len"] == len(resvec) and rec["dofs_scatterer"] == 3 * ns
    op.close()
