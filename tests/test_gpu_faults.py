"""Failure handling on the device path, with every failure made on the host
(no kernel is made to fault, trap or hang): non-convergence is a flag,
non-finite inputs and allocation failures are error statuses, a bounded
device wait that runs out is a status, and the library stays usable
afterwards."""
import numpy as np
import pytest

from oracle import vie_oracle as vo

pytestmark = pytest.mark.gpu
FREQ = 298e6


def sphere(L=8, dx=5e-3, R=0.018):
    r = vo.grid(L, L, L, dx)
    er = np.ones((L, L, L), complex)
    er[np.sum(r * r, axis=3) < R**2] = 50 - 30j
    em = vo.EMconstants(FREQ)
    E, _ = vo.PlaneWave_Excitation(r, [0, 0, em["ko"]], em["omega_mu"], [1, 0, 0])
    return r, np.asfortranarray(er), np.asfortranarray(E)


def test_non_convergence_is_a_flag_not_an_error():
    import marie_gb300 as mg

    r, er, E = sphere()
    op = mg.Operator.assemble(8, 8, 8, 5e-3, FREQ)
    Je, flag, relres, it, resvec, _ = mg.JVIE_Solver(E, er, r, FREQ, op, tol=1e-12, inner_it=2, outer_it=1, solver="G")
    assert flag == 1 and relres > 1e-12
    assert it == [2, 1] and len(resvec) == 3


def test_non_finite_input_is_reported_and_library_recovers():
    import marie_gb300 as mg

    r, er, E = sphere()
    op = mg.Operator.assemble(8, 8, 8, 5e-3, FREQ)
    Ebad = E.copy(order="F")
    Ebad[3, 3, 3, 0] = np.nan
    with pytest.raises(mg.MarieError, match="non-finite"):
        mg.JVIE_Solver(Ebad, er, r, FREQ, op, tol=1e-8, solver="G")
    out = mg.JVIE_Solver(E, er, r, FREQ, op, tol=1e-8, solver="G")
    assert out[1] == 0


def test_air_only_and_zero_excitation():
    import marie_gb300 as mg

    r, er, E = sphere()
    op = mg.Operator.assemble(8, 8, 8, 5e-3, FREQ)
    air = np.ones_like(er)
    Je, flag, relres, *_ = mg.JVIE_Solver(E, air, r, FREQ, op, tol=1e-8, solver="G")
    assert flag == 0 and not np.any(Je)
    Je, flag, relres, *_ = mg.JVIE_Solver(np.zeros_like(E), er, r, FREQ, op, tol=1e-8, solver="G")
    assert flag == 0 and relres == 0 and not np.any(Je)


@pytest.mark.parametrize("nth", [1, 3, 6, 12])
def test_allocation_failure_is_enomem_and_plan_stays_usable(nth):
    """An allocation failure (injected on the host at the nth device allocation
    of the solve) surfaces as MARIE_ENOMEM; the next solve succeeds."""
    import marie_gb300 as mg

    r, er, E = sphere()
    op = mg.Operator.assemble(8, 8, 8, 5e-3, FREQ)
    lib = mg.load()
    lib.marie_inject_alloc_failure(nth)
    try:
        with pytest.raises(mg.MarieError) as ei:
            mg.JVIE_Solver(E, er, r, FREQ, op, tol=1e-8, solver="G")
        assert ei.value.code == -2
    finally:
        lib.marie_inject_alloc_failure(0)
    out = mg.JVIE_Solver(E, er, r, FREQ, op, tol=1e-8, solver="G")
    assert out[1] == 0


@pytest.mark.parametrize("solver", ["B", "D"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_other_solvers_flags_zero_rhs_and_allocation_failures(solver, precision):
    """Solvers 'B' (bicgstab) and 'D' (pgmresDR): non-convergence is a flag, a
    zero excitation gives J = 0, injected allocation failures are MARIE_ENOMEM
    and the plan solves afterwards."""
    import marie_gb300 as mg

    r, er, E = sphere()
    op = mg.Operator.assemble(8, 8, 8, 5e-3, FREQ, precision=precision)
    kw = dict(max_it=1) if solver == "B" else dict(inner_it=3, outer_it=1)
    Je, flag, relres, it, resvec, _ = mg.JVIE_Solver(E, er, r, FREQ, op, tol=1e-12, solver=solver, **kw)
    if precision == "fp64":
        # the solver's own iteration limit ends it (the mixed refinement repeats
        # the limited inner solve and may still converge)
        assert flag != 0 and relres > 1e-12
    assert np.isfinite(relres) and (flag == 0) == (relres <= 1e-12)
    Je, flag, relres, *_ = mg.JVIE_Solver(np.zeros_like(E), er, r, FREQ, op, tol=1e-8, solver=solver)
    assert flag == 0 and relres == 0 and not np.any(Je)
    lib = mg.load()
    for nth in (1, 4, 9):
        lib.marie_inject_alloc_failure(nth)
        try:
            with pytest.raises(mg.MarieError) as ei:
                mg.JVIE_Solver(E, er, r, FREQ, op, tol=1e-8, solver=solver)
            assert ei.value.code == -2
        finally:
            lib.marie_inject_alloc_failure(0)
    out = mg.JVIE_Solver(E, er, r, FREQ, op, tol=1e-8, solver=solver)
    assert out[1] == 0 and out[2] <= 1e-8


def test_bounded_tile_wait_that_runs_out_is_a_status():
    """The z pass waits for its bulk tile copy with a time limit.  Armed (on
    the host) for more bytes than the copy delivers, the wait runs out after
    5 ms, the pass sets the plan's status word and finishes, mv_AN returns
    MARIE_ETIMEOUT, and the next product is right again."""
    import marie_gb300 as mg

    L = 16
    r, er, E = sphere(L=L, dx=2.5e-3, R=0.012)
    S = vo.jvie_setup(E, er, r, FREQ, 2)
    op = mg.Operator.assemble(L, L, L, 2.5e-3, FREQ, precision="mixed")
    rng = np.random.default_rng(5)
    n = S["idxS3"].size
    J = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    args = (S["Mr"], S["Mc"], S["Gram"], "notransp", S["idxS3"])
    ref = mg.mv_AN(J, op, *args, precision="fp32")
    lib = mg.load()
    lib.marie_inject_tile_timeout(1)
    try:
        with pytest.raises(mg.MarieError) as ei:
            mg.mv_AN(J, op, *args, precision="fp32")
        assert ei.value.code == -6
    finally:
        lib.marie_inject_tile_timeout(0)
    again = mg.mv_AN(J, op, *args, precision="fp32")
    assert np.array_equal(again, ref)
    op.close()


def test_release_cached_memory(cuda):
    """The pool's cached blocks go back to the device and later calls still work."""
    import torch

    import marie_gb300 as mg

    L, dx = 16, 5e-3
    r = vo.grid(L, L, L, dx)
    er = np.ones((L, L, L), complex)
    er[np.sum(r * r, axis=3) < 0.035**2] = 50 - 30j
    er = np.asfortranarray(er)
    em = vo.EMconstants(298e6)
    E, _ = vo.PlaneWave_Excitation(r, [0, 0, em["ko"]], em["omega_mu"], [1, 0, 0])
    op = mg.Operator.assemble(L, L, L, dx, 298e6, precision="mixed")
    J1 = mg.JVIE_Solver(np.asfortranarray(E), er, r, 298e6, op, tol=1e-6, solver="G")[0]
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    mg.release_cached_memory()
    assert torch.cuda.mem_get_info()[0] >= free0
    J2 = mg.JVIE_Solver(np.asfortranarray(E), er, r, 298e6, op, tol=1e-6, solver="G")[0]
    assert np.array_equal(J1, J2)
