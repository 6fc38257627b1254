"""GPU parity of the solver variants of JVIE_Solver against their oracle
restatements: bicgstab (solver 'B', the reference's default, a MATLAB
built-in) and pgmresDR (solver 'D', pgmresDR.m / pgmresDR_iter.m /
getHarmVecs1.m / getHarmVecs2.m), through the function-handle entry points and
through JVIE_Solver, in FP64 and in the mixed-precision refinement."""
import numpy as np
import pytest

from oracle import vie_oracle as vo

pytestmark = pytest.mark.gpu
FREQ = 298e6


def dense(n, seed):
    """Well-conditioned (spectrum in a disk of radius ~1.1 around 3): BiCGSTAB
    converges in ~20 steps and rounding cannot change its decisions."""
    rng = np.random.default_rng(seed)
    A = np.eye(n) * 3 + 0.1 * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    return A, b


def hard_dense(n, seed):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    lam = np.concatenate([[0.01, 0.02, 0.05], np.linspace(1, 4, n - 3)]) * np.exp(0.3j * rng.random(n))
    A = Q @ np.diag(lam) @ Q.conj().T + 0.01 * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    return A, b


@pytest.mark.parametrize("case", ["plain", "M1", "M1M2", "x0", "maxit"])
def test_bicgstab_handles_match_oracle(case):
    import marie_gb300 as mg

    A, b = dense(60, 3) if case != "maxit" else hard_dense(80, 1)
    P = np.diag(1.0 / np.diag(A))
    kw, tol, maxit = {}, 1e-10, 200
    if case == "M1":
        kw = dict(M1=lambda v: P @ v)
    elif case == "M1M2":
        kw = dict(M1=lambda v: P @ v, M2=lambda v: 0.5 * v)
    elif case == "x0":
        kw = dict(x0=np.full(60, 0.1 - 0.05j))
    elif case == "maxit":
        tol, maxit = 1e-12, 3
    ref = vo.bicgstab(lambda v: A @ v, b, tol, maxit, **kw)
    out = mg.bicgstab(lambda v: A @ v, b, tol, maxit, **kw)
    assert out[1] == ref[1]
    assert out[3] == ref[3]
    np.testing.assert_allclose(out[4], ref[4], rtol=1e-7, atol=1e-9 * ref[4][0])
    np.testing.assert_allclose(out[0], ref[0], rtol=1e-7, atol=1e-12)
    assert abs(out[2] - ref[2]) <= 1e-7 * ref[2] + 1e-15


def test_bicgstab_breakdown_and_zero_rhs():
    import marie_gb300 as mg

    A, b = dense(40, 4)
    x, flag, relres, it, resvec = mg.bicgstab(lambda v: 0 * v, b, 1e-8, 10)
    assert flag == 4
    x, flag, relres, it, resvec = mg.bicgstab(lambda v: A @ v, np.zeros(40, complex), 1e-8, 10)
    assert flag == 0 and it == 0 and not np.any(x)


@pytest.mark.parametrize("restart,ritz,kw", [(12, 4, {}), (10, 3, {"L1": True}), (10, 5, {"R1": True}),
                                             (60, None, {})])
def test_pgmresdr_handles_match_oracle(restart, ritz, kw):
    import marie_gb300 as mg

    A, b = hard_dense(120, 2)
    P = np.diag(1.0 / np.diag(A))
    kw = {k: (lambda v: P @ v) for k in kw}
    ref = vo.pgmresDR(lambda v: A @ v, b, restart, 1e-9, 100, ritz, **kw)
    out = mg.pgmresDR(lambda v: A @ v, b, restart, 1e-9, 100, ritz, **kw)
    assert out[1] == ref[1] == 0
    assert out[3] == ref[3]
    np.testing.assert_allclose(out[4], ref[4], rtol=1e-6, atol=1e-13)
    np.testing.assert_allclose(out[0], ref[0], rtol=1e-7)


def sphere_problem(L, dx, radius, eps_r=50.0, sigma=0.5):
    r = vo.grid(L, L, L, dx)
    er = np.ones((L, L, L), complex)
    er[np.sum(r * r, axis=3) < radius**2] = eps_r - 1j * sigma / (vo.EPS0 * 2 * np.pi * FREQ)
    em = vo.EMconstants(FREQ)
    E, _ = vo.PlaneWave_Excitation(r, [0, 0, em["ko"]], em["omega_mu"], [1, 0, 0])
    return r, np.asfortranarray(er), np.asfortranarray(E)


@pytest.mark.parametrize("solver,form,precond", [("B", 2, 0), ("B", 1, "L"), ("D", 2, 0), ("D", 1, "R")])
def test_jvie_solver_variants_match_oracle(solver, form, precond):
    import marie_gb300 as mg

    L, dx = 8, 5e-3
    r, er, E = sphere_problem(L, dx, 0.018)
    fN = vo.getOPERATORS(r, FREQ)
    ref = vo.JVIE_Solver(E, er, r, FREQ, fN, tol=1e-10, form=form, solver=solver, precond=precond, inner_it=12,
                         ritz=4)
    op = mg.Operator.from_array(fN)
    out = mg.JVIE_Solver(E, er, r, FREQ, op, tol=1e-10, form=form, solver=solver, precond=precond, inner_it=12,
                         ritz=4)
    assert out[1] == ref[1] == 0
    assert out[3] == ref[3]
    # entries near round-off (1e-8 of the initial residual and below) agree absolutely
    np.testing.assert_allclose(out[4], ref[4], rtol=1e-6, atol=1e-9 * ref[4][0])
    assert np.max(np.abs(out[0] - ref[0])) < 1e-8 * np.max(np.abs(ref[0]))


@pytest.mark.parametrize("solver", ["B", "D"])
def test_mixed_precision_variants_match_fp64(solver):
    import marie_gb300 as mg

    L, dx = 16, 5e-3
    r, er, E = sphere_problem(L, dx, 0.035)
    op64 = mg.Operator.assemble(L, L, L, dx, FREQ, precision="fp64")
    opm = mg.Operator.assemble(L, L, L, dx, FREQ, precision="mixed")
    J64 = mg.JVIE_Solver(E, er, r, FREQ, op64, tol=1e-6, solver="G")[0]
    Jm, fm, rrm, itm, resm, _ = mg.JVIE_Solver(E, er, r, FREQ, opm, tol=1e-6, solver=solver, inner_it=30)
    assert fm == 0 and rrm <= 1e-6
    assert np.linalg.norm(Jm - J64) / np.linalg.norm(J64) < 2e-5
