"""GPU checks of the adjoint gradient (c4 structure on a small grid): central
finite differences (relative step 1e-6) on random body voxels, the objective
value against the oracle's forward solve, the mixed-precision gradient against
the FP64 adjoint gradient, and the torch.autograd.Function wrapper."""
import numpy as np
import pytest

from oracle import vie_oracle as vo

pytestmark = pytest.mark.gpu
FREQ = 298e6


def body(L=12, dx=3e-3, seed=0):
    from marie_gb300 import phantoms

    r, er, _ = phantoms.ellipsoids(L, L, L, dx, 4, seed, FREQ)
    eps = er.real.copy(order="F")
    sig = (-er.imag * vo.EPS0 * 2 * np.pi * FREQ).copy(order="F")
    em = vo.EMconstants(FREQ)
    E, _ = vo.PlaneWave_Excitation(r, [0, 0, em["ko"]], em["omega_mu"], [1, 0, 0])
    return r, eps, sig, np.asfortranarray(E)


def F_of(op, E, eps, sig, dx, objective="power", Et=None, tol=1e-12):
    from marie_gb300.autograd import adjoint_gradient, complex_permittivity

    er = np.asfortranarray(complex_permittivity(eps, sig, FREQ))
    return adjoint_gradient(op, E, er, dx, FREQ, objective, Et, tol)


@pytest.mark.parametrize("objective", ["power", "misfit"])
def test_adjoint_gradient_matches_central_differences(objective):
    import marie_gb300 as mg

    L, dx = 12, 3e-3
    r, eps, sig, E = body(L, dx)
    op = mg.Operator.assemble(L, L, L, dx, FREQ, precision="fp64")
    Et = None
    if objective == "misfit":
        rng = np.random.default_rng(1)
        inside = eps > 1.0 + 1e-9
        eps_t = eps.copy(order="F")
        sig_t = sig.copy(order="F")
        eps_t[inside] *= 1 + 0.05 * rng.standard_normal(inside.sum())
        sig_t[inside] *= 1 + 0.05 * rng.standard_normal(inside.sum())
        from marie_gb300.autograd import complex_permittivity

        Jt = mg.JVIE_Solver(E, np.asfortranarray(complex_permittivity(eps_t, sig_t, FREQ)), r, FREQ, op, tol=1e-12, solver="G")[0]
        Et = np.asfortranarray(mg.E_field_Nop(Jt, op, dx**3, FREQ, E))
    F, ge, gs, flags, iters = F_of(op, E, eps, sig, dx, objective, Et)
    assert flags == (0, 0)
    rng = np.random.default_rng(7)
    body_idx = np.argwhere(eps > 1.0 + 1e-9)
    pick = body_idx[rng.choice(len(body_idx), 6, replace=False)]
    for (i, j, k) in pick:
        for name, arr, g in (("eps", eps, ge), ("sig", sig, gs)):
            h = 1e-6 * abs(arr[i, j, k])
            a_p = arr.copy(order="F")
            a_m = arr.copy(order="F")
            a_p[i, j, k] += h
            a_m[i, j, k] -= h
            if name == "eps":
                Fp = F_of(op, E, a_p, sig, dx, objective, Et)[0]
                Fm = F_of(op, E, a_m, sig, dx, objective, Et)[0]
            else:
                Fp = F_of(op, E, eps, a_p, dx, objective, Et)[0]
                Fm = F_of(op, E, eps, a_m, dx, objective, Et)[0]
            fd = (Fp - Fm) / (2 * h)
            assert abs(fd - g[i, j, k]) <= 1e-4 * max(abs(fd), 1e-3 * np.max(np.abs(g))), (name, fd, g[i, j, k])


def test_objective_value_matches_oracle_forward_solve():
    import marie_gb300 as mg
    from marie_gb300.autograd import complex_permittivity

    L, dx = 8, 3e-3
    r, eps, sig, E = body(L, dx, seed=2)
    op = mg.Operator.assemble(L, L, L, dx, FREQ, precision="fp64")
    F, *_ = F_of(op, E, eps, sig, dx)
    er = complex_permittivity(eps, sig, FREQ)
    Je = vo.JVIE_Solver(E, er, r, FREQ, op.to_array(), tol=1e-12, solver="G")[0]
    inside = np.abs(er - 1) > 1e-12
    Ei = Je[inside] / (1j * 2 * np.pi * FREQ * vo.EPS0 * (er[inside] - 1)[:, None])
    F_ref = np.sum(0.5 * sig[inside][:, None] * np.abs(Ei) ** 2)
    assert abs(F - F_ref) < 1e-9 * F_ref


def test_mixed_precision_gradient_matches_fp64_adjoint():
    import marie_gb300 as mg

    L, dx = 16, 3e-3
    r, eps, sig, E = body(L, dx, seed=3)
    op64 = mg.Operator.assemble(L, L, L, dx, FREQ, precision="fp64")
    opm = mg.Operator.assemble(L, L, L, dx, FREQ, precision="mixed")
    F64, ge64, gs64, *_ = F_of(op64, E, eps, sig, dx, tol=1e-10)
    Fm, gem, gsm, *_ = F_of(opm, E, eps, sig, dx, tol=1e-8)
    assert abs(Fm - F64) < 1e-6 * abs(F64)
    assert np.linalg.norm(gem - ge64) < 1e-5 * np.linalg.norm(ge64)
    assert np.linalg.norm(gsm - gs64) < 1e-5 * np.linalg.norm(gs64)


def test_torch_autograd_function(cuda):
    import torch

    import marie_gb300 as mg
    from marie_gb300.autograd import jvie_objective

    L, dx = 8, 3e-3
    r, eps, sig, E = body(L, dx, seed=4)
    op = mg.Operator.assemble(L, L, L, dx, FREQ, precision="fp64")
    te = torch.tensor(eps, dtype=torch.float64, requires_grad=True)
    ts = torch.tensor(sig, dtype=torch.float64, requires_grad=True)
    F = jvie_objective(te, ts, op, E, dx, FREQ, "power", tol=1e-12)
    (2.0 * F).backward()
    F2, ge, gs, *_ = F_of(op, E, eps, sig, dx)
    assert abs(F.item() - F2) <= 1e-12 * abs(F2)
    np.testing.assert_allclose(te.grad.numpy(), 2.0 * ge, rtol=1e-12, atol=0)
    np.testing.assert_allclose(ts.grad.numpy(), 2.0 * gs, rtol=1e-12, atol=0)
