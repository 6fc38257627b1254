"""Parity at the workload sizes, not only on small grids.

  c2  mv_AN on the 128^3 phantom (256^3 FFT, the device-assembled operator),
      both flags, element-wise against the oracle's mv_AN (mv_AN.m:40-146):
      FP64 within 1e-12 and FP32 within 1e-5 of max|out|.
  c1  the 32^3 sphere (r 7.5 cm, eps_r 50, sigma 0.5 S/m, 5 mm, 298 MHz): the
      default operator (DIRECTFN singular integrals) against the oracle's
      getOPERATORS at 1e-12, then JVIE_Solver with GMRES(50), tol 1e-6, form 2
      and form 1 with the right preconditioner (RUN_Sphere_VIE_MIE.m:168-172)
      against the oracle's JVIE_Solver: the same flag and iteration counts,
      residual histories within 1e-6 relative and fields within the tolerance.
  c4  the 64^3 ellipsoid phantom at 3 mm: the absorbed-power adjoint gradient
      against central finite differences on 32 random body voxels, for eps_r
      and sigma, within 1e-4; the mixed-precision gradient against the FP64
      adjoint gradient.  The finite differences take a relative step of 1e-4,
      not 1e-6: at this size one voxel moves F (about 546) by ~1e-11 of itself
      per 1e-6 step, while F from an FP64 solve carries ~2e-15 of rounding, so
      a 1e-6 difference is off by ~1e-4 from rounding alone.  Measured on one
      voxel: the difference to the adjoint gradient is 1.6e-4, 6e-6, 5e-7 and
      5e-8 at steps 1e-6, 1e-5, 1e-4 and 1e-3 (central differences converge
      onto the adjoint value).  The bar adds that rounding allowance
      (1e-14 |F| / h) to 1e-4 of the gradient.
"""
import math
import os

import numpy as np
import pytest

from oracle import vie_oracle as vo

pytestmark = pytest.mark.gpu
FREQ = 298e6


def relerr(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b))


# ---------------------------------------------------------------------------
# c2: the headline workload's matvec
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def c2():
    import marie_gb300 as mg
    from marie_gb300 import phantoms

    L, dx = 128, 2e-3
    r, er, _ = phantoms.ellipsoids(L, L, L, dx, 12, 0, FREQ)
    em = vo.EMconstants(FREQ)
    E, _ = mg.PlaneWave_Excitation(r, [0, 0, em["ko"]], em["omega_mu"], [1, 0, 0])
    S = vo.jvie_setup(np.asarray(E), er, r, FREQ, 2)
    op = mg.Operator.assemble(L, L, L, dx, FREQ, precision="mixed")
    fN = op.to_array()
    yield S, op, fN
    op.close()


@pytest.mark.parametrize("flag", ["notransp", "transp"])
def test_c2_mv_AN_matches_oracle_elementwise(c2, flag):
    import marie_gb300 as mg

    S, op, fN = c2
    rng = np.random.default_rng(11)
    n = S["idxS3"].size
    J = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ref = vo.mv_AN(J, fN, S["Mr"], S["Mc"], S["Gram"], flag, S["idxS3"], workers=os.cpu_count())
    scale = np.max(np.abs(ref))
    for precision, tol in (("fp64", 1e-12), ("fp32", 1e-5)):
        out = mg.mv_AN(J, op, S["Mr"], S["Mc"], S["Gram"], flag, S["idxS3"], precision=precision)
        err = np.max(np.abs(out - ref)) / scale
        assert err < tol, (flag, precision, err)


# ---------------------------------------------------------------------------
# c1: the Mie sphere, operator and solves
# ---------------------------------------------------------------------------
def test_c1_operator_and_solves_match_oracle():
    import marie_gb300 as mg
    from marie_gb300 import phantoms

    L, dx = 32, 5e-3
    r, er = phantoms.sphere(L, L, L, dx, 0.075, 50.0, 0.5, FREQ)
    em = vo.EMconstants(FREQ)
    E, _ = vo.PlaneWave_Excitation(r, [0, 0, em["ko"]], em["omega_mu"], [1, 0, 0])
    E = np.asfortranarray(E)
    fN = vo.getOPERATORS(r, FREQ)
    op = mg.Operator.assemble(L, L, L, dx, FREQ, precision="fp64")
    assert relerr(op.to_array(), fN) < 1e-12
    for form, precond in ((2, 0), (1, "R")):
        kw = dict(tol=1e-6, form=form, precond=precond, inner_it=50, outer_it=200, solver="G")
        ref = vo.JVIE_Solver(E, er, r, FREQ, fN, workers=os.cpu_count(), **kw)
        out = mg.JVIE_Solver(E, er, r, FREQ, op, **kw)
        assert out[1] == ref[1] == 0, (form, out[1], ref[1])
        assert list(out[3]) == list(ref[3]), (form, out[3], ref[3])
        np.testing.assert_allclose(out[4], ref[4], rtol=1e-6, atol=1e-13)
        assert np.linalg.norm(out[0] - ref[0]) <= 1e-6 * np.linalg.norm(ref[0]), form


# ---------------------------------------------------------------------------
# c4: adjoint gradient at 64^3 against finite differences
# ---------------------------------------------------------------------------
def _power(Je, eps, sig):
    """F = sum over body voxels of 0.5 sigma |E|^2 with E = J / (j omega eps0 chi)
    (the absorbed-power objective of marie_jvie_adjoint_grad), summed exactly."""
    omega = 2 * math.pi * FREQ
    er = eps - 1j * sig / (vo.EPS0 * omega)
    chi = er - 1.0
    body = np.abs(chi) > 1e-12
    E = Je[body] / (1j * omega * vo.EPS0 * chi[body])[:, None]
    terms = 0.5 * sig[body][:, None] * (E.real**2 + E.imag**2)
    return math.fsum(terms.ravel())


def test_c4_adjoint_gradient_matches_finite_differences():
    import marie_gb300 as mg
    from marie_gb300 import phantoms
    from marie_gb300.autograd import adjoint_gradient, complex_permittivity

    L, dx = 64, 3e-3
    r, er, _ = phantoms.ellipsoids(L, L, L, dx, 12, 0, FREQ)
    eps = np.asfortranarray(er.real)
    sig = np.asfortranarray(-er.imag * vo.EPS0 * 2 * np.pi * FREQ)
    em = vo.EMconstants(FREQ)
    E, _ = vo.PlaneWave_Excitation(r, [0, 0, em["ko"]], em["omega_mu"], [1, 0, 0])
    E = np.asfortranarray(E)
    op = mg.Operator.assemble(L, L, L, dx, FREQ, precision="fp64")
    F, ge, gs, flags, _ = adjoint_gradient(op, E, np.asfortranarray(er), dx, FREQ, "power", None, 1e-13)
    assert flags == (0, 0)

    def F_of(e, s):
        Je, flag, *_ = mg.JVIE_Solver(E, np.asfortranarray(complex_permittivity(e, s, FREQ)), r, FREQ, op,
                                      tol=1e-13, form=2, inner_it=50, outer_it=400, solver="G")
        assert flag == 0
        return _power(Je, e, s)

    assert abs(F_of(eps, sig) - F) <= 1e-9 * abs(F)
    step = 1e-4
    rng = np.random.default_rng(4)
    body = np.argwhere(eps > 1.0 + 1e-9)
    pick = body[rng.choice(len(body), 32, replace=False)]
    gmax = {"eps": np.max(np.abs(ge)), "sig": np.max(np.abs(gs))}
    for (i, j, k) in pick:
        for name, arr, g in (("eps", eps, ge), ("sig", sig, gs)):
            h = step * abs(arr[i, j, k])
            ap, am = arr.copy(order="F"), arr.copy(order="F")
            ap[i, j, k] += h
            am[i, j, k] -= h
            if name == "eps":
                fd = (F_of(ap, sig) - F_of(am, sig)) / (2 * h)
            else:
                fd = (F_of(eps, ap) - F_of(eps, am)) / (2 * h)
            bar = 1e-4 * max(abs(fd), 1e-3 * gmax[name]) + 1e-14 * abs(F) / h
            assert abs(fd - g[i, j, k]) <= bar, (name, (i, j, k), fd, g[i, j, k])
    # the mixed-precision gradient against the FP64 adjoint gradient
    opm = mg.Operator.assemble(L, L, L, dx, FREQ, precision="mixed")
    Fm, gem, gsm, flm, _ = adjoint_gradient(opm, E, np.asfortranarray(er), dx, FREQ, "power", None, 1e-6)
    assert flm == (0, 0)
    assert np.linalg.norm(gem - ge) <= 1e-4 * np.linalg.norm(ge)
    assert np.linalg.norm(gsm - gs) <= 1e-4 * np.linalg.norm(gs)
    op.close()
    opm.close()


# ---------------------------------------------------------------------------
# c3: the 16-dipole batch on the 128^3 body against 16 single solves
# ---------------------------------------------------------------------------
def test_c3_batch_gives_the_single_solves():
    """The 16 z-directed dipoles on the 0.15 m cylinder around the 128^3 body
    (z in {-5, 0, 5, 10} cm), solved as one batch (two groups, one graph
    launch), give bit for bit the currents, flags, relres and iteration
    counts of 16 single solves: each system refines with its own tolerances."""
    import marie_gb300 as mg
    from marie_gb300 import phantoms

    L, dx = 128, 2e-3
    r, er, _ = phantoms.ellipsoids(L, L, L, dx, 12, 0, FREQ)
    em = mg.EMconstants(FREQ)
    pos = phantoms.dipole_ring(0.15, [-0.05, 0.0, 0.05, 0.10], 4)
    Es = [np.asarray(mg.Dipole_Excitation(r, em["ko"], np.array([[0, 0, 1.0]]), p[None])) for p in pos]
    op = mg.Operator.assemble(L, L, L, dx, FREQ, precision="mixed", nrhs_max=16)
    Jb, flags, relres, iters, _ = mg.JVIE_Solver_batch(np.asfortranarray(np.stack(Es, axis=4)), er, r, FREQ, op,
                                                      tol=1e-6)
    for e, E in enumerate(Es):
        Js, fs, rs, its, _, _ = mg.JVIE_Solver(np.asfortranarray(E), er, r, FREQ, op, tol=1e-6, solver="G")
        assert flags[e] == fs == 0 and relres[e] == rs <= 1e-6, e
        assert list(iters[e]) == list(its), e
        np.testing.assert_array_equal(Jb[..., e], Js)
    op.close()
