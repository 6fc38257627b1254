"""The 128^3 workload at full size (12-ellipsoid phantom at 2 mm, 256^3 FFT,
about 1.36 M DOFs, 298 MHz), checked through properties that hold at any
size (its element-by-element parity with the oracle is in
test_gpu_config_parity.py): the adjoint identity of the two mv_AN flags, the
transpose as the Mc similarity (N complex symmetric), linearity, FP32
products against FP64 ones, and the FP64 residual of the currents
JVIE_Solver returns.  The largest grid (512 x 384 x 320 FFT) gets the same
identities and an element-by-element comparison with the oracle's mv_AN."""
import numpy as np
import pytest

from oracle import vie_oracle as vo

pytestmark = pytest.mark.gpu
L = M = N = 128
DX, FREQ, N_ELL = 2e-3, 298e6, 12


@pytest.fixture(scope="module")
def c2():
    import marie_gb300 as mg
    from marie_gb300 import phantoms

    r, er, _ = phantoms.ellipsoids(L, M, N, DX, N_ELL, 0, FREQ)
    em = mg.EMconstants(FREQ)
    E, _ = mg.PlaneWave_Excitation(r, [0, 0, em["ko"]], em["omega_mu"], [1, 0, 0])
    E = np.asfortranarray(E)
    op = mg.Operator.assemble(L, M, N, DX, FREQ, precision="mixed")
    S = vo.jvie_setup(E, er, r, FREQ, form=2)  # form-2 system: A = Gram*1 - Mc*N on the DOFs idxS3
    S["Mr"], S["Mc"] = np.asfortranarray(S["Mr"]), np.asfortranarray(S["Mc"])
    yield r, er, E, op, S
    op.close()


def _vecs(n, seed):
    rng = np.random.default_rng(seed)
    return [rng.standard_normal(n) + 1j * rng.standard_normal(n) for _ in range(2)]


def _A(op, S, x, flag="notransp", precision="fp64"):
    import marie_gb300 as mg

    return mg.mv_AN(x, op, S["Mr"], S["Mc"], S["Gram"], flag, S["idxS3"], precision=precision)


def relerr(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def test_full_size_problem_shape(c2):
    _, er, _, _, S = c2
    n = S["idxS3"].size
    assert n == 3 * int(np.count_nonzero(np.abs(er - 1) > 1e-12)) and n > 1_000_000


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 1e-5)])
def test_adjoint_identity_full_size(c2, precision, tol):
    *_, op, S = c2
    x, y = _vecs(S["idxS3"].size, 1)
    lhs = np.vdot(y, _A(op, S, x, "notransp", precision))
    rhs = np.vdot(_A(op, S, y, "transp", precision), x)
    assert abs(lhs - rhs) <= tol * abs(lhs)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("fp32", 1e-4)])
def test_transpose_is_Mc_similarity_full_size(c2, precision, tol):
    *_, op, S = c2
    x, _ = _vecs(S["idxS3"].size, 2)
    V = L * M * N
    mc = S["Mc"].reshape(-1, order="F")[(S["idxS3"] - 1) % V]
    ATx = np.conj(_A(op, S, np.conj(x), "transp", precision))
    sim = _A(op, S, mc * x, "notransp", precision) / mc
    assert relerr(sim, ATx) < tol


def test_linearity_full_size(c2):
    *_, op, S = c2
    x, y = _vecs(S["idxS3"].size, 3)
    a, b = 2.0 - 0.5j, -3.0j
    lhs = _A(op, S, a * x + b * y)
    rhs = a * _A(op, S, x) + b * _A(op, S, y)
    assert relerr(lhs, rhs) < 1e-12


def test_fp32_products_track_fp64_full_size(c2):
    *_, op, S = c2
    x, _ = _vecs(S["idxS3"].size, 4)
    for flag in ("notransp", "transp"):
        assert relerr(_A(op, S, x, flag, "fp32"), _A(op, S, x, flag, "fp64")) < 1e-5


@pytest.mark.parametrize("solver", ["G", "B"])
def test_solutions_meet_the_tolerance_in_fp64_full_size(c2, solver):
    """||Vrhs - A Je(idxS3)|| / ||Vrhs|| recomputed with the FP64 mv_AN equals
    the relres JVIE_Solver reports and is below tol."""
    import marie_gb300 as mg

    r, er, E, op, S = c2
    tol = 1e-6
    Je, flag, relres, it, resvec, t = mg.JVIE_Solver(E, er, r, FREQ, op, tol=tol, solver=solver)
    assert flag == 0
    v = Je.reshape(-1, order="F")[S["idxS3"] - 1]
    res = np.linalg.norm(S["Vrhs"] - _A(op, S, v)) / np.linalg.norm(S["Vrhs"])
    assert res <= tol and abs(res - relres) <= 1e-3 * relres
    # no current in air
    air = np.ones(3 * L * M * N, bool)
    air[S["idxS3"] - 1] = False
    assert not np.any(Je.reshape(-1, order="F")[air])


def test_largest_grid_adjoint_and_precision():
    """The largest workload's grid, 256 x 192 x 160 voxels (512 x 384 x 320
    FFT), with a 15 cm sphere (5.3 M DOFs): adjoint identity in FP64 and
    FP32, FP32 products within 1e-5 of FP64, repeated, and the product
    element by element against the oracle's mv_AN.  This grid once
    showed the fused passes' first clusters, started early by programmatic
    dependent launch, reading the spectrum before the z pass had written it
    (wrong leading DOFs in three calls out of four)."""
    import marie_gb300 as mg
    from marie_gb300 import phantoms

    Lc, Mc_, Nc = 256, 192, 160
    r, er = phantoms.sphere(Lc, Mc_, Nc, DX, 0.15, 50.0, 0.5, FREQ)
    V = Lc * Mc_ * Nc
    idxS = np.flatnonzero(np.abs(er.reshape(-1, order="F") - 1) > 1e-12) + 1
    S = {"Mr": np.ones_like(er), "Mc": np.asfortranarray((er - 1) / er), "Gram": DX**3,
         "idxS3": np.concatenate([idxS, V + idxS, 2 * V + idxS]).astype(np.int64)}
    op = mg.Operator.assemble(Lc, Mc_, Nc, DX, FREQ, precision="mixed")
    try:
        x, y = _vecs(S["idxS3"].size, 5)
        for precision, tol in (("fp64", 1e-12), ("fp32", 1e-5)):
            lhs = np.vdot(y, _A(op, S, x, "notransp", precision))
            rhs = np.vdot(_A(op, S, y, "transp", precision), x)
            assert abs(lhs - rhs) <= tol * abs(lhs)
        for flag in ("notransp", "transp"):
            ref = _A(op, S, x, flag, "fp64")
            for _ in range(4):
                assert relerr(_A(op, S, x, flag, "fp32"), ref) < 1e-5, flag
        # element by element against the oracle's mv_AN (mv_AN.m:40-146) on
        # the device-assembled operator: FP64 1e-12, FP32 1e-5 of max|out|
        import os

        fN = op.to_array()
        orc = vo.mv_AN(x, fN, S["Mr"], S["Mc"], S["Gram"], "notransp", S["idxS3"], workers=os.cpu_count())
        del fN
        assert relerr(_A(op, S, x, "notransp", "fp64"), orc) < 1e-12
        assert relerr(_A(op, S, x, "notransp", "fp32"), orc) < 1e-5
    finally:
        op.close()
