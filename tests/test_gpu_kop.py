"""GPU parity of the K operator path against the oracle restatements of
getOPERATORS(r, f, 'K') (assembly_kop.m, cubature_kop.cpp,
cubature_kop_near_sym.m, nearby_correct_kop.m, circulant_kop.m), mv_K.m and
H_field_Kop.m.  Bars: assembly 1e-12, FP64 matvec 1e-12 and FP32 1e-5 of
max|out|, as for the N operator."""
import numpy as np
import pytest

from oracle import vie_oracle as vo

pytestmark = pytest.mark.gpu
FREQ = 298e6
TOL = {"fp64": 1e-12, "fp32": 1e-5}


def relerr(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b))


@pytest.mark.parametrize("shape,dx", [((8, 4, 12), 4e-3), ((12, 8, 16), 2e-3)])
def test_get_operators_k_matches_oracle(shape, dx):
    import marie_gb300 as mg

    r = vo.grid(*shape, dx)
    T = vo.getOPERATORS(r, FREQ, "K", "T")
    for typ in ("T", "C", "FFTofC"):
        ref = T if typ == "T" else (vo.circulant_kop(T) if typ == "C" else vo.fft_operator(vo.circulant_kop(T)))
        out = mg.getOPERATORS(r, FREQ, "K", typ)
        assert out.shape == ref.shape
        assert relerr(out, ref) < 1e-12, typ


def k_problem(L, M, N, seed, symmetric=True, frac=0.6):
    rng = np.random.default_rng(seed)
    if symmetric:
        G = rng.standard_normal((L, M, N, 3)) + 1j * rng.standard_normal((L, M, N, 3))
        G[0, :, :, 0] = 0  # odd components vanish on their axis' zero plane
        G[:, 0, :, 1] = 0
        G[:, :, 0, 2] = 0
        fK = vo.fft_operator(vo.circulant_kop(G))
    else:
        fK = rng.standard_normal((2 * L, 2 * M, 2 * N, 3)) + 1j * rng.standard_normal((2 * L, 2 * M, 2 * N, 3))
    mask = rng.random(L * M * N) < frac
    mask[0] = True
    idxS = np.nonzero(mask)[0] + 1
    V = L * M * N
    idx = np.concatenate([idxS, V + idxS, 2 * V + idxS])
    J = rng.standard_normal(idx.size) + 1j * rng.standard_normal(idx.size)
    return np.asfortranarray(fK), idx, J


@pytest.mark.parametrize("shape", [(4, 8, 12), (12, 20, 24), (32, 32, 4), (48, 12, 20), (8, 8, 256), (64, 64, 8)])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_mv_K_matches_oracle(shape, precision):
    import marie_gb300 as mg

    fK, idx, J = k_problem(*shape, seed=sum(shape))
    ref = vo.mv_K(J, fK, shape, idx)
    op = mg.Operator.from_array_k(fK, precision="mixed")
    out = mg.mv_K(J, op, None, idx, precision=precision)
    assert relerr(out, ref) < TOL[precision]
    op.close()


def test_mv_K_full_layout_and_batched_rhs():
    import marie_gb300 as mg

    L, M, N = 8, 12, 20
    fK, idx, J = k_problem(L, M, N, seed=3, symmetric=False)
    rng = np.random.default_rng(4)
    Jb = np.asfortranarray(rng.standard_normal((idx.size, 3)) + 1j * rng.standard_normal((idx.size, 3)))
    op = mg.Operator.from_array_k(fK, precision="fp64", nrhs_max=2)
    out = mg.mv_K(Jb, op, None, idx)
    for c in range(3):
        assert relerr(out[:, c], vo.mv_K(Jb[:, c], fK, (L, M, N), idx)) < 1e-12
    op.close()


def test_h_field_kop_and_device_assembly():
    import marie_gb300 as mg

    L, dx = 12, 4e-3
    r = vo.grid(L, L, L, dx)
    fK = vo.getOPERATORS(r, FREQ, "K")
    rng = np.random.default_rng(7)
    J = np.asfortranarray(rng.standard_normal((L, L, L, 3)) + 1j * rng.standard_normal((L, L, L, 3)))
    Hinc = np.asfortranarray(rng.standard_normal((L, L, L, 3)) + 1j * rng.standard_normal((L, L, L, 3)))
    ref = vo.H_field_Kop(J, fK, dx**3, Hinc)
    # K assembled on the device next to N in one plan
    op = mg.Operator.assemble(L, L, L, dx, FREQ, precision="fp64").assemble_k(dx, FREQ)
    out = mg.H_field_Kop(J, op, dx**3, Hinc)
    assert relerr(out - Hinc, ref - Hinc) < 1e-11
    # the N operator of the same plan is untouched
    E = mg.E_field_Nop(J, op, dx**3, FREQ)
    Eref = vo.E_field_Nop(J, op.to_array(), dx**3, FREQ)
    assert relerr(E, Eref) < 1e-12
    op.close()


@pytest.mark.parametrize("solver", ["G", "B"])
def test_scat_solver_matches_oracle(solver):
    """Scat_Solver.m end to end (RUN_Sphere_VIE_MIE-type sphere, plane wave E
    and H): current, SAR, total E, B, global SAR and absorbed power."""
    import marie_gb300 as mg

    L, dx = 12, 5e-3
    r = vo.grid(L, L, L, dx)
    em = vo.EMconstants(FREQ)
    inside = np.sum(r * r, axis=3) < 0.02**2
    eps = np.where(inside, 50.0, 1.0)
    sig = np.where(inside, 0.5, 0.0)
    rho = np.where(inside, 1000.0, 0.0)
    E, H = vo.PlaneWave_Excitation(r, [0, 0, em["ko"]], em["omega_mu"], [1, 0, 0])
    E, H = np.asfortranarray(E), np.asfortranarray(H)
    fN = vo.getOPERATORS(r, FREQ, "N")
    fK = vo.getOPERATORS(r, FREQ, "K")
    ref = vo.Scat_Solver(E, H, FREQ, r, eps, sig, rho, 1e-10, fN, fK, 2, solver, 0, 1000, 50, 200, 5)
    op = mg.Operator.from_array(fN).set_k(fK)
    out = mg.Scat_Solver(E, H, FREQ, r, eps, sig, rho, 1e-10, op, None, 2, solver)
    for a, b, name in zip(out[:4], ref[:4], ("J", "SAR", "E", "B")):
        assert relerr(a, b) < 1e-8, name
    assert abs(out[4] - ref[4]) <= 1e-8 * abs(ref[4])
    assert abs(out[5] - ref[5]) <= 1e-8 * abs(ref[5])
    op.close()
