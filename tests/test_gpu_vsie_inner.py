"""The J-VIE solve as the coil solvers' inner solver: fVIEsolver_Assembly.m
(crop, operator cache, tau3, Scoord) and jvie2solver.m (BiCGSTAB with an
initial guess) against the oracle restatement."""
import numpy as np
import pytest

from oracle import vie_oracle as vo

pytestmark = pytest.mark.gpu
FREQ = 298e6


def body(L, dx, region):
    """RHBM dict on an L^3 grid: a lossy block (region = index slices) in air."""
    r = vo.grid(L, L, L, dx)
    eps = np.ones((L, L, L))
    sig = np.zeros((L, L, L))
    eps[region] = 45.0
    sig[region] = 0.6
    inner = tuple(slice(s.start + 1, s.stop - 1) for s in region)
    eps[inner] = 70.0
    return {"r": r, "epsilon_r": np.asfortranarray(eps), "sigma_e": np.asfortranarray(sig), "fN": None,
            "freqfN": None}


def incident(R, Scoord, tau3):
    """tau3 .* E_inc at the non-air voxels (the coil solvers' right-hand side)."""
    em = vo.EMconstants(FREQ)
    E, _ = vo.PlaneWave_Excitation(R["r"], [0, 0, em["ko"]], em["omega_mu"], [1, 0.5, 0])
    nonair = np.flatnonzero(np.abs(R["epsilon_r"].reshape(-1, order="F") - 1) > 0)
    Es = np.concatenate([E[..., c].reshape(-1, order="F")[nonair] for c in range(3)])
    return tau3 * Es


@pytest.mark.parametrize("region", [
    (slice(4, 14), slice(4, 14), slice(4, 14)),
    (slice(5, 14), slice(3, 12), slice(6, 15)),
])
def test_fviesolver_matches_oracle(region):
    import marie_gb300 as mg

    R = body(20, 5e-3, region)
    solver, Gram, tau3, Scoord, op = mg.fVIEsolver_Assembly(R, FREQ)
    rsolver, rGram, rtau3, rScoord, (re_r, ridx, rfN) = vo.fVIEsolver_Assembly(R, FREQ)
    # the reference's crop (the oracle), extended with air to the next FFT size
    assert re_r.shape[0] < 20 and (op.L, op.M, op.N) == tuple(mg.supported_size(n) for n in re_r.shape)
    assert Gram == rGram
    np.testing.assert_allclose(tau3, rtau3, rtol=1e-15)
    np.testing.assert_array_equal(Scoord, rScoord)
    b = incident(R, Scoord, tau3)
    x, flag, relres, it = rsolver(b, 1e-8)
    xs = solver(b, 1e-8)
    assert flag == 0
    assert np.linalg.norm(xs - x) <= 1e-6 * np.linalg.norm(x)


def test_jvie2solver_initial_guess_and_zero_rhs(cuda):
    import torch

    import marie_gb300 as mg

    R = body(16, 5e-3, (slice(3, 11), slice(4, 12), slice(2, 10)))
    solver, Gram, tau3, Scoord, op = mg.fVIEsolver_Assembly(R, FREQ)
    rsolver, _, _, _, (re_r, ridx, rfN) = vo.fVIEsolver_Assembly(R, FREQ)
    b = incident(R, Scoord, tau3)
    # the low-level entry with the cropped body's data: iterations and flags as the oracle
    e_r = np.ones((op.L, op.M, op.N), complex, order="F")
    e_r[:re_r.shape[0], :re_r.shape[1], :re_r.shape[2]] = re_r
    nd = e_r.size
    idxS = np.flatnonzero(np.abs(e_r.reshape(-1, order="F") - 1) > 1e-12)
    idx = np.concatenate([idxS, nd + idxS, 2 * nd + idxS]).astype(np.int64) + 1
    Mr, Mc = np.asfortranarray(e_r / e_r), np.asfortranarray((e_r - 1) / e_r)
    x, flag, relres, it, _ = mg.jvie2solver(b, op, idx, Mr, Mc, Gram, 1e-9)
    rx, rflag, rrelres, rit = rsolver(b, 1e-9)
    assert flag == rflag == 0 and abs(it - rit) <= 1.0, (it, rit)
    assert np.linalg.norm(x - rx) <= 1e-6 * np.linalg.norm(rx)
    # starting from the solution: converged at once
    x2, flag2, relres2, it2, _ = mg.jvie2solver(b, op, idx, Mr, Mc, Gram, 1e-6, Vini=x)
    assert flag2 == 0 and it2 == 0 and relres2 <= 1e-6
    # an all-zero right-hand side is returned as the solution
    z, fz, rz, iz, _ = mg.jvie2solver(np.zeros_like(b), op, idx, Mr, Mc, Gram, 1e-6)
    assert not np.any(z) and fz == 0 and iz == 0
    # device vectors in place
    bd = torch.from_numpy(b).to(cuda)
    xd = solver(bd, 1e-9)
    assert xd.is_cuda and np.linalg.norm(xd.cpu().numpy() - rx) <= 1e-6 * np.linalg.norm(rx)
