"""CPU tests of the oracle (the checker) against the reference's golden vectors
and known-answer identities.  No GPU."""
import numpy as np
import pytest

from oracle import vie_oracle as vo

FREQ = 298e6


def test_gauss_rules_match_reference_table(golden):
    for n in (4, 10, 20):
        w, x = vo.gauss_1d(n)
        g = golden["gauss_1d"][str(n)]
        np.testing.assert_allclose(x, g["x"], rtol=0, atol=2e-15)
        np.testing.assert_allclose(w, g["w"], rtol=0, atol=2e-15)


def test_near_classes_match_nearby_correct_tables(golden):
    for key, codes in golden["nearby"].items():
        m = tuple(int(c) for c in key.split(","))
        mine = [[vo.near_class(m, i, j) for j in range(6)] for i in range(6)]
        assert mine == codes, key


def test_cubature_matches_reference_cpp(golden):
    for case in golden["cubature_nop"]:
        dx, ko = case["dx"], case["ko"]
        Np, w, u, v = vo.gauss_2d(case["order"])
        Rf = vo.cube_faces(dx, dx, dx)
        I = vo.cubature_nop_batch(Np, w, u, v, np.array(case["m"], float)[None] * dx, Rf, ko, dx)[0]
        ref = np.array(case["re"]) + 1j * np.array(case["im"])
        # touching faces evaluate 1/0 at coincident Gauss points in both codes
        fin = np.isfinite(ref)
        assert np.array_equal(fin, np.isfinite(I))
        np.testing.assert_allclose(I[fin], ref[fin], rtol=1e-13, atol=1e-13 * np.abs(ref[fin]).max())


def test_converged_singular_integrals_static_closed_form():
    # int_{[0,1]^2} int_{[0,1]^2} 1/|x-y| = 4 ln(1+sqrt 2) + (4/3)(1 - sqrt 2)
    s = vo.singular_integrals(1e-12, 1.0, method="CONVERGED")
    exact = 4 * np.log(1 + np.sqrt(2)) + 4 / 3 * (1 - np.sqrt(2))
    assert abs(s[0].real - exact) < 1e-14 * exact


def test_directfn_restatement_pinned_to_reference(golden):
    """The DIRECTFN restatement (oracle/directfn.py) against the reference's
    own C++ cores through the singular_st/ea/va.m geometry, at the reference's
    Np_1D = 20 for five frequencies and four voxel sizes (the values the
    default getOPERATORS uses): 1e-13 relative."""
    for d in golden["directfn"]:
        if d["Np"] != 20:
            continue
        ref = np.array(d["re"]) + 1j * np.array(d["im"])
        mine = vo.singular_integrals(d["ko"], d["dx"])
        rel = np.abs(mine - ref) / np.abs(ref)
        assert rel.max() < 1e-13, (d["ko"], d["dx"], rel)


def test_directfn_single_calls_pinned_to_reference(golden):
    """One call of each DIRECTFN core with its MEX gateway's vertex order, on
    seeded random triangles at Np_1D 8/12/20: 1e-12 relative (random
    triangles may cross each other, so sums of larger terms cancel)."""
    from oracle import directfn as df

    fns = {"st": df.mex_st, "ea": df.mex_ea, "va": df.mex_va}
    for c in golden["directfn_tri"]:
        if c["Np"] == 20 and c["kind"] == "st":
            continue  # covered through the square sums; keeps the CPU suite short
        v = fns[c["kind"]](*c["r"], c["ko"], c["Np"])
        ref = c["re"] + 1j * c["im"]
        assert abs(v - ref) / abs(ref) < 1e-12, (c["kind"], c["Np"], abs(v - ref) / abs(ref))


def test_converged_singular_integrals_vs_directfn(golden):
    """The converged quadrature (singular='CONVERGED', not a reference method)
    differs from DIRECTFN at Np_1D = 20 by its truncation error, up to ~3.4e-5
    (edge-adjacent terms), and from DIRECTFN at Np_1D = 64 by less than 1e-6:
    DIRECTFN converges towards it.  The converged quadrature is
    self-converged to machine precision."""
    for d in golden["directfn"]:
        if d["ko"] != golden["directfn"][0]["ko"]:
            continue
        ref = np.array(d["re"]) + 1j * np.array(d["im"])
        mine = vo.singular_integrals(d["ko"], d["dx"], method="CONVERGED")
        rel = np.abs(mine - ref) / np.abs(ref)
        assert rel.max() < (4e-5 if d["Np"] == 20 else 1e-6), (d["Np"], rel)
        # the imaginary (smooth) parts agree to round-off at every Np
        np.testing.assert_allclose(mine.imag, ref.imag, rtol=1e-12)
    a = vo.singular_integrals(6.2, 5e-3, method="CONVERGED", n=24)
    b = vo.singular_integrals(6.2, 5e-3, method="CONVERGED", n=48)
    assert np.max(np.abs(a - b) / np.abs(b)) < 1e-14


def test_circulant_parity_structure():
    rng = np.random.default_rng(0)
    L, M, N = 4, 3, 5
    G = rng.standard_normal((L, M, N, 6)) + 1j * rng.standard_normal((L, M, N, 6))
    C = vo.circulant_nop(G)
    par = [(1, 1, 1), (-1, -1, 1), (-1, 1, -1), (1, 1, 1), (1, -1, -1), (1, 1, 1)]
    for q in range(6):
        for ix in range(2 * L):
            for iy in range(2 * M):
                for iz in range(2 * N):
                    if ix == L or iy == M or iz == N:
                        assert C[ix, iy, iz, q] == 0
                        continue
                    s = 1
                    sx, sy, sz = ix, iy, iz
                    if ix > L:
                        sx, s = 2 * L - ix, s * par[q][0]
                    if iy > M:
                        sy, s = 2 * M - iy, s * par[q][1]
                    if iz > N:
                        sz, s = 2 * N - iz, s * par[q][2]
                    assert C[ix, iy, iz, q] == s * G[sx, sy, sz, q]


def _random_problem(L, M, N, seed=0, frac=0.6):
    rng = np.random.default_rng(seed)
    fN = rng.standard_normal((2 * L, 2 * M, 2 * N, 6)) + 1j * rng.standard_normal((2 * L, 2 * M, 2 * N, 6))
    Mr = 1 + rng.random((L, M, N)) + 1j * rng.random((L, M, N))
    Mc = Mr - 1
    mask = rng.random(L * M * N) < frac
    idxS = np.nonzero(mask)[0] + 1
    V = L * M * N
    idx = np.concatenate([idxS, V + idxS, 2 * V + idxS])
    J = rng.standard_normal(idx.size) + 1j * rng.standard_normal(idx.size)
    return fN, Mr, Mc, idx, J


def test_mv_AN_delta_operator_is_diagonal():
    """fN = FFT of a delta at the origin (xx=yy=zz=1): N J = J, so
    mv_AN = (Gram*Mr - Mc) J."""
    L, M, N = 4, 5, 3
    _, Mr, Mc, idx, J = _random_problem(L, M, N)
    fN = np.zeros((2 * L, 2 * M, 2 * N, 6), complex)
    fN[..., 0] = fN[..., 3] = fN[..., 5] = 1.0
    out = vo.mv_AN(J, fN, Mr, Mc, 0.3, "notransp", idx)
    v = (idx - 1) % (L * M * N)
    exp = (0.3 * Mr.reshape(-1, order="F")[v] - Mc.reshape(-1, order="F")[v]) * J
    np.testing.assert_allclose(out, exp, rtol=1e-13, atol=1e-13)


def test_mv_AN_transp_is_hermitian_adjoint():
    L, M, N = 4, 3, 4
    fN0, Mr, Mc, idx, x = _random_problem(L, M, N, seed=1)
    # a physical fN is the FFT of a parity-symmetric circulant (N symmetric)
    rng = np.random.default_rng(5)
    G = rng.standard_normal((L, M, N, 6)) + 1j * rng.standard_normal((L, M, N, 6))
    # components odd along an axis vanish on the zero-offset plane of that axis
    G[0, :, :, [1, 2]] = 0
    G[:, 0, :, [1, 4]] = 0
    G[:, :, 0, [2, 4]] = 0
    fN = vo.fft_operator(vo.circulant_nop(G))
    y = rng.standard_normal(idx.size) + 1j * rng.standard_normal(idx.size)
    Ax = vo.mv_AN(x, fN, Mr, Mc, 0.7, "notransp", idx)
    AHy = vo.mv_AN(y, fN, Mr, Mc, 0.7, "transp", idx)
    lhs = np.vdot(y, Ax)
    rhs = np.vdot(AHy, x)
    assert abs(lhs - rhs) < 1e-12 * abs(lhs)


def test_mv_AN_transpose_is_Mc_similarity():
    """A = Gram*Mr - Mc*N with N complex symmetric (a physical circulant), so
    A^T = Gram*Mr - N*Mc = Mc^-1 A Mc; A^T x = conj(A^H conj(x)) through the
    'transp' flag."""
    L, M, N = 4, 5, 3
    _, Mr, Mc, idx, x = _random_problem(L, M, N, seed=2)
    rng = np.random.default_rng(7)
    G = rng.standard_normal((L, M, N, 6)) + 1j * rng.standard_normal((L, M, N, 6))
    G[0, :, :, [1, 2]] = 0
    G[:, 0, :, [1, 4]] = 0
    G[:, :, 0, [2, 4]] = 0
    fN = vo.fft_operator(vo.circulant_nop(G))
    mc = Mc.reshape(-1, order="F")[(idx - 1) % (L * M * N)]
    ATx = np.conj(vo.mv_AN(np.conj(x), fN, Mr, Mc, 0.4, "transp", idx))
    sim = vo.mv_AN(mc * x, fN, Mr, Mc, 0.4, "notransp", idx) / mc
    assert np.max(np.abs(ATx - sim)) < 1e-12 * np.max(np.abs(ATx))


def test_pgmres_dense_system_matches_solve():
    rng = np.random.default_rng(3)
    n = 40
    A = np.eye(n) * 4 + 0.3 * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    x, flag, relres, it, resvec = vo.pgmres(lambda v: A @ v, b, 10, 1e-12, 20)
    assert flag == 0 and relres <= 1e-12
    np.testing.assert_allclose(x, np.linalg.solve(A, b), rtol=1e-10)
    assert resvec[0] == pytest.approx(1.0)


def test_jvie_field_current_identity():
    """Inside the body E = J/(j omega eps0 (eps_c - 1)) for the converged J
    (E_field_Nop.m:84 with JVIE_Solver.m:151-156)."""
    L = M = N = 6
    dx = 5e-3
    r = vo.grid(L, M, N, dx)
    er = np.ones((L, M, N), complex)
    inside = np.sum(r * r, axis=3) < (2.2 * dx) ** 2
    er[inside] = 40 - 20j
    fN = vo.getOPERATORS(r, FREQ)
    em = vo.EMconstants(FREQ)
    E, _ = vo.PlaneWave_Excitation(r, [0, 0, em["ko"]], em["omega_mu"], [1, 0, 0])
    Je, flag, relres, it, resvec = vo.JVIE_Solver(E, er, r, FREQ, fN, tol=1e-10, form=1, solver="G")
    assert flag == 0
    Et = vo.E_field_Nop(Je, fN, dx**3, FREQ, E)
    Ej = Je[inside] / (1j * em["omega"] * vo.EPS0 * (er[inside, None] - 1))
    np.testing.assert_allclose(Et[inside], Ej, rtol=1e-6, atol=1e-6 * np.abs(Ej).max())


def test_getoperators_small_grid_self_consistency():
    """Toeplitz / circulant / FFT outputs of the restatement agree with each other."""
    L, M, N = 3, 4, 2
    r = vo.grid(L, M, N, 5e-3)
    T = vo.getOPERATORS(r, FREQ, typ="T")
    Cc = vo.getOPERATORS(r, FREQ, typ="C")
    F = vo.getOPERATORS(r, FREQ)
    np.testing.assert_allclose(Cc[:L, :M, :N], T)
    np.testing.assert_allclose(np.fft.fftn(Cc, axes=(0, 1, 2)), F, rtol=1e-12, atol=1e-12 * np.abs(F).max())
    # the diagonal components dominate and are even
    assert np.abs(T[0, 0, 0, 0]) > np.abs(T[0, 0, 0, 1])


def hard_dense(n, seed):
    """Complex system whose spectrum has a few small eigenvalues, so that
    restarted GMRES stalls and deflation helps."""
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    lam = np.concatenate([[0.01, 0.02, 0.05], np.linspace(1, 4, n - 3)]) * np.exp(0.3j * rng.random(n))
    A = Q @ np.diag(lam) @ Q.conj().T + 0.01 * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    return A, b


def test_bicgstab_dense_systems_converge_to_solve():
    for seed in range(3):
        rng = np.random.default_rng(seed)
        n = 60
        A = np.eye(n) * 3 + 0.4 * (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)))
        b = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        x, flag, relres, it, resvec = vo.bicgstab(lambda v: A @ v, b, 1e-10, 200)
        assert flag == 0 and relres <= 1e-10
        assert 2 * it + 1 == len(resvec)  # one norm per half step plus the initial one
        np.testing.assert_allclose(x, np.linalg.solve(A, b), rtol=1e-8)
        # a left preconditioner (Jacobi) as M1 gives the same solution
        P = np.diag(1.0 / np.diag(A))
        xp, flagp, *_ = vo.bicgstab(lambda v: A @ v, b, 1e-10, 200, lambda v: P @ v)
        assert flagp == 0
        np.testing.assert_allclose(xp, x, rtol=1e-8)


def test_bicgstab_flags_and_best_iterate():
    A, b = hard_dense(80, 1)
    x, flag, relres, it, resvec = vo.bicgstab(lambda v: A @ v, b, 1e-12, 3)
    assert flag == 1
    # the returned iterate is the best one seen, with its true residual
    assert np.isclose(relres, np.linalg.norm(b - A @ x) / np.linalg.norm(b))
    assert relres <= resvec[-1] / np.linalg.norm(b) * (1 + 1e-12)
    # zero right-hand side: x = 0 at once
    x0, f0, r0, i0, rv0 = vo.bicgstab(lambda v: A @ v, np.zeros(80, complex), 1e-8, 10)
    assert f0 == 0 and i0 == 0 and not np.any(x0)
    # breakdown scalar: rho = r~'r = 0 cannot occur, but A = 0 gives r~'v = 0
    _, f4, *_ = vo.bicgstab(lambda v: 0 * v, b, 1e-8, 10)
    assert f4 == 4


def test_pgmresdr_dense_systems():
    A, b = hard_dense(120, 2)
    xs = np.linalg.solve(A, b)
    # one cycle long enough: pgmresDR is plain GMRES
    x1, f1, r1, it1, rv1 = vo.pgmresDR(lambda v: A @ v, b, 119, 1e-10, 1, 5)
    x2, f2, r2, it2, rv2 = vo.pgmres(lambda v: A @ v, b, 119, 1e-10, 1)
    # (pgmresDR.m counts only the cycles after the first in iter(2))
    assert f1 == f2 == 0 and it1[0] == it2[0] and it1[1] == it2[1] - 1
    np.testing.assert_allclose(rv1, rv2, rtol=1e-8)
    # short restarts: deflation converges in fewer matvecs than GMRES(m)
    xd, fd, rd, itd, rvd = vo.pgmresDR(lambda v: A @ v, b, 12, 1e-8, 200, 4)
    xg, fg, rg, itg, rvg = vo.pgmres(lambda v: A @ v, b, 12, 1e-8, 200)
    assert fd == 0 and rd <= 1e-8
    np.testing.assert_allclose(xd, xs, rtol=1e-6)
    assert len(rvd) < len(rvg)
    # preconditioned forms reach the same solution
    P = np.diag(1.0 / np.diag(A))
    for kw in (dict(L1=lambda v: P @ v), dict(R1=lambda v: P @ v)):
        xp, fp, *_ = vo.pgmresDR(lambda v: A @ v, b, 12, 1e-10, 200, 4, **kw)
        assert fp == 0
        np.testing.assert_allclose(xp, xs, rtol=1e-7)


def test_cubature_kop_matches_reference_cpp(golden):
    for case in golden["cubature_kop"]:
        dx, ko = case["dx"], case["ko"]
        Np, w, u, v = vo.gauss_2d(case["order"])
        Rf = vo.cube_faces(dx, dx, dx)
        I = vo.cubature_kop_batch(Np, w, u, v, np.array(case["m"], float)[None] * dx, Rf, ko)[0]
        ref = np.array(case["re"]) + 1j * np.array(case["im"])
        # touching faces evaluate 0/0 at coincident Gauss points in both codes
        fin = np.isfinite(ref)
        assert np.array_equal(fin, np.isfinite(I))
        if fin.any():
            np.testing.assert_allclose(I[fin], ref[fin], rtol=1e-12, atol=1e-12 * np.abs(ref[fin]).max())


def test_nearby_correct_kop_drops_exactly_the_reference_st_pairs(golden):
    for key, st in golden["nearby_kop_st"].items():
        m = tuple(int(c) for c in key.split(","))
        mine = [[1 if vo.near_class(m, i, j) == 1 else 0 for j in range(6)] for i in range(6)]
        assert mine == st, key


def test_k_operator_structure():
    """Toeplitz K: component c odd in axis c (zero on that axis' zero plane);
    the circulant has the gperiodic_coeff_kop parities; mv_K is the cross
    product fK x J (so K applied to J and K applied to J + a J' differ linearly)."""
    r = vo.grid(6, 5, 4, 4e-3)
    T = vo.getOPERATORS(r, FREQ, "K", "T")
    scale = np.abs(T).max()
    assert np.abs(T[0, :, :, 0]).max() < 1e-12 * scale
    assert np.abs(T[:, 0, :, 1]).max() < 1e-12 * scale
    assert np.abs(T[:, :, 0, 2]).max() < 1e-12 * scale
    C = vo.circulant_kop(T)
    L, M, N = 6, 5, 4
    for c in range(3):
        s = np.ones(3)
        s[c] = -1
        np.testing.assert_allclose(C[2 * L - 2, 1, 1, c], s[0] * C[2, 1, 1, c])
        np.testing.assert_allclose(C[1, 2 * M - 1, 1, c], s[1] * C[1, 1, 1, c])
        np.testing.assert_allclose(C[1, 1, 2 * N - 3, c], s[2] * C[1, 1, 3, c])
    fK = vo.fft_operator(C)
    rng = np.random.default_rng(0)
    idx = np.arange(1, 3 * L * M * N + 1)
    J1 = rng.standard_normal(idx.size) + 1j * rng.standard_normal(idx.size)
    J2 = rng.standard_normal(idx.size) + 1j * rng.standard_normal(idx.size)
    a = 0.3 - 1.1j
    lhs = vo.mv_K(J1 + a * J2, fK, (L, M, N), idx)
    rhs = vo.mv_K(J1, fK, (L, M, N), idx) + a * vo.mv_K(J2, fK, (L, M, N), idx)
    np.testing.assert_allclose(lhs, rhs, atol=1e-12 * np.abs(rhs).max())
    # a current along x at one voxel gives no x component of the output
    Jx = np.zeros(idx.size, complex)
    Jx[1 + L * 2 + L * M * 1] = 1.0
    out = vo.mv_K(Jx, fK, (L, M, N), idx).reshape((L, M, N, 3), order="F")
    assert np.abs(out[..., 0]).max() < 1e-12 * np.abs(out).max()
