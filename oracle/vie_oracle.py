"""numpy/scipy restatement of the reference J-VIE path (TEST INFRASTRUCTURE ONLY).

Arrays follow the reference's MATLAB layout: numpy arrays of shape
(L, M, N[, 3 or 6]) addressed in Fortran (column-major) order; idx vectors are
1-based.  Every function cites the reference file:line it restates.
"""
from __future__ import annotations

import functools

import numpy as np
import scipy.fft
import scipy.special as sp

# ---------------------------------------------------------------------------
# constants: src_vie/src_solver/EMconstants.m:13-20
# ---------------------------------------------------------------------------
MU0 = 4 * np.pi * 1e-7
C0 = 299792458.0
EPS0 = 1.0 / C0**2 / MU0


def EMconstants(freq):
    omega = 2 * np.pi * freq
    lam = C0 / freq
    ko = 2 * np.pi / lam
    return dict(mu=MU0, co=C0, eo=EPS0, omega=omega, ko=ko, omega_mu=omega * MU0)


def _fftn(x, s, workers):
    return scipy.fft.fftn(x, s=s, axes=(0, 1, 2), workers=workers)


def _ifftn(x, workers):
    return scipy.fft.ifftn(x, axes=(0, 1, 2), workers=workers)


# ---------------------------------------------------------------------------
# matvecs
# ---------------------------------------------------------------------------
def mv_AN(JIn0, fN, Mr, Mc, Gram, transp_flag, idx, workers=None):
    """src_vie/src_mvp/mv_AN.m:40-146 ('notransp' :101-131, 'transp' :65-99)."""
    LfN, MfN, NfN, _ = fN.shape
    L, M, N = Mr.shape
    s = (LfN, MfN, NfN)
    flat = np.zeros(L * M * N * 3, dtype=complex)
    flat[np.asarray(idx) - 1] = JIn0
    JIn = flat.reshape((L, M, N, 3), order="F")
    JOut = np.zeros((L, M, N, 3), dtype=complex)
    sym = ((0, 1, 2), (1, 3, 4), (2, 4, 5))  # x->(1,2,3), y->(2,4,5), z->(3,5,6)
    acc = [0, 0, 0]
    if transp_flag == "transp":
        Mcc = np.conj(Mc)
        for c in range(3):
            fJ = _fftn(np.conj(Mcc * JIn[:, :, :, c]), s, workers)
            for o in range(3):
                acc[o] = acc[o] + fN[:, :, :, sym[c][o]] * fJ
        for o in range(3):
            Jo = _ifftn(acc[o], workers)
            JOut[:, :, :, o] = Gram * np.conj(Mr) * JIn[:, :, :, o] - np.conj(Jo[:L, :M, :N])
    elif transp_flag == "notransp":
        for c in range(3):
            fJ = _fftn(JIn[:, :, :, c], s, workers)
            for o in range(3):
                acc[o] = acc[o] + fN[:, :, :, sym[c][o]] * fJ
        for o in range(3):
            Jo = _ifftn(acc[o], workers)
            JOut[:, :, :, o] = Gram * Mr * JIn[:, :, :, o] - Mc * Jo[:L, :M, :N]
    else:
        raise ValueError("transp_flag must be 'transp' or 'notransp'")
    return JOut.reshape(-1, order="F")[np.asarray(idx) - 1]


def mv_N(JIn0, fN, r_shape, idx, workers=None):
    """src_vie/src_mvp/mv_N.m:1-95: crop(N J) on the entries idx (mv_L without
    the Gram term)."""
    return mv_L(JIn0, fN, r_shape, 0.0, idx, workers)


def mv_L(JIn0, fN, r_shape, Gram, idx, workers=None):
    """src_vie/src_mvp/mv_L.m:30-97: crop(N J) - Gram J on the entries idx."""
    LfN, MfN, NfN, _ = fN.shape
    L, M, N = r_shape[:3]
    flat = np.zeros(L * M * N * 3, dtype=complex)
    flat[np.asarray(idx) - 1] = JIn0
    JIn = flat.reshape((L, M, N, 3), order="F")
    JOut = np.zeros((L, M, N, 3), dtype=complex)
    sym = ((0, 1, 2), (1, 3, 4), (2, 4, 5))
    acc = [0, 0, 0]
    for c in range(3):
        fJ = _fftn(JIn[:, :, :, c], (LfN, MfN, NfN), workers)
        for o in range(3):
            acc[o] = acc[o] + fN[:, :, :, sym[c][o]] * fJ
    for o in range(3):
        Jo = _ifftn(acc[o], workers)
        JOut[:, :, :, o] = Jo[:L, :M, :N] - Gram * JIn[:, :, :, o]
    return JOut.reshape(-1, order="F")[np.asarray(idx) - 1]


def E_field_Nop(J, fN, Gram, freq, Einc=None, workers=None):
    """src_vie/src_fields/src_op/E_field_Nop.m:59-84."""
    if Einc is None:
        Einc = np.zeros_like(J)
    if not np.any(J):
        return Einc
    omega = 2 * np.pi * freq
    L, M, N, _ = J.shape
    idx = np.arange(1, 3 * L * M * N + 1)
    E = mv_L(J.reshape(-1, order="F"), fN, J.shape, Gram, idx, workers)
    E = E.reshape((L, M, N, 3), order="F")
    return Einc + E / (Gram * 1j * omega * EPS0)


# ---------------------------------------------------------------------------
# GMRES: src_numeric/src_iterative/pgmres.m:70-181, pgmres_iter.m:22-150
# ---------------------------------------------------------------------------
def pgmres_iter(A, x, r, m, L1, L2, R1, R2, tol):
    n = r.shape[0]
    V = np.zeros((n, m + 1), dtype=complex)
    V[:, 0] = r / np.linalg.norm(r)
    H = np.zeros((m + 1, m), dtype=complex)
    resvec = np.zeros(m)
    y = res = None
    k = 0
    for k in range(1, m + 1):
        w = V[:, k - 1]
        if R1 is not None:
            w = R1(w)
        if R2 is not None:
            w = R2(w)
        w = A(w)
        if L1 is not None:
            w = L1(w)
        if L2 is not None:
            w = L2(w)
        H[:k, k - 1] = V[:, :k].conj().T @ w          # pgmres_iter.m:106 (CGS)
        w = w - V[:, :k] @ H[:k, k - 1]              # :107
        H[k, k - 1] = np.linalg.norm(w)              # :109
        with np.errstate(divide="ignore", invalid="ignore"):
            V[:, k] = w / H[k, k - 1]                # :110
        rhs = np.zeros(k + 1, dtype=complex)
        rhs[0] = np.linalg.norm(r)
        Hc = H[:k + 1, :k]
        y = np.linalg.lstsq(Hc, rhs, rcond=None)[0]  # :118  y = Hc \ rhs
        res = rhs - Hc @ y
        resvec[k - 1] = np.linalg.norm(res)
        if resvec[k - 1] < tol:
            break
    resvec = resvec[:k]
    xupd = V[:, :k] @ y
    if R1 is not None:
        xupd = R1(xupd)
    if R2 is not None:
        xupd = R2(xupd)
    x = x + xupd
    with np.errstate(invalid="ignore"):
        r = V[:, :k + 1] @ res
    return x, r, k, resvec


def pgmres(A, b, restart=50, tol=1e-3, maxit=10, L1=None, L2=None, R1=None, R2=None, x0=None):
    """Returns (x, flag, relres, iter, resvec) like pgmres.m."""
    if x0 is None:
        x0 = np.zeros_like(b)
    r = b - A(x0) if np.count_nonzero(x0) else b.copy()
    bp = b.copy()
    if L1 is not None:
        r = L1(r)
        bp = L1(bp)
    if L2 is not None:
        r = L2(r)
        bp = L2(bp)
    bnorm = np.linalg.norm(bp)
    resvec = [np.linalg.norm(r) / bnorm]
    outit = 0
    x = x0.copy()
    p = 0
    while resvec[-1] > tol and outit < maxit:
        outit += 1
        x, r, p, rin = pgmres_iter(A, x, r, restart, L1, L2, R1, R2, tol * bnorm)
        resvec.extend(list(rin / bnorm))
    relres = np.linalg.norm(b - A(x)) / np.linalg.norm(b)
    flag = 0 if relres <= tol else 1
    return x, flag, relres, [p, outit], np.array(resvec)


# ---------------------------------------------------------------------------
# GMRES with deflated restarting: src_numeric/src_iterative/pgmresDR.m:84-282,
# pgmresDR_iter.m:36-142, getHarmVecs1.m, getHarmVecs2.m
# ---------------------------------------------------------------------------
def _lsq(A, b):
    """MATLAB A \\ b for a tall full-rank A (least squares)."""
    return np.linalg.lstsq(A, b, rcond=None)[0]


def pgmresDR_iter(A, r, m, L1, L2, R1, R2, C, tol):
    """pgmresDR_iter.m:76-142: GMRES cycle on A R1 R2 (left L1, L2) with the
    Krylov vectors kept orthogonal to the columns of C (B = C' w).  Returns
    (V, H, B, k, resvec) truncated to the k steps taken."""
    n = r.shape[0]
    V = np.zeros((n, m + 1), dtype=complex)
    nr = np.linalg.norm(r)
    V[:, 0] = r / nr
    nc = 0 if C is None else C.shape[1]
    Bm = np.zeros((nc, m), dtype=complex)
    H = np.zeros((m + 1, m), dtype=complex)
    resvec = np.zeros(m)
    k = 0
    for k in range(1, m + 1):
        w = V[:, k - 1]
        if R2 is not None:
            w = R2(w)
        if R1 is not None:
            w = R1(w)
        w = A(w)
        if L1 is not None:
            w = L1(w)
        if L2 is not None:
            w = L2(w)
        if nc:
            Bm[:, k - 1] = C.conj().T @ w
            w = w - C @ Bm[:, k - 1]
        H[:k, k - 1] = V[:, :k].conj().T @ w
        w = w - V[:, :k] @ H[:k, k - 1]
        H[k, k - 1] = np.linalg.norm(w)
        with np.errstate(divide="ignore", invalid="ignore"):
            V[:, k] = w / H[k, k - 1]
        rhs = np.zeros(k + 1, dtype=complex)
        rhs[0] = nr
        Hc = H[:k + 1, :k]
        res = rhs - Hc @ _lsq(Hc, rhs)
        resvec[k - 1] = np.linalg.norm(res)
        if resvec[k - 1] < tol:
            return V[:, :k + 1], H[:k + 1, :k], Bm[:, :k], k, resvec[:k]
    return V, H, Bm, k, resvec


def _sorted_eig(evals, evecs):
    """Eigenpairs ordered by ascending |eigenvalue| (the sortrows on
    [abs(diag(D)) V'] of getHarmVecs1.m:25-27 / getHarmVecs2.m:31-33)."""
    order = np.argsort(np.abs(evals), kind="stable")
    return evecs[:, order]


def getHarmVecs1(m, k, H):
    """getHarmVecs1.m:17-28: the k harmonic Ritz vectors of smallest |theta|
    from H_m + h_{m+1,m}^2 f e_m^T with f = H_m^{-H} e_m."""
    Hm = H[:m, :]
    F = np.linalg.solve(Hm.conj().T, np.eye(m))
    F[:, :m - 1] = 0
    Mh = Hm + H[m, m - 1] ** 2 * F
    evals, evecs = np.linalg.eig(Mh)
    return _sorted_eig(evals, evecs)[:, :k]


def getHarmVecs2(m, k, H2, V, U, C):
    """getHarmVecs2.m:17-34: generalized problem (H2' W) g = theta (H2' H2) g,
    W = [C'U, 0; V'U, I; 0 0]; the k eigenvectors of largest |theta|."""
    import scipy.linalg

    Bm = H2.conj().T @ H2
    W = np.zeros((m + 1, m), dtype=complex)
    W[:k, :k] = C.conj().T @ U
    W[k:m + 1, :k] = V.conj().T @ U
    W[k:m, k:m] = np.eye(m - k)
    Am = H2.conj().T @ W
    evals, evecs = scipy.linalg.eig(Am, Bm)
    return _sorted_eig(evals, evecs)[:, m - k:]


def pgmresDR(A, b, restart=50, tol=1e-3, maxit=10, ritz=None, L1=None, L2=None, R1=None, R2=None, x0=None):
    """Returns (x, flag, relres, iter, resvec) like pgmresDR.m: GMRES(restart)
    that carries ritz harmonic Ritz vectors of each cycle into the next."""
    if ritz is None:
        ritz = min(10, int(np.floor(restart / 2 + 0.5)))
    else:
        ritz = min(ritz, restart - 1)
    if x0 is None:
        x0 = np.zeros_like(b)
    r = b - A(x0)
    bp = b.copy()
    if L1 is not None:
        r = L1(r)
        bp = L1(bp)
    if L2 is not None:
        r = L2(r)
        bp = L2(bp)
    bnorm = np.linalg.norm(bp)
    resvec = [np.linalg.norm(r) / bnorm]
    outit = 0
    V, H, _, p, rin = pgmresDR_iter(A, r, restart, L1, L2, R1, R2, None, tol * bnorm)
    resvec.extend(list(rin / bnorm))
    y = _lsq(H, V.conj().T @ r)
    x = V[:, :p] @ y
    r = r - V @ (H @ y)
    U = C = None
    if resvec[-1] > tol:
        P = getHarmVecs1(p, min(ritz, p - 1), H)
        U = V[:, :p] @ P
        Cq, R = np.linalg.qr(H @ P)
        C = V @ Cq
        U = np.linalg.solve(R.T, U.T).T  # U / R
    while resvec[-1] > tol and outit < maxit:
        outit += 1
        V, H, Bm, p, rin = pgmresDR_iter(A, r, restart, L1, L2, R1, R2, C, tol * bnorm)
        resvec.extend(list(rin / bnorm))
        kr = U.shape[1]
        d = np.linalg.norm(U, axis=0)
        D = np.diag(1.0 / d)
        U = U @ D
        H2 = np.zeros((kr + H.shape[0], kr + H.shape[1]), dtype=complex)
        H2[:kr, :kr] = D
        H2[:kr, kr:] = Bm
        H2[kr:, kr:] = H
        CV = np.concatenate([C, V], axis=1)
        y = _lsq(H2, CV.conj().T @ r)
        x = x + np.concatenate([U, V[:, :p]], axis=1) @ y
        r = r - CV @ (H2 @ y)
        if resvec[-1] > tol:
            P = getHarmVecs2(p + kr, kr, H2, V, U, C)
            U = np.concatenate([U, V[:, :p]], axis=1) @ P
            Q, R = np.linalg.qr(H2 @ P)
            C = CV @ Q
            U = np.linalg.solve(R.T, U.T).T
    if R2 is not None:
        x = R2(x)
    if R1 is not None:
        x = R1(x)
    x = x0 + x
    relres = np.linalg.norm(b - A(x)) / np.linalg.norm(b)
    flag = 0 if relres <= tol else 1
    return x, flag, relres, [p, outit], np.array(resvec)


def bicgstab(A, b, tol=1e-6, maxit=None, M1=None, M2=None, x0=None):
    """Returns (x, flag, relres, iter, resvec) like MATLAB's bicgstab, which
    JVIE_Solver.m:451-499 calls for its default solver 'B'.

    bicgstab is a MATLAB built-in (about R2014a, the release getOPERATORS.m:55
    tests for), not part of the reference sources.  This restates the published
    BiCGSTAB iteration (van der Vorst, SIAM J. Sci. Stat. Comput. 13, 1992) with
    the documented MATLAB interface: preconditioner applied as ph = M2(M1(p))
    (function handles), iter counted in half steps, resvec the absolute
    residual norm after every half step (initial residual first), flag 0
    converged / 1 maxit / 2 non-finite preconditioner output / 3 stagnation /
    4 a breakdown scalar (rho, beta, r~'v, t't zero or infinite).  Convergence
    reported by the recurrence is confirmed with a true residual b - A x, which
    then replaces the recurrence residual; up to min(n/50, 5, n - maxit)
    confirmations may fail before flag 3.  Without convergence the iterate with
    the smallest residual norm is returned."""
    n = b.size
    maxit = min(n, 20) if maxit is None else int(maxit)
    eps = np.finfo(float).eps
    nrm = np.linalg.norm

    def prec(v):
        if M1 is not None:
            v = M1(v)
        if M2 is not None:
            v = M2(v)
        return v

    nb = nrm(b)
    if nb == 0:
        return np.zeros_like(b), 0, 0.0, 0.0, np.array([0.0])
    x = np.zeros_like(b) if x0 is None else np.array(x0, dtype=complex)
    r = b - A(x) if np.count_nonzero(x) else b.copy()
    tolb = tol * nb
    nr = nrm(r)
    resvec = [nr]
    if nr <= tolb:
        return x, 0, nr / nb, 0.0, np.array(resvec)
    rt = r.copy()
    best_nr, best_x, best_it = nr, x.copy(), 0.0
    rho_old = alpha = omega = 1.0
    p = v = np.zeros_like(b)
    flag, it, stag, extra = 1, float(maxit), 0, 0
    max_extra = min(n // 50, 5, n - maxit)
    nr_act = nr

    def confirm(xc, rc, nrc):
        """True-residual check behind a small recurrence residual; returns
        (residual vector, its norm, outcome) with outcome 'ok', 'go' or 'stop'."""
        nonlocal stag, extra
        if not (nrc <= tolb or stag >= 3 or extra):
            return rc, nrc, "go"
        rc = b - A(xc)
        nrc = nrm(rc)
        if nrc <= tolb:
            return rc, nrc, "ok"
        if stag >= 3 and extra == 0:
            stag = 0
        extra += 1
        return rc, nrc, ("stop" if extra >= max_extra else "go")

    for i in range(1, maxit + 1):
        rho = np.vdot(rt, r)
        if rho == 0 or not np.isfinite(rho):
            flag = 4
            break
        if i == 1:
            p = r.copy()
        else:
            beta = (rho / rho_old) * (alpha / omega)
            if beta == 0 or not np.isfinite(beta):
                flag = 4
                break
            p = r + beta * (p - omega * v)
        ph = prec(p)
        if not np.all(np.isfinite(ph)):
            flag = 2
            break
        v = A(ph)
        rtv = np.vdot(rt, v)
        if rtv == 0 or not np.isfinite(rtv):
            flag = 4
            break
        alpha = rho / rtv
        stag = stag + 1 if abs(alpha) * nrm(ph) < eps * nrm(x) else 0
        xh = x + alpha * ph
        s = r - alpha * v
        s, nr_act, out = confirm(xh, s, nrm(s))
        resvec.append(nr_act)
        if out != "go":
            x = xh
            flag, it = (0, i - 0.5) if out == "ok" else (3, i - 0.5)
            break
        if nr_act < best_nr:
            best_nr, best_x, best_it = nr_act, xh.copy(), i - 0.5
        sh = prec(s)
        if not np.all(np.isfinite(sh)):
            flag = 2
            break
        t = A(sh)
        tt = np.vdot(t, t).real
        if tt == 0 or not np.isfinite(tt):
            flag = 4
            break
        omega = np.vdot(t, s) / tt
        stag = stag + 1 if abs(omega) * nrm(sh) < eps * nrm(xh) else 0
        x = xh + omega * sh
        r = s - omega * t
        r, nr_act, out = confirm(x, r, nrm(r))
        resvec.append(nr_act)
        if out != "go":
            flag, it = (0, float(i)) if out == "ok" else (3, float(i))
            break
        if nr_act < best_nr:
            best_nr, best_x, best_it = nr_act, x.copy(), float(i)
        if omega == 0:
            flag = 4
            break
        rho_old = rho
    if flag == 0:
        relres = nr_act / nb
    else:
        if flag in (2, 4):
            it = len(resvec) / 2 - 0.5
        nb_best = nrm(b - A(best_x))
        if nb_best <= nr_act:
            x, it, relres = best_x, best_it, nb_best / nb
        else:
            relres = nr_act / nb
    return x, flag, relres, it, np.array(resvec)


# ---------------------------------------------------------------------------
# JVIE_Solver (solver 'G'): src_vie/src_solver/JVIE_Solver.m:71-156,176-299,513-514
# ---------------------------------------------------------------------------
def jvie_setup(Einc, e_r, r, freq, form=2):
    em = EMconstants(freq)
    Mr = e_r.astype(complex).copy()
    Mc = e_r - 1.0
    dx = r[1, 0, 0, 0] - r[0, 0, 0, 0]
    Gram = dx**3
    L, M, N = e_r.shape
    nD = L * M * N
    idxS = np.nonzero(np.abs(Mc.reshape(-1, order="F")) > 1e-12)[0] + 1
    idxS3 = np.concatenate([idxS, nD + idxS, 2 * nD + idxS])
    tau = 1j * em["omega"] * em["eo"] * Mc
    tau3 = np.concatenate([tau.reshape(-1, order="F")] * 3)
    Vrhs = Gram * tau3[idxS3 - 1] * Einc.reshape(-1, order="F")[idxS3 - 1]
    if form != 1:
        Mc = Mc / Mr
        mr = Mr.reshape(-1, order="F")[idxS - 1]
        Vrhs = Vrhs / np.concatenate([mr, mr, mr])
        Mr = Mr / Mr
    return dict(Mr=Mr, Mc=Mc, Gram=Gram, idxS3=idxS3, Vrhs=Vrhs, shape=(L, M, N))


def JVIE_Solver(Einc, e_r, r, freq, fN, tol=1e-3, form=2, solver="B", precond=0, max_it=1000, inner_it=50,
                outer_it=200, ritz=5, workers=None):
    """JVIE_Solver.m:71-122 argument handling, :176-299 operators, :300-499 the
    solver dispatch ('G' pgmres, 'D' pgmresDR, anything else 'B' bicgstab)."""
    if tol < 1e-15 or tol >= 1:
        tol = 1e-3
    if solver not in ("G", "D"):
        solver = "B"
    if precond not in ("L", "R"):
        precond = 0
    S = jvie_setup(Einc, e_r, r, freq, form)
    Mr, Mc, Gram, idx = S["Mr"], S["Mc"], S["Gram"], S["idxS3"]

    def fA(J):
        return mv_AN(J, fN, Mr, Mc, Gram, "notransp", idx, workers)

    def fP(J):
        return mv_AN(J, fN, 1.0 / Mr, 1.0 / Mr - 1.0, Gram, "notransp", idx, workers)

    if solver == "B":
        # JVIE_Solver.m:451-499: either precond letter makes fP bicgstab's M1
        vsol, flag, relres, it, resvec = bicgstab(fA, S["Vrhs"], tol, max_it, fP if precond else None)
    elif solver == "D":
        ritz = min(ritz if ritz and ritz >= 1 else 5, inner_it - 1)
        L1, R1 = (fP, None) if precond == "L" else ((None, fP) if precond == "R" else (None, None))
        vsol, flag, relres, it, resvec = pgmresDR(fA, S["Vrhs"], inner_it, tol, outer_it, ritz, L1, None, R1)
    elif precond == "R":
        vsol, flag, relres, it, resvec = pgmres(fA, S["Vrhs"], inner_it, tol, outer_it, None, None, fP)
    elif precond == "L":
        vsol, flag, relres, it, resvec = pgmres(fA, S["Vrhs"], inner_it, tol, outer_it, fP)
    else:
        vsol, flag, relres, it, resvec = pgmres(fA, S["Vrhs"], inner_it, tol, outer_it)
    L, M, N = S["shape"]
    Je = np.zeros(L * M * N * 3, dtype=complex)
    Je[idx - 1] = vsol
    return Je.reshape((L, M, N, 3), order="F"), flag, relres, it, resvec


def Scat_Solver(Einc, Hinc, freq, r, epsilon_r, sigma_e, rho, tol=1e-3, fN=None, fK=None, form=2, solver="B",
                precond=0, max_it=1000, inner_it=50, outer_it=200, ritz=5):
    """src_vie/src_solver/Scat_Solver.m:143-194: current, SAR, total E,
    B = mu0 H, global SAR and absorbed power."""
    em = EMconstants(freq)
    e_r = epsilon_r - 1j * sigma_e / (em["eo"] * em["omega"])
    dx = r[1, 0, 0, 0] - r[0, 0, 0, 0]
    Gram = dx**3
    if fN is None:
        fN = getOPERATORS(r, freq, "N")
    if fK is None:
        fK = getOPERATORS(r, freq, "K")
    Jout = JVIE_Solver(Einc, e_r, r, freq, fN, tol, form, solver, precond, max_it, inner_it, outer_it, ritz)[0]
    denom = 2 * sigma_e * rho
    S = np.sum(np.abs(Jout) ** 2, axis=3)
    with np.errstate(divide="ignore", invalid="ignore"):
        Sout = np.where(np.abs(denom) > 1e-10, S / denom, 0.0)
    Eout = E_field_Nop(Jout, fN, Gram, freq, Einc)
    Bout = 4 * np.pi * 1e-7 * H_field_Kop(Jout, fK, Gram, Hinc)
    Pabs = 0.5 * np.real(np.sum(Eout * np.conj(Jout))) * Gram
    Gsar = np.sum(Sout) * Gram
    return Jout, Sout, Eout, Bout, Gsar, Pabs


# ---------------------------------------------------------------------------
# excitations
# ---------------------------------------------------------------------------
def PlaneWave_Excitation(r, k, omega_mu, Eo):
    """src_vie/src_fields/src_excitations/PlaneWave_Excitation.m:39-95 (E and H)."""
    L, M, N, _ = r.shape
    dx = r[1, 0, 0, 0] - r[0, 0, 0, 0]
    dy = r[0, 1, 0, 1] - r[0, 0, 0, 1]
    dz = r[0, 0, 1, 2] - r[0, 0, 0, 2]
    k = np.asarray(k, dtype=float)
    Eo = np.asarray(Eo, dtype=complex)
    Ho = (1 / omega_mu) * np.cross(k, Eo)
    fac = []
    for a, d in zip(range(3), (dx, dy, dz)):
        if k[a] != 0:
            fac.append(np.exp(-1j * k[a] * r[:, :, :, a]) * (np.exp(-1j * k[a] * d / 2) - np.exp(1j * k[a] * d / 2))
                       / (-1j * k[a]))
        else:
            fac.append(d * np.ones((L, M, N)))
    Eexc = fac[0] * fac[1] * fac[2]
    E = np.stack([Eo[i] * Eexc for i in range(3)], axis=3) / (dx * dy * dz)
    H = np.stack([Ho[i] * Eexc for i in range(3)], axis=3) / (dx * dy * dz)
    return E, H


def E_field_DGF(J, Icoord, Ocoord, ko):
    """src_vie/src_fields/src_dgf/E_field_DGF.m:36-99; J is Ni x 3, coords are N x 3."""
    omega = ko * C0
    J = np.asarray(J, dtype=complex).reshape(-1, 3)
    X = Ocoord[:, 0:1] - Icoord[None, :, 0]
    Y = Ocoord[:, 1:2] - Icoord[None, :, 1]
    Z = Ocoord[:, 2:3] - Icoord[None, :, 2]
    R2 = X * X + Y * Y + Z * Z
    R = np.sqrt(R2)
    R3 = R * R2
    chi = 1j * omega * MU0 * np.exp(-1j * ko * R) / (4 * np.pi * ko * ko * R3)
    P = 1j * ko * R + 1
    Q = ko * ko * R2 - P
    P = (Q - 2 * P) / R2
    Q = chi * Q
    P = chi * P
    E = np.zeros((Ocoord.shape[0], 3), dtype=complex)
    E[:, 0] = (P * X * X - Q) @ J[:, 0] + (P * (X * Y)) @ J[:, 1] + (P * (X * Z)) @ J[:, 2]
    E[:, 1] = (P * (X * Y)) @ J[:, 0] + (P * (Y * Y) - Q) @ J[:, 1] + (P * (Y * Z)) @ J[:, 2]
    E[:, 2] = (P * (X * Z)) @ J[:, 0] + (P * (Y * Z)) @ J[:, 1] + (P * (Z * Z) - Q) @ J[:, 2]
    return E


def Dipole_Excitation(r, ko, DipJ, DipCoord):
    """src_vie/src_fields/src_excitations/Dipole_Excitation.m:39-54 (E only)."""
    L, M, N, _ = r.shape
    O = r.reshape((L * M * N, 3), order="F")
    E = E_field_DGF(DipJ, np.asarray(DipCoord, dtype=float).reshape(-1, 3), O, ko)
    return E.reshape((L, M, N, 3), order="F")


# ---------------------------------------------------------------------------
# operator assembly: src_vie/src_operators/*
# ---------------------------------------------------------------------------
def gauss_1d(n):
    """cubatures/gauss_1d.m: Gauss-Legendre on [-1,1], ascending (pinned to the table)."""
    x, w = np.polynomial.legendre.leggauss(n)
    return w, x


def gauss_2d(n):
    """cubatures/gauss_2d.m:1-19."""
    w1, x1 = gauss_1d(n)
    W = np.outer(w1, w1).reshape(-1) / 4
    U = np.repeat((x1 + 1) / 2, n)
    V = np.tile((x1 + 1) / 2, n)
    return n * n, W, U, V


def cube_faces(dx, dy, dz):
    """cube_faces.m:4-38 -> R_faces[3, 4, 6] (coordinate, corner, face)."""
    R = np.zeros((3, 4, 6))
    R[:, :, 0] = np.array([[0, 0, 0], [0, dy, 0], [0, dy, dz], [0, 0, dz]]).T
    R[:, :, 1] = np.array([[dx, 0, 0], [dx, dy, 0], [dx, dy, dz], [dx, 0, dz]]).T
    R[:, :, 2] = np.array([[0, 0, 0], [dx, 0, 0], [dx, 0, dz], [0, 0, dz]]).T
    R[:, :, 3] = np.array([[0, dy, 0], [dx, dy, 0], [dx, dy, dz], [0, dy, dz]]).T
    R[:, :, 4] = np.array([[0, 0, 0], [dx, 0, 0], [dx, dy, 0], [0, dy, 0]]).T
    R[:, :, 5] = np.array([[0, 0, dz], [dx, 0, dz], [dx, dy, dz], [0, dy, dz]]).T
    return R


INDEX_OBS = [0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 4, 4, 5]  # cubature_nop.cpp:24
INDEX_SRC = [0, 1, 2, 3, 4, 5, 0, 2, 3, 4, 5, 2, 3, 4, 5, 2, 4, 5, 4, 5, 4]  # cubature_nop.cpp:26
MIRROR = [((1, 1), (0, 0)), ((2, 0), (1, 3)), ((2, 1), (0, 3)), ((3, 0), (1, 2)), ((3, 1), (0, 2)),
          ((3, 3), (2, 2)), ((4, 0), (1, 5)), ((4, 1), (0, 5)), ((4, 2), (3, 5)), ((4, 3), (2, 5)),
          ((5, 0), (1, 4)), ((5, 1), (0, 4)), ((5, 2), (3, 4)), ((5, 3), (2, 4)), ((5, 5), (4, 4))]  # :100-115


def cubature_nop_batch(Np, w, u, v, r_m, R_faces, ko, dx):
    """cubature_nop.cpp:8-125 for a batch of observation offsets r_m (B x 3), r_n = 0.

    Returns I_mn of shape (B, 6, 6), already multiplied by dx^4."""
    r_m = np.atleast_2d(r_m)
    B = r_m.shape[0]
    I = np.zeros((B, 6, 6), dtype=complex)
    W = np.outer(w, w)
    for io, isrc in zip(INDEX_OBS, INDEX_SRC):
        p1, p2, p4 = R_faces[:, 0, io], R_faces[:, 1, io], R_faces[:, 3, io]
        q1, q2, q4 = R_faces[:, 0, isrc], R_faces[:, 1, isrc], R_faces[:, 3, isrc]
        rp = p1[None, :] + np.outer(u, p2 - p1) + np.outer(v, p4 - p1)  # Np x 3
        rq = q1[None, :] + np.outer(u, q2 - q1) + np.outer(v, q4 - q1)
        d = rq[None, None, :, :] - (rp[None, :, None, :] + r_m[:, None, None, :])  # B x Np x Np x 3
        R = np.sqrt(np.sum(d * d, axis=-1))
        # coincident points of a face with itself give 1/0 here, as in the
        # C++ core; those entries are replaced by the singular integrals later
        with np.errstate(divide="ignore", invalid="ignore"):
            G = np.exp(-1j * ko * R) / R
            I[:, io, isrc] = np.sum(W[None] * G, axis=(1, 2))
    for (a, b), (c, d_) in MIRROR:
        I[:, a, b] = I[:, c, d_]
    return dx**4 * I


def vector_projection():
    """vector_projection.m:10-25 -> P[6, 6, 6]."""
    e = np.eye(3)
    KL = np.array([-e[0], e[0], -e[1], e[1], -e[2], e[2]])
    comps = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
    P = np.zeros((6, 6, 6))
    for kk in range(6):
        for ll in range(6):
            for c, (a, b) in enumerate(comps):
                P[kk, ll, c] = np.dot(np.cross(KL[kk], e[a]), np.cross(KL[ll], e[b]))
    return P


def near_class(m, i, j):
    """Geometric class of face pair (obs face i of the voxel at offset m in {0,1}^3,
    src face j at the origin): 0 regular, 1 ST, 2 EAc, 3 EAo, 4 VAc, 5 VAo.  This
    restates the C/P tables of nearby_correct.m:5-143 (pinned by a fixture)."""
    ai, si, aj, sj = i // 2, i % 2, j // 2, j % 2
    if ai == aj:
        if m[ai] + si != sj:
            return 0
        shifted = sum(m[b] for b in range(3) if b != ai)
        return 1 if shifted == 0 else (2 if shifted == 1 else 4)
    ci, cj = m[ai] + si, sj
    if not (m[aj] <= cj <= m[aj] + 1) or not (0 <= ci <= 1):
        return 0
    b = 3 - ai - aj
    return 3 if m[b] == 0 else 5


def nearby_correct(m, I_non, sing):
    """nearby_correct.m: replace the weakly singular pairs with sing[cls-1]."""
    J = I_non.copy()
    for i in range(6):
        for j in range(6):
            c = near_class(m, i, j)
            if c:
                J[i, j] = sing[c - 1]
    return J


@functools.lru_cache(maxsize=64)
def _directfn_cached(ko, dx, n):
    from . import directfn

    return directfn.singular_integrals(ko, dx, n)


def singular_integrals(ko, dx, method="DIRECTFN", n=None):
    """{ST, EAc, EAo, VAc, VAo} for cubic voxels of edge dx.  'DIRECTFN' (the
    reference default, getOPERATORS.m:39-41) restates singular_st/ea/va.m at
    Np_1D = n (default 20, assembly_nop.m:16) in oracle/directfn.py;
    'CONVERGED' is the converged quadrature of singular_integrals_converged
    (not a reference method)."""
    if method == "DIRECTFN":
        return _directfn_cached(float(ko), float(dx), int(n or 20)).copy()
    if method == "CONVERGED":
        return singular_integrals_converged(ko, dx, n or 32)
    raise ValueError("method must be 'DIRECTFN' or 'CONVERGED'")


def singular_integrals_converged(ko, a, n=32):
    """Weakly singular square-square integrals {ST, EAc, EAo, VAc, VAo} of
    exp(-j ko R)/R for voxel edge a, converged to machine precision (not the
    reference's DIRECTFN, which carries a truncation error of up to 3.4e-5 at
    Np_1D = 20).  Relative coordinates turn each into an integral of f(|u|)
    times hat-function weights; a Duffy substitution removes the 1/R point
    singularity at the origin."""
    x, w = np.polynomial.legendre.leggauss(n)
    x = (x + 1) / 2
    w = w / 2
    S, T = np.meshgrid(x, x, indexing="ij")
    W2 = np.outer(w, w)
    S3, T1, T2 = np.meshgrid(x, x, x, indexing="ij")
    W3 = np.einsum("i,j,k->ijk", w, w, w)
    k = ko

    def e2(s, t):
        rho = np.sqrt(1 + t * t)
        return np.exp(-1j * k * a * s * rho) / rho

    def e3(s, t1, t2):
        rho = np.sqrt(1 + t1 * t1 + t2 * t2)
        return np.exp(-1j * k * a * s * rho) / rho

    def f(R):
        return np.exp(-1j * k * R) / R

    a3 = a**3
    ST = 8 * a3 * np.sum(W2 * e2(S, T) * (1 - S) * (1 - S * T))
    p1 = a3 * np.sum(W2 * e2(S, T) * (S * (1 - S * T) + S * T * (1 - S)))
    U1, U2 = a + a * S, a * T
    p2 = a * a * np.sum(W2 * f(np.hypot(U1, U2)) * (2 * a - U1) * (a - U2))
    EAc = 2 * (p1 + p2)
    EAo = 2 * a3 * np.sum(W3 * e3(S3, T1, T2) * (S3 * (1 - S3 * T1) + S3 * (1 - S3) + S3 * (1 - S3 * T2)))
    q0 = 2 * a3 * np.sum(W2 * e2(S, T) * S * S * T)
    q1 = a * a * np.sum(W2 * f(np.hypot(a + a * S, a * T)) * (2 * a - (a + a * S)) * (a * T))
    q2 = a * a * np.sum(W2 * f(np.hypot(a + a * S, a + a * T)) * (2 * a - (a + a * S)) * (2 * a - (a + a * T)))
    VAc = q0 + 2 * q1 + q2
    s0 = a3 * np.sum(W3 * e3(S3, T1, T2) * (S3 * S3 * T1 + S3 * S3 + S3 * S3 * T2))
    U1, U2, U3 = a * S3, a + a * T1, a * T2
    s1 = a3 * np.sum(W3 * f(np.sqrt(U1**2 + U2**2 + U3**2)) * (2 * a - U2))
    VAo = s0 + s1
    return np.array([ST, EAc, EAo, VAc, VAo])


def assembly_nop(L, M, N, ko, dx, sing):
    """assembly_nop.m:7-136 -> G_mn (L, M, N, 6)."""
    R_faces = cube_faces(dx, dx, dx)
    J = np.zeros((L, M, N, 6, 6), dtype=complex)
    d = np.array([dx, dx, dx])
    # far: all offsets, 4-point rule (assembly_nop.m:37-59); batched over x
    Np, w, u, v = gauss_2d(4)
    for mz in range(N):
        for my in range(M):
            mx = np.arange(L)
            r_m = np.stack([mx * dx, np.full(L, my * dx), np.full(L, mz * dx)], axis=1)
            J[:, my, mz] = cubature_nop_batch(Np, w, u, v, r_m, R_faces, ko, dx)
    # medium: offsets 1..5 per axis with the 10-point rule (:67-83)
    Np, w, u, v = gauss_2d(10)
    for mx in range(min(5, L)):
        for my in range(min(5, M)):
            for mz in range(min(5, N)):
                J[mx, my, mz] = cubature_nop_batch(Np, w, u, v, np.array([mx, my, mz]) * d, R_faces, ko, dx)[0]
    # near: 20-point rule + singular corrections (:96-114)
    Np, w, u, v = gauss_2d(20)
    for mx in range(min(2, L)):
        for my in range(min(2, M)):
            for mz in range(min(2, N)):
                I_non = cubature_nop_batch(Np, w, u, v, np.array([mx, my, mz]) * d, R_faces, ko, dx)[0]
                J[mx, my, mz] = nearby_correct((mx, my, mz), I_non, sing)
    P = vector_projection()
    G = np.einsum("xyzij,ijk->xyzk", J, P)
    return G / (4 * np.pi)


# gperiodic_coeff_nop.m:4-30
_GP = {
    "L": [+1, -1, -1, +1, +1, +1], "M": [+1, -1, +1, +1, -1, +1], "N": [+1, +1, -1, +1, -1, +1],
    "LM": [+1, +1, -1, +1, -1, +1], "LN": [+1, -1, +1, +1, -1, +1], "MN": [+1, -1, -1, +1, +1, +1],
}


def circulant_nop(G):
    """circulant_nop.m:23-40 (block copies with the gperiodic coefficients)."""
    L, M, N, _ = G.shape
    C = np.zeros((2 * L, 2 * M, 2 * N, 6), dtype=complex)
    C[:L, :M, :N] = G
    for ii in range(6):
        C[L + 1:, :M, :N, ii] = G[L - 1:0:-1, :, :, ii] * _GP["L"][ii]
        C[:L, M + 1:, :N, ii] = G[:, M - 1:0:-1, :, ii] * _GP["M"][ii]
        C[:L, :M, N + 1:, ii] = G[:, :, N - 1:0:-1, ii] * _GP["N"][ii]
        C[L + 1:, M + 1:, :N, ii] = G[L - 1:0:-1, M - 1:0:-1, :, ii] * _GP["LM"][ii]
        C[L + 1:, :M, N + 1:, ii] = G[L - 1:0:-1, :, N - 1:0:-1, ii] * _GP["LN"][ii]
        C[:L, M + 1:, N + 1:, ii] = G[:, M - 1:0:-1, N - 1:0:-1, ii] * _GP["MN"][ii]
    C[L + 1:, M + 1:, N + 1:] = G[L - 1:0:-1, M - 1:0:-1, N - 1:0:-1]
    return C


# ---------------------------------------------------------------------------
# K operator: assembly_kop.m:7-120, cubature_kop.cpp:8-120,
# cubature_kop_near_sym.m:1-105, nearby_correct_kop.m:1-134,
# circulant_kop.m:1-41, gperiodic_coeff_kop.m:1-36
# ---------------------------------------------------------------------------
# cubature_kop.cpp:30-32: the 12 integrated (obs, src) face pairs and their signs
KOP_OBS = [0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5]
KOP_SRC = [0, 1, 0, 1, 2, 3, 2, 3, 4, 5, 4, 5]
KOP_SIGN = [1.0, -1.0, -1.0, 1.0, 1.0, -1.0, -1.0, 1.0, 1.0, -1.0, -1.0, 1.0]


def _kop_pair(Np, w, u, v, r_m, R_faces, ko, io, isrc):
    """sum over point pairs of w_p w_q G(R) (r_p - r_q), G = (1 - e^{-jkR}(1 + jkR)) / R^3,
    for observation offsets r_m (B x 3); returns (B, 3)."""
    p1, p2, p4 = R_faces[:, 0, io], R_faces[:, 1, io], R_faces[:, 3, io]
    q1, q2, q4 = R_faces[:, 0, isrc], R_faces[:, 1, isrc], R_faces[:, 3, isrc]
    rp = p1[None, :] + np.outer(u, p2 - p1) + np.outer(v, p4 - p1)
    rq = q1[None, :] + np.outer(u, q2 - q1) + np.outer(v, q4 - q1)
    d = (rp[None, :, None, :] + r_m[:, None, None, :]) - rq[None, None, :, :]  # B x Np x Np x 3
    R = np.sqrt(np.sum(d * d, axis=-1))
    with np.errstate(divide="ignore", invalid="ignore"):
        G = (1.0 - np.exp(-1j * ko * R) * (1.0 + 1j * ko * R)) / R**3
    W = np.outer(w, w)
    return np.einsum("bpq,bpqc->bc", W[None] * G, d)


def cubature_kop_batch(Np, w, u, v, r_m, R_faces, ko):
    """cubature_kop.cpp:8-120 (r_n = 0): IK_mn (B x 3), without the dx^4 factor."""
    r_m = np.atleast_2d(r_m)
    out = np.zeros((r_m.shape[0], 3), dtype=complex)
    for io, isrc, sg in zip(KOP_OBS, KOP_SRC, KOP_SIGN):
        out += sg * _kop_pair(Np, w, u, v, r_m, R_faces, ko, io, isrc)
    return out


def cubature_kop_near_sym(Np, w, u, v, r_m, m, R_faces, ko):
    """cubature_kop_near_sym.m:17-105 for one offset: the 21 unique face pairs
    with the 20-point rule, the 15 mirrored copies, nearby_correct_kop (the
    coincident pairs dropped) and the face-normal combination."""
    I = np.zeros((6, 6, 3), dtype=complex)
    rm = np.asarray(r_m, float)[None]
    for io, isrc in zip(INDEX_OBS, INDEX_SRC):
        I[io, isrc] = _kop_pair(Np, w, u, v, rm, R_faces, ko, io, isrc)[0]
    for (a, b), (c, d_) in MIRROR:
        I[a, b] = I[c, d_]
    I = nearby_correct_kop(m, I)
    J = np.zeros((6, 6), dtype=complex)
    for i in range(6):
        J[i] = (1.0 if i % 2 else -1.0) * I[i, :, i // 2]
    return np.array([np.sum(J[:, 2 * c + 1] - J[:, 2 * c]) for c in range(3)])


def nearby_correct_kop(m, I_non):
    """nearby_correct_kop.m:5-134: only the coincident (ST) face pairs are
    changed (to zero); every other pair keeps its 20-point value."""
    I = I_non.copy()
    for i in range(6):
        for j in range(6):
            if near_class(m, i, j) == 1:
                I[i, j] = 0.0
    return I


def assembly_kop(L, M, N, ko, dx):
    """assembly_kop.m:7-120 -> IK_mn (L, M, N, 3)."""
    R_faces = cube_faces(dx, dx, dx)
    K = np.zeros((L, M, N, 3), dtype=complex)
    d = np.array([dx, dx, dx])
    Np, w, u, v = gauss_2d(4)
    for mz in range(N):
        for my in range(M):
            mx = np.arange(L)
            r_m = np.stack([mx * dx, np.full(L, my * dx), np.full(L, mz * dx)], axis=1)
            K[:, my, mz] = cubature_kop_batch(Np, w, u, v, r_m, R_faces, ko)
    Np, w, u, v = gauss_2d(10)
    for mx in range(min(5, L)):
        for my in range(min(5, M)):
            for mz in range(min(5, N)):
                K[mx, my, mz] = cubature_kop_batch(Np, w, u, v, np.array([mx, my, mz]) * d, R_faces, ko)[0]
    Np, w, u, v = gauss_2d(20)
    for mx in range(min(2, L)):
        for my in range(min(2, M)):
            for mz in range(min(2, N)):
                K[mx, my, mz] = cubature_kop_near_sym(Np, w, u, v, np.array([mx, my, mz]) * d, (mx, my, mz),
                                                      R_faces, ko)
    return dx**4 / (1j * ko) ** 2 / (4 * np.pi) * K


# gperiodic_coeff_kop.m:4-34: component i of K is odd along axis i
_GPK = {"L": [-1, 1, 1], "M": [1, -1, 1], "N": [1, 1, -1], "LM": [-1, -1, 1], "LN": [-1, 1, -1],
        "MN": [1, -1, -1], "LMN": [-1, -1, -1]}


def circulant_kop(G):
    """circulant_kop.m:17-41."""
    L, M, N, _ = G.shape
    C = np.zeros((2 * L, 2 * M, 2 * N, 3), dtype=complex)
    C[:L, :M, :N] = G
    for ii in range(3):
        C[L + 1:, :M, :N, ii] = G[L - 1:0:-1, :, :, ii] * _GPK["L"][ii]
        C[:L, M + 1:, :N, ii] = G[:, M - 1:0:-1, :, ii] * _GPK["M"][ii]
        C[:L, :M, N + 1:, ii] = G[:, :, N - 1:0:-1, ii] * _GPK["N"][ii]
        C[L + 1:, M + 1:, :N, ii] = G[L - 1:0:-1, M - 1:0:-1, :, ii] * _GPK["LM"][ii]
        C[L + 1:, :M, N + 1:, ii] = G[L - 1:0:-1, :, N - 1:0:-1, ii] * _GPK["LN"][ii]
        C[:L, M + 1:, N + 1:, ii] = G[:, M - 1:0:-1, N - 1:0:-1, ii] * _GPK["MN"][ii]
        C[L + 1:, M + 1:, N + 1:, ii] = G[L - 1:0:-1, M - 1:0:-1, N - 1:0:-1, ii] * _GPK["LMN"][ii]
    return C


def mv_K(JIn0, fK, r_shape, idx, workers=None):
    """src_vie/src_mvp/mv_K.m:30-93: crop(IFFT(fK x FFT(J))) on the entries idx
    (the curl-type product out = [K3 J2 - K2 J3, K1 J3 - K3 J1, K2 J1 - K1 J2])."""
    LfK, MfK, NfK, _ = fK.shape
    L, M, N = r_shape[:3]
    s = (LfK, MfK, NfK)
    flat = np.zeros(L * M * N * 3, dtype=complex)
    flat[np.asarray(idx) - 1] = JIn0
    JIn = flat.reshape((L, M, N, 3), order="F")
    f1 = _fftn(JIn[:, :, :, 0], s, workers)
    f2 = _fftn(JIn[:, :, :, 1], s, workers)
    f3 = _fftn(JIn[:, :, :, 2], s, workers)
    o1 = fK[..., 2] * f2 - fK[..., 1] * f3
    o2 = fK[..., 0] * f3 - fK[..., 2] * f1
    o3 = fK[..., 1] * f1 - fK[..., 0] * f2
    JOut = np.zeros((L, M, N, 3), dtype=complex)
    for c, o in enumerate((o1, o2, o3)):
        JOut[:, :, :, c] = _ifftn(o, workers)[:L, :M, :N]
    return JOut.reshape(-1, order="F")[np.asarray(idx) - 1]


def H_field_Kop(J, fK, Gram, Hinc=None, workers=None):
    """src_vie/src_fields/src_op/H_field_Kop.m:46-77: Hinc + mv_K(J) / Gram."""
    if Hinc is None:
        Hinc = np.zeros_like(J)
    if not np.any(J):
        return Hinc
    L, M, N, _ = J.shape
    idx = np.arange(1, 3 * L * M * N + 1)
    H = mv_K(J.reshape(-1, order="F"), fK, J.shape, idx, workers).reshape((L, M, N, 3), order="F")
    return Hinc + H / Gram


def fft_operator(A, workers=None):
    """fft_operator.m:6-8."""
    return scipy.fft.fftn(A, axes=(0, 1, 2), workers=workers)


def getOPERATORS(r, f, op="N", typ="FFTofC", sing=None):
    """getOPERATORS.m:36-127 for op 'N' and 'K'.  sing = the five singular
    integrals of N (default: DIRECTFN at Np_1D = 20, as the reference's
    default singular = 'DIRECTFN' computes them, assembly_nop.m:96-98)."""
    dx = r[1, 0, 0, 0] - r[0, 0, 0, 0]
    ko = 2 * np.pi / 299792458 * f
    L, M, N, _ = r.shape
    if op == "K":
        T = assembly_kop(L, M, N, ko, dx)
        if typ == "T":
            return T
        C = circulant_kop(T)
        return C if typ == "C" else fft_operator(C)
    if op != "N":
        raise ValueError("op must be 'N' or 'K'")
    if sing is None:
        sing = singular_integrals(ko, dx)
    T = assembly_nop(L, M, N, ko, dx, sing)
    if typ == "T":
        return T
    C = circulant_nop(T)
    if typ == "C":
        return C
    return fft_operator(C)


# ---------------------------------------------------------------------------
# grid helpers (grid3d.m:35-61 layout: L x M x N x 3 voxel centres)
# ---------------------------------------------------------------------------
def jvie2solver(Vrhs, fVIE, tol, Vini=None, max_it=1000):
    """jvie2solver.m:35-77: an all-zero right-hand side is its own solution;
    otherwise bicgstab(fVIE, Vrhs, tol, max_it, [], [], Vini)."""
    if not np.any(Vrhs):
        return Vrhs.copy(), 0, 0.0, 0.0
    x, flag, relres, it, resvec = bicgstab(fVIE, Vrhs, tol, max_it, None, None, Vini)
    return x, flag, relres, it


def fVIEsolver_Assembly(RHBM, freq):
    """fVIEsolver_Assembly.m:41-196 without the GPU branch: e_r, Gram, the
    non-air DOFs and their coordinates (:54-71), the crop to one voxel around
    the non-air bounding box (:77-94) when it is below 70 % of the voxels or
    no operator for this frequency is cached (:100-122), Mr, Mc and tau3
    (:130-138), and the solver handle of jvie2solver (:196).  Returns
    (fVIEsolver, Gram, tau3, Scoord, (e_r, idxS3, fN)) with the cropped
    e_r, its 1-based DOF indices and the operator."""
    eo = EPS0
    omega = 2 * np.pi * freq
    r = RHBM["r"]
    e_r = RHBM["epsilon_r"] - 1j * RHBM["sigma_e"] / (eo * omega)
    dx = r[1, 0, 0, 0] - r[0, 0, 0, 0]
    Gram = dx**3
    L, M, N = e_r.shape
    ND = L * M * N
    idxS = np.flatnonzero(np.abs(e_r.reshape(-1, order="F") - 1) > 1e-12)
    Scoord = np.stack([r[..., a].reshape(-1, order="F")[idxS] for a in range(3)], axis=1)
    lims = []
    for a in range(3):
        c = r[..., a].reshape(-1, order="F")[idxS]
        lims.append((c.min() - dx, c.max() + dx))
    gx, gy, gz = r[:, 0, 0, 0], r[0, :, 0, 1], r[0, 0, :, 2]
    idxX = np.flatnonzero((gx >= lims[0][0]) & (gx <= lims[0][1]))
    idxY = np.flatnonzero((gy >= lims[1][0]) & (gy <= lims[1][1]))
    idxZ = np.flatnonzero((gz >= lims[2][0]) & (gz <= lims[2][1]))
    e_rnew = e_r[np.ix_(idxX, idxY, idxZ)]
    Lf, Mf, Nf = e_rnew.shape
    fN = RHBM.get("fN")
    if Lf * Mf * Nf < 0.7 * ND or fN is None or RHBM.get("freqfN") != freq:
        rnew = r[np.ix_(idxX, idxY, idxZ)]
        fN = getOPERATORS(rnew, freq)
        e_r = e_rnew
        L, M, N = e_r.shape
        ND = L * M * N
        idxS = np.flatnonzero(np.abs(e_r.reshape(-1, order="F") - 1) > 1e-12)
    idxS3 = np.concatenate([idxS, ND + idxS, 2 * ND + idxS]) + 1
    Mr = e_r / e_r
    Mc = (e_r - 1.0) / e_r
    tau = (1j * omega * eo * Mc).reshape(-1, order="F")[idxS]
    tau3 = np.concatenate([tau, tau, tau])
    fVIE = lambda J: mv_AN(J, fN, Mr, Mc, Gram, "notransp", idxS3)
    fVIEsolver = lambda Vrhs, tol, Vini=None: jvie2solver(Vrhs, fVIE, tol, Vini)
    return fVIEsolver, Gram, tau3, Scoord, (e_r, idxS3, fN)


def grid(L, M, N, dx, center=(0.0, 0.0, 0.0)):
    xs = (np.arange(L) - (L - 1) / 2) * dx + center[0]
    ys = (np.arange(M) - (M - 1) / 2) * dx + center[1]
    zs = (np.arange(N) - (N - 1) / 2) * dx + center[2]
    X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
    return np.stack([X, Y, Z], axis=3)
