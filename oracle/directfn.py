"""numpy restatement of the reference's DIRECTFN weakly singular integrals
(TEST INFRASTRUCTURE ONLY).

The reference evaluates the five square-square singular integrals of
exp(-j ko R)/R that `nearby_correct.m` needs (ST, EAc, EAo, VAc, VAo) by
splitting each square face into two triangles and calling the DIRECTFN cores
for constant basis functions on triangle pairs
(src_vie/src_operators/cubatures/singular_st.m:14-17, singular_ea.m:17-28,
singular_va.m:20-34), at Np_1D = 20 Gauss-Legendre points per dimension
(assembly_nop.m:16).  The method (Polimeridis & Mosig, IJNME 83, 2010;
Polimeridis, Vipiana, Mosig & Wilton, IEEE TAP 61(6), 2013) maps both
triangles onto the equilateral triangle (eta, xi) with vertices (-1, 0),
(1, 0), (0, sqrt 3), moves to polar-type relative coordinates, splits the
angular ranges into subdomains in which the radial limit is one straight
edge, and integrates all four dimensions with Gauss-Legendre rules; the
radial Jacobian cancels the 1/R singularity.

Restated here:
  directfn_st  coincident triangles      directfn_ws_st_const.cpp:48-183
  directfn_ea  edge-adjacent triangles   directfn_ws_ea_const.cpp:48-182
  directfn_va  vertex-adjacent triangles directfn_ws_va_const.cpp:47-243
and the MEX gateways' vertex order: the EA gateway passes the second
triangle as (r4, r2, r1) (directfn_ws_ea_const_mex.cpp:50), the VA gateway
as (r4, r5, r1) (directfn_ws_va_const_mex.cpp:51).  The subdomain limits and
the nesting of the rules are the reference's: they define the quadrature,
and another split would change its value at Np_1D = 20 by up to 3e-5.  Sums
are vectorised (another order than the reference's loops), which moves the
results by rounding only.
"""
from __future__ import annotations

import numpy as np

SQ3 = np.sqrt(3.0)
PI3 = np.pi / 3


def _gl(n):
    return np.polynomial.legendre.leggauss(n)


def _map(x, w, a, b):
    """Gauss-Legendre rule of [-1, 1] onto [a, b]; a and b broadcast against
    a trailing axis of len(x)."""
    a = np.asarray(a, float)[..., None]
    b = np.asarray(b, float)[..., None]
    h = (b - a) / 2.0
    return h * x + (b + a) / 2.0, h * w


def _point(tri, eta, xi):
    """Point of triangle tri at equilateral parameters (eta, xi)
    (barycentric weights: directfn_ws_st_const.cpp:542-555)."""
    w1 = (SQ3 * (1 - eta) - xi) / (2 * SQ3)
    w2 = (SQ3 * (1 + eta) - xi) / (2 * SQ3)
    w3 = xi / SQ3
    return [w1 * tri[0][c] + w2 * tri[1][c] + w3 * tri[2][c] for c in range(3)]


def _green(ko, P, Q):
    R = np.sqrt((P[0] - Q[0]) ** 2 + (P[1] - Q[1]) ** 2 + (P[2] - Q[2]) ** 2)
    return np.exp(-1j * ko * R) / R


def _jac(tri):
    """Area of tri over the equilateral triangle's area sqrt(3)."""
    a = tri[1] - tri[0]
    b = tri[2] - tri[0]
    return 0.5 * np.linalg.norm(np.cross(a, b)) / SQ3


def _tri(rs):
    return [np.asarray(r, float) for r in rs]


# ---------------------------------------------------------------------------
# coincident triangles: directfn_ws_st_const.cpp:48-183 (loops), :189-229
# (psi ranges), :233-287 (eta ranges), :291-464 (lambda limits), :468-515
# (rho rule), :519-538 (the three sub-triangle rotations)
# ---------------------------------------------------------------------------
# per subdomain m = 1..8: psi range in units of pi/3, eta-range kind, lambda-limit kind
_ST = [((0, 1), "01", 1), ((1, 2), "01", 2), ((2, 3), "a1_1", 2), ((2, 3), "0_a1", 3),
       ((0, 1), "a2_0", 1), ((0, 1), "m1_a2", 4), ((1, 2), "m10", 4), ((2, 3), "m10", 3)]


def _st_eta_range(kind, psi):
    one = np.ones_like(psi)
    if kind == "01":
        return 0 * one, one
    if kind == "m10":
        return -one, 0 * one
    if kind in ("a1_1", "0_a1"):
        b1 = np.tan(np.pi - psi) / SQ3
        a1 = (1 - b1) / (1 + b1)
        return (a1, one) if kind == "a1_1" else (0 * one, a1)
    b2 = np.tan(psi) / SQ3
    a2 = -(1 - b2) / (1 + b2)
    return (a2, 0 * one) if kind == "a2_0" else (-one, a2)


def _st_lambda(kind, psi, eta):
    return {1: (1 - eta) / np.cos(psi), 2: SQ3 * (1 - eta) / np.sin(psi),
            3: -(1 + eta) / np.cos(psi), 4: SQ3 * (1 + eta) / np.sin(psi)}[kind]


def _rotate(kk, eta, xi):
    if kk == 1:
        return eta, xi
    if kk == 2:
        return 0.5 - 0.5 * eta - SQ3 / 2 * xi, SQ3 / 2 + SQ3 / 2 * eta - 0.5 * xi
    return -0.5 - 0.5 * eta + SQ3 / 2 * xi, SQ3 / 2 - SQ3 / 2 * eta - 0.5 * xi


def directfn_st(r1, r2, r3, ko, n=20):
    """Coincident triangle (r1, r2, r3), constant basis (the gateway passes
    the vertices through, directfn_ws_st_const_mex.cpp:47)."""
    x, w = _gl(n)
    tri = _tri((r1, r2, r3))
    total = 0j
    for kk in (1, 2, 3):
        for (pa, pb), ekind, lkind in _ST:
            psi, wpsi = _map(x, w, pa * PI3, pb * PI3)            # (n,)
            ea, eb = _st_eta_range(ekind, psi)
            eta, weta = _map(x, w, ea, eb)                        # (n, n)
            ps = psi[:, None]
            lam, wlam = _map(x, w, 0.0, _st_lambda(lkind, ps, eta))   # (n, n, n)
            rho, wrho = _map(x, w, 0.0, lam)                      # (n, n, n, n)
            s, c = np.sin(ps)[..., None, None], np.cos(ps)[..., None, None]
            ep = np.broadcast_to(eta[..., None, None], rho.shape)
            xp = np.broadcast_to(lam[..., None] * s, rho.shape)
            eq, xq = rho * c + ep, -rho * s + xp
            P = _point(tri, *_rotate(kk, ep, xp))
            Q = _point(tri, *_rotate(kk, eq, xq))
            W = wpsi[:, None, None, None] * weta[..., None, None] * wlam[..., None] * wrho * s * rho
            total += np.sum(W * _green(ko, P, Q))
    return _jac(tri) ** 2 * total


# ---------------------------------------------------------------------------
# edge-adjacent triangles: directfn_ws_ea_const.cpp:48-182 (loops), :188-218
# (theta ranges), :224-260 (psi ranges), :266-456 (eta ranges and lambda
# limits), :462-498 (lambda rule), :504-546 (parameter points; B = 1, 2 flips
# the sign of eta on both triangles)
# ---------------------------------------------------------------------------
_EA_THETA = [(0.0, PI3), (PI3, np.pi / 2), (PI3, np.pi / 2), (np.pi / 2, np.pi), (0.0, np.pi / 2),
             (np.pi / 2, np.pi)]
_EA_PSI = ["0_B", "A_B", "0_A", "0_A", "B_h", "A_h"]


def _ea_psi_range(kind, th):
    A = np.arctan(np.sin(th) - SQ3 * np.cos(th))
    B = np.arctan(np.sin(th) + SQ3 * np.cos(th))
    z, h = np.zeros_like(th), np.full_like(th, np.pi / 2)
    return {"0_B": (z, B), "A_B": (A, B), "0_A": (z, A), "B_h": (B, h), "A_h": (A, h)}[kind]


def _ea_pieces(m, psi, th):
    """The eta pieces of subdomain m as (eta_a, eta_b, lambda-limit kind)."""
    z, o = np.zeros_like(psi), np.ones_like(psi)
    if m in (1, 2):
        g = np.tan(psi) / (np.sin(th) + SQ3 * np.cos(th))
        h = (1 - g) / (1 + g)
        return [(z, h, "L3"), (h, o, "L2")]
    if m == 3:
        h = SQ3 / np.tan(th)
        return [(z, h, "L3"), (h, o, "L1")]
    if m == 4:
        return [(z, o, "L1")]
    return [(z, o, "L2")]


def _ea_lambda(kind, psi, th, eta):
    if kind == "L3":
        return SQ3 * (1 + eta) / (np.cos(psi) * (np.sin(th) + SQ3 * np.cos(th)))
    if kind == "L2":
        return SQ3 * (1 - np.abs(eta)) / np.sin(psi)
    return SQ3 * (1 - np.abs(eta)) / (np.cos(psi) * (np.sin(th) - SQ3 * np.cos(th)))


def directfn_ea(tp, tq, ko, n=20):
    """Edge-adjacent triangles tp = (p1, p2, p3), tq = (q1, q2, q3) in the
    order the reference core receives them."""
    x, w = _gl(n)
    tp, tq = _tri(tp), _tri(tq)
    total = 0j
    for m in range(1, 7):
        th, wth = _map(x, w, *_EA_THETA[m - 1])                   # (n,)
        psi, wpsi = _map(x, w, *_ea_psi_range(_EA_PSI[m - 1], th))    # (n, n)
        th2 = np.broadcast_to(th[:, None], psi.shape)
        for ea, eb, lkind in _ea_pieces(m, psi, th2):
            eta, weta = _map(x, w, ea, eb)                        # (n, n, n)
            p3, t3 = psi[..., None], th2[..., None]
            lam, wlam = _map(x, w, 0.0, _ea_lambda(lkind, p3, t3, eta))   # (n, n, n, n)
            p4, t4, e4 = p3[..., None], t3[..., None], eta[..., None]
            W = (wth[:, None, None, None] * wpsi[..., None, None] * weta[..., None] * wlam
                 * np.cos(p4) * lam * lam)
            xp = lam * np.sin(p4)
            xq = lam * np.cos(p4) * np.sin(t4)
            eq0 = lam * np.cos(p4) * np.cos(t4) - e4
            for sgn in (1.0, -1.0):
                P = _point(tp, np.broadcast_to(sgn * e4, lam.shape), xp)
                Q = _point(tq, sgn * eq0, xq)
                total += np.sum(W * _green(ko, P, Q))
    return _jac(tp) * _jac(tq) * total


# ---------------------------------------------------------------------------
# vertex-adjacent triangles: directfn_ws_va_const.cpp:47-243 (theta_p,
# theta_q on [0, pi/3], psi split at atan(Lq/Lp), lambda^3 sin cos Jacobian),
# :249-266 (parameter points)
# ---------------------------------------------------------------------------
def directfn_va(tp, tq, ko, n=20):
    """Vertex-adjacent triangles tp, tq in the order the reference core
    receives them."""
    x, w = _gl(n)
    tp, tq = _tri(tp), _tri(tq)
    tp_, wtp = _map(x, w, 0.0, PI3)                              # (n,)
    Lp = 2 * SQ3 / (np.sin(tp_) + SQ3 * np.cos(tp_))
    Tp, Tq = np.meshgrid(tp_, tp_, indexing="ij")
    Wt = np.outer(wtp, wtp)
    LP, LQ = np.meshgrid(Lp, Lp, indexing="ij")
    split = np.arctan(LQ / LP)
    total = 0j
    for lo, hi, lim in ((np.zeros_like(split), split, "p"), (split, np.full_like(split, np.pi / 2), "q")):
        psi, wpsi = _map(x, w, lo, hi)                            # (n, n, n)
        lb = LP[..., None] / np.cos(psi) if lim == "p" else LQ[..., None] / np.sin(psi)
        lam, wlam = _map(x, w, 0.0, lb)                           # (n, n, n, n)
        p4 = psi[..., None]
        tp4, tq4 = Tp[..., None, None], Tq[..., None, None]
        P = _point(tp, lam * np.cos(p4) * np.cos(tp4) - 1.0, lam * np.cos(p4) * np.sin(tp4))
        Q = _point(tq, lam * np.sin(p4) * np.cos(tq4) - 1.0, lam * np.sin(p4) * np.sin(tq4))
        W = Wt[..., None, None] * wpsi[..., None] * wlam * lam ** 3 * np.sin(p4) * np.cos(p4)
        total += np.sum(W * _green(ko, P, Q))
    return _jac(tp) * _jac(tq) * total


# ---------------------------------------------------------------------------
# gateway vertex orders and the square-face sums
# ---------------------------------------------------------------------------
def mex_st(r1, r2, r3, ko, n):
    """mexdirectfn_ws_st_const(r1, r2, r3, ko, Np) (directfn_ws_st_const_mex.cpp:47)."""
    return directfn_st(r1, r2, r3, ko, n)


def mex_ea(r1, r2, r3, r4, ko, n):
    """mexdirectfn_ws_ea_const(r1, r2, r3, r4, ko, Np): the core receives
    (r1, r2, r3) and (r4, r2, r1) (directfn_ws_ea_const_mex.cpp:50)."""
    return directfn_ea((r1, r2, r3), (r4, r2, r1), ko, n)


def mex_va(r1, r2, r3, r4, r5, ko, n):
    """mexdirectfn_ws_va_const(r1, .., r5, ko, Np): the core receives
    (r1, r2, r3) and (r4, r5, r1) (directfn_ws_va_const_mex.cpp:51)."""
    return directfn_va((r1, r2, r3), (r4, r5, r1), ko, n)


def singular_st(n, ko, dx, dy):
    """singular_st.m:4-17 ('DIRECTFN')."""
    r1, r2, r3, r4 = (0, 0, 0), (dx, 0, 0), (dx, dy, 0), (0, dy, 0)
    return (mex_st(r1, r2, r3, ko, n) + mex_ea(r1, r3, r2, r4, ko, n) + mex_ea(r1, r3, r4, r2, ko, n)
            + mex_st(r1, r3, r4, ko, n))


def singular_ea(n, ko, dx, dy, dz):
    """singular_ea.m:4-28 ('DIRECTFN'): (EAc, EAo)."""
    r1, r2, r3, r4 = (0, 0, 0), (dx, 0, 0), (dx, dy, 0), (0, dy, 0)
    out = []
    for r5, r6 in (((2 * dx, 0, 0), (2 * dx, dy, 0)), ((dx, 0, dz), (dx, dy, dz))):
        out.append(mex_ea(r2, r3, r1, r5, ko, n) + mex_va(r3, r1, r2, r5, r6, ko, n)
                   + mex_va(r3, r4, r1, r2, r5, ko, n) + mex_va(r3, r4, r1, r5, r6, ko, n))
    return tuple(out)


def singular_va(n, ko, dx, dy, dz):
    """singular_va.m:4-34 ('DIRECTFN'): (VAc, VAo)."""
    r1, r2, r3, r4 = (0, 0, 0), (dx, 0, 0), (dx, dy, 0), (0, dy, 0)
    out = []
    for r5, r6, r7 in (((2 * dx, dy, 0), (2 * dx, 2 * dy, 0), (dx, 2 * dy, 0)),
                       ((dx, dy, dz), (dx, 2 * dy, dz), (dx, 2 * dy, 0))):
        out.append(mex_va(r3, r1, r2, r5, r6, ko, n) + mex_va(r3, r1, r2, r6, r7, ko, n)
                   + mex_va(r3, r4, r1, r5, r6, ko, n) + mex_va(r3, r4, r1, r6, r7, ko, n))
    return tuple(out)


def singular_integrals(ko, dx, n=20):
    """{ST, EAc, EAo, VAc, VAo} as assembly_nop.m:96-98 computes them
    (cubic voxels, Np_DEMCEM = 20 at assembly_nop.m:16)."""
    ST = singular_st(n, ko, dx, dx)
    EAc, EAo = singular_ea(n, ko, dx, dx, dx)
    VAc, VAo = singular_va(n, ko, dx, dx, dx)
    return np.array([ST, EAc, EAo, VAc, VAo])
