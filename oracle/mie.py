"""Mie series inside a lossy dielectric sphere (TEST INFRASTRUCTURE ONLY).

Restates scripts/vie_solver_mie/src_mie: MIE_SERIES.m:19-44,
polar_transmitted_field.m:1-60, calc_miecoef.m:9-17, calc_sphbessel.m:11-23,
calc_MNpot.m:8-47, calc_MNpot_bj.m:8-12, Spher2Cartes_field.m:4-6.  The field
is for a unit x-polarised plane wave travelling +z.
"""
from __future__ import annotations

import numpy as np
import scipy.special as sp

MU0 = 4 * np.pi * 1e-7
C0 = 299792458.0
EPS0 = 1.0 / C0**2 / MU0


def _sph(n, z):
    """calc_sphbessel.m: spherical j and h2 with the derivative form used there."""
    nd = np.concatenate([[n[0] - 1], n])
    bj = np.sqrt(np.pi / 2 / z) * sp.jv(nd + 0.5, z)
    bh = np.sqrt(np.pi / 2 / z) * sp.hankel2(nd + 0.5, z)
    dbj = z * bj[:-1] - n * bj[1:]
    dbh = z * bh[:-1] - n * bh[1:]
    return bj[1:], dbj, bh[1:], dbh


def _miecoef(n, ka, k1a, k1overk):
    """calc_miecoef.m:9-17 (cn, dn only)."""
    bje, dbje, bh, dbh = _sph(n, ka)
    bji, dbji, _, _ = _sph(n, k1a)
    den1 = k1overk**2 * bji * dbh - bh * dbji
    den2 = bji * dbh - bh * dbji
    cn = (bje * dbh - bh * dbje) / den2
    dn = k1overk * (bje * dbh - bh * dbje) / den1
    return cn, dn


def _series_terms(k, k1, a):
    """polar_transmitted_field.m:15-36 truncation loop."""
    cn = np.zeros(0, complex)
    dn = np.zeros(0, complex)
    n = np.zeros(0)
    tn = np.arange(1, 81, dtype=float)
    while True:
        c, d = _miecoef(tn, k * a, k1 * a, k1 / k)
        cn = np.concatenate([cn, c])
        dn = np.concatenate([dn, d])
        n = np.concatenate([n, tn])
        nn = n[-1]
        if nn > 100:
            break
        if abs(cn[0]) < 1e-6 or abs(dn[0]) < 1e-6:
            break
        if (abs(cn[-1] / cn[0] * (2 * nn + 1) / (nn**2 + nn)) < 1e-4
                and abs(dn[-1] / dn[0] * (2 * nn + 1) / (nn**2 + nn)) < 1e-4):
            break
        tn = np.arange(tn[-1] + 1, tn[-1] + 1 + 2 * len(tn))
    return n, cn, dn


def MIE_SERIES(r, Rad, Er, Se, freq):
    """MIE_SERIES.m:19-44 -> E (L, M, N, 3) inside the sphere, zero outside."""
    omega = 2 * np.pi * freq
    ko = omega / C0
    eps = Er - 1j * Se / (EPS0 * omega)
    k1 = ko * np.sqrt(eps)
    n, cn, dn = _series_terms(ko, k1, Rad)
    En = (-1j) ** n * (2 * n + 1) / (n * (n + 1))
    L, M, N, _ = r.shape
    E = np.zeros((L, M, N, 3), complex)
    pts = r.reshape(-1, 3, order="F")
    out = E.reshape(-1, 3, order="F")
    for q, (x, y, z) in enumerate(pts):
        rr = np.sqrt(x * x + y * y + z * z)
        if rr > Rad:
            continue
        phi = np.arctan2(y, x)
        theta = np.pi / 2 - np.arctan2(z, np.hypot(x, y))  # cart2sph elevation -> polar
        th = theta
        if th == 0:
            th += 1e-6
        if th == np.pi:
            th -= 1e-6
        rho = k1 * rr
        bj, dbj, _, _ = _sph(n, rho)
        ct, st = np.cos(th), np.sin(th)
        P0 = -sp.lpmv(0, n, ct)
        P1 = -sp.lpmv(1, n, ct)
        pin = P1 / st
        taun = -1 / st * (n * (n + 1) * abs(st) * P0 + ct * P1)
        Mo = np.array([0 * n, np.cos(phi) * pin * bj, -np.sin(phi) * taun * bj])
        Ne = np.array([np.cos(phi) * n * (n + 1) * st * pin * bj / rho, np.cos(phi) * taun * dbj / rho,
                       -np.sin(phi) * pin * dbj / rho])
        Et = (cn[None] * Mo + 1j * dn[None] * Ne) @ En
        s0, c0 = np.sin(theta), np.cos(theta)  # Spher2Cartes_field.m uses the un-nudged angle
        StoC = np.array([[s0 * np.cos(phi), c0 * np.cos(phi), -np.sin(phi)],
                         [s0 * np.sin(phi), c0 * np.sin(phi), np.cos(phi)],
                         [c0, -s0, 0.0]])
        out[q] = StoC @ Et
    return out.reshape((L, M, N, 3), order="F")
