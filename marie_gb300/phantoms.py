"""Seeded synthetic bodies and excitations for the J-VIE workloads.

The reference measures on MRI body models it ships as MAT files; the workloads
here are synthetic stand-ins with the stated shapes and value distributions:

  sphere       homogeneous sphere (homogensphere.m:76-97 semantics, strict '<')
  ellipsoids   a 20 x 15 x 25 cm outer ellipsoid holding n random axis-aligned
               ellipsoids (semi-axes 1-10 cm, eps_r ~ U[5, 80], sigma ~ U[0.02, 2]
               S/m), painted in order (homogenellipse.m:79-100 semantics); all
               lengths shrink by one factor when the grid span is smaller than
               the outer ellipsoid
  dipoles      z-directed unit Hertzian dipoles on a cylinder around the body

Grids are voxel centres (L, M, N, 3), column-major, centred on the origin
(grid3d.m:35-61 layout).  Complex permittivity e_r = eps_r - j sigma/(eps0 omega)
(Scat_Solver.m:144).
"""
from __future__ import annotations

import math

import numpy as np

MU0 = 4 * math.pi * 1e-7
C0 = 299792458.0
EPS0 = 1.0 / C0**2 / MU0
OUTER_SEMI_AXES = (0.10, 0.075, 0.125)


def grid(L, M, N, dx):
    xs = (np.arange(L) - (L - 1) / 2) * dx
    ys = (np.arange(M) - (M - 1) / 2) * dx
    zs = (np.arange(N) - (N - 1) / 2) * dx
    X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
    return np.asfortranarray(np.stack([X, Y, Z], axis=3))


def complex_permittivity(eps_r, sigma, freq):
    omega = 2 * math.pi * freq
    return eps_r - 1j * sigma / (EPS0 * omega)


def sphere(L, M, N, dx, radius, eps_r, sigma, freq):
    r = grid(L, M, N, dx)
    inside = np.sum(r * r, axis=3) < radius * radius
    er = np.ones((L, M, N), dtype=complex, order="F")
    er[inside] = complex_permittivity(eps_r, sigma, freq)
    return r, np.asfortranarray(er)


def ellipsoids(L, M, N, dx, n_ell, seed, freq):
    """Returns (r, e_r, scale): the outer ellipsoid and n_ell random inner ones."""
    rng = np.random.default_rng(seed)
    r = grid(L, M, N, dx)
    span = np.array([L, M, N]) * dx
    outer = np.array(OUTER_SEMI_AXES)
    scale = float(min(1.0, np.min(0.95 * span / (2 * outer))))
    outer = outer * scale
    eps = np.ones((L, M, N))
    sig = np.zeros((L, M, N))
    q = (r[..., 0] / outer[0]) ** 2 + (r[..., 1] / outer[1]) ** 2 + (r[..., 2] / outer[2]) ** 2
    body = q < 1.0
    eps[body] = rng.uniform(5, 80)
    sig[body] = rng.uniform(0.02, 2)
    for _ in range(n_ell):
        while True:  # centre uniformly inside the outer ellipsoid
            c = rng.uniform(-1, 1, 3)
            if np.sum(c * c) < 1.0:
                break
        c = c * outer
        ax = rng.uniform(0.01, 0.10, 3) * scale
        e = rng.uniform(5, 80)
        s = rng.uniform(0.02, 2)
        qi = (((r[..., 0] - c[0]) / ax[0]) ** 2 + ((r[..., 1] - c[1]) / ax[1]) ** 2
              + ((r[..., 2] - c[2]) / ax[2]) ** 2)
        m = (qi < 1.0) & body
        eps[m] = e
        sig[m] = s
    er = np.asfortranarray(complex_permittivity(eps, sig, freq).astype(complex))
    return r, er, scale


def dipole_ring(radius, heights, n_az, phase0=0.0):
    """Positions (K, 3) of z-directed dipoles: n_az azimuths x len(heights)."""
    pos = []
    for z in heights:
        for a in range(n_az):
            t = phase0 + 2 * math.pi * a / n_az
            pos.append((radius * math.cos(t), radius * math.sin(t), z))
    return np.array(pos, dtype=float)


def plane_wave_k(freq, direction=(0.0, 0.0, 1.0)):
    ko = 2 * math.pi * freq / C0
    d = np.asarray(direction, dtype=float)
    return ko * d / np.linalg.norm(d)
