"""Body models for the J-VIE solve: Import_RHBM (src_geometry/src_scat/Import_RHBM.m:1).

A body is described by a .vmm file (line 1: the model name, line 2: the data
file) and a MATLAB MAT v5 file holding r (L x M x N x 3 voxel centres),
epsilon_r, sigma_e and rho.  The reference also reads a voxel .dat format
through a MEX parser (RHBMDat_ParseMEX); that format and MAT v7.3 (HDF5) files
are not read here.  Host-side data preparation only (numpy / scipy.io).
"""
from __future__ import annotations

import os

import numpy as np


def _nearest(axis_vals, q):
    """Index of the nearest grid line of axis_vals (sorted) for each query q,
    -1 outside [axis_vals[0], axis_vals[-1]] (interp3 'nearest' returns NaN
    there); ties go to the higher line."""
    a = np.asarray(axis_vals, dtype=np.float64)
    tol = 1e-9 * (a[-1] - a[0] if a.size > 1 else 1.0)
    j = np.clip(np.searchsorted(a, q), 1, max(a.size - 1, 1))
    lo = a[j - 1]
    hi = a[np.minimum(j, a.size - 1)]
    idx = np.where((q - lo) < (hi - q), j - 1, np.minimum(j, a.size - 1))
    out = (q < a[0] - tol) | (q > a[-1] + tol)
    return np.where(out, -1, idx)


def _resample(V, x, y, z, xq, yq, zq):
    """V sampled at the grid (xq, yq, zq) by nearest neighbour; NaN -> 0
    (Import_RHBM.m:116-126)."""
    ix, iy, iz = _nearest(x, xq), _nearest(y, yq), _nearest(z, zq)
    out = np.zeros((xq.size, yq.size, zq.size), dtype=np.float64, order="F")
    vx, vy, vz = ix >= 0, iy >= 0, iz >= 0
    sub = np.asarray(V, dtype=np.float64)[np.ix_(ix[vx], iy[vy], iz[vz])]
    out[np.ix_(vx, vy, vz)] = sub
    return out


def Import_RHBM(vmmfile, resolution=None, xlimits=None, ylimits=None, zlimits=None):
    """Import_RHBM.m:1-150: reads the body, fits it to a regular grid of
    spacing `resolution` (default: the smallest spacing of the file's grid)
    over the given limits (default: the file's extent), nearest-neighbour
    resampling with air outside the file's grid, and zero density in air.
    Returns a dict with name, r, epsilon_r, sigma_e, rho, idxS (1-based
    non-air indices) and empty operator caches (fN, freqfN, fK, freqfK)."""
    with open(vmmfile) as f:
        lines = [ln.strip() for ln in f.read().splitlines()]
    name, data = lines[0], lines[1]
    if not data.endswith(".mat"):
        raise ValueError(f"unsupported body data file {data!r}: only MAT v5 .mat files are read")
    path = data if os.path.isabs(data) else os.path.join(os.path.dirname(os.path.abspath(vmmfile)), data)
    import scipy.io as sio

    try:
        d = sio.loadmat(path)
    except NotImplementedError as e:  # MAT v7.3 (HDF5)
        raise ValueError(f"{path}: MAT v7.3 (HDF5) body files are not read; save as MAT v5") from e
    r0 = np.asarray(d["r"], dtype=np.float64)
    x, y, z = (np.unique(r0[..., a]) for a in range(3))
    eps, sig, rho = d["epsilon_r"], d["sigma_e"], d["rho"]
    xmin, xmax = (x.min(), x.max()) if xlimits is None else (min(xlimits), max(xlimits))
    ymin, ymax = (y.min(), y.max()) if ylimits is None else (min(ylimits), max(ylimits))
    zmin, zmax = (z.min(), z.max()) if zlimits is None else (min(zlimits), max(zlimits))
    if resolution is None:
        dx = min(np.diff(x).min(), np.diff(y).min(), np.diff(z).min())
    else:
        dx = float(resolution)
    nX, nY, nZ = (int(np.ceil((hi - lo) / dx)) for lo, hi in ((xmin, xmax), (ymin, ymax), (zmin, zmax)))
    xn = xmin + dx * np.arange(nX + 1)
    yn = ymin + dx * np.arange(nY + 1)
    zn = zmin + dx * np.arange(nZ + 1)
    r = np.zeros((xn.size, yn.size, zn.size, 3), order="F")
    r[..., 0], r[..., 1], r[..., 2] = np.meshgrid(xn, yn, zn, indexing="ij")
    epsilon_r = _resample(np.asarray(eps, dtype=np.float64) - 1.0, x, y, z, xn, yn, zn) + 1.0
    sigma_e = _resample(sig, x, y, z, xn, yn, zn)
    rho = _resample(rho, x, y, z, xn, yn, zn)
    flat = lambda a: a.reshape(-1, order="F")
    idxS = np.flatnonzero(np.abs(flat(epsilon_r) - 1 + 1j * flat(sigma_e)) > 1e-20)
    air = np.setdiff1d(np.flatnonzero(np.abs(flat(rho)) > 1e-20), idxS)
    rho_f = flat(rho).copy()
    rho_f[air] = 0
    rho = rho_f.reshape(rho.shape, order="F")
    return {"name": name, "r": r, "epsilon_r": np.asfortranarray(epsilon_r), "sigma_e": np.asfortranarray(sigma_e),
            "rho": np.asfortranarray(rho), "idxS": idxS + 1, "freqfN": None, "freqfK": None, "fN": None,
            "fK": None}
