"""Body import (Import_RHBM.m) on synthetic MAT v5 files, and on the
reference's own body file when the reference tree is present (CPU)."""
import os

import numpy as np
import pytest

from marie_gb300.bodies import Import_RHBM

# the reference checkout: MARIE_REFERENCE, else a directory "reference" beside this repository
_REF_ROOT = os.environ.get("MARIE_REFERENCE") or os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                                                              os.pardir, "reference")
REF_BODY = os.path.join(_REF_ROOT, "data", "bodies", "Cube_side10cm.vmm")


def write_body(tmp_path, L=10, M=12, N=9, dx=4e-3, seed=0):
    sio = pytest.importorskip("scipy.io")
    x = (np.arange(L) - L / 2) * dx
    y = (np.arange(M) - M / 2) * dx
    z = (np.arange(N) - N / 2) * dx
    r = np.zeros((L, M, N, 3))
    r[..., 0], r[..., 1], r[..., 2] = np.meshgrid(x, y, z, indexing="ij")
    rng = np.random.default_rng(seed)
    inside = np.sum((r / (0.35 * np.array([L, M, N]) * dx)) ** 2, axis=3) < 1
    eps = np.where(inside, rng.integers(20, 80, size=inside.shape), 1).astype(np.uint8)
    sig = np.where(inside, rng.uniform(0.1, 1.0, size=inside.shape), 0.0)
    rho = rng.integers(1, 1100, size=inside.shape).astype(np.uint16)  # also in air: zeroed on import
    sio.savemat(tmp_path / "body.mat", {"r": r, "epsilon_r": eps, "sigma_e": sig, "rho": rho})
    (tmp_path / "body.vmm").write_text("Synthetic body\nbody.mat\n")
    return r, eps, sig, rho, inside


def test_import_native_resolution(tmp_path):
    r, eps, sig, rho, inside = write_body(tmp_path)
    R = Import_RHBM(str(tmp_path / "body.vmm"))
    L, M, N = eps.shape
    assert R["name"] == "Synthetic body"
    # the grid spans the file's extent at its smallest spacing (the last line
    # may fall one spacing beyond, as with MATLAB's ceil on the same doubles)
    sub = (slice(0, L), slice(0, M), slice(0, N))
    assert np.allclose(R["r"][sub], r, atol=1e-12)
    assert np.array_equal(R["epsilon_r"][sub], eps.astype(float))
    assert np.array_equal(R["sigma_e"][sub], sig)
    assert np.all(R["epsilon_r"][L:] == 1) and np.all(R["sigma_e"][:, M:] == 0)
    assert np.array_equal(R["rho"][sub], np.where(inside, rho, 0).astype(float))
    assert np.array_equal(R["idxS"] - 1, np.flatnonzero(np.pad(inside, [(0, s - d) for s, d in
                                                                          zip(R["epsilon_r"].shape, inside.shape)])
                                                        .reshape(-1, order="F")))


def test_import_coarser_resolution_and_limits(tmp_path):
    r, eps, sig, rho, inside = write_body(tmp_path, L=12, M=12, N=12, dx=3e-3, seed=1)
    R = Import_RHBM(str(tmp_path / "body.vmm"), resolution=6e-3)
    # every other grid line of the file: nearest neighbour is the line itself
    coarse = eps.astype(float)[::2, ::2, ::2]
    k = coarse.shape[0]
    assert np.array_equal(R["epsilon_r"][:k, :k, :k], coarse)
    # a line beyond the file's last one reads air (interp3 returns NaN there)
    assert np.all(R["epsilon_r"][k:] == 1) and np.all(R["rho"][k:] == 0)
    lim = [r[2, 0, 0, 0], r[9, 0, 0, 0]]
    R2 = Import_RHBM(str(tmp_path / "body.vmm"), xlimits=lim)
    dxf = np.diff(np.unique(r[..., 0])).min()
    assert np.isclose(R2["r"][0, 0, 0, 0], lim[0])
    assert R2["r"].shape[0] == int(np.ceil((lim[1] - lim[0]) / dxf)) + 1
    assert np.array_equal(R2["epsilon_r"][:8, :12, :12], eps.astype(float)[2:10])


def test_import_rejects_other_formats(tmp_path):
    (tmp_path / "b.vmm").write_text("b\nvoxels.dat\nx.dat\ny.dat\nz.dat\n")
    with pytest.raises(ValueError):
        Import_RHBM(str(tmp_path / "b.vmm"))


@pytest.mark.skipif(not os.path.exists(REF_BODY), reason="reference body files not present")
def test_import_reference_body():
    sio = pytest.importorskip("scipy.io")
    R = Import_RHBM(REF_BODY)
    d = sio.loadmat(os.path.join(os.path.dirname(REF_BODY), "Cube_side10cm.mat"))
    L, M, N = d["epsilon_r"].shape
    assert np.array_equal(R["epsilon_r"][:L, :M, :N], d["epsilon_r"].astype(float))
    assert np.array_equal(R["sigma_e"][:L, :M, :N], d["sigma_e"])
    assert np.abs(R["r"][:L, :M, :N] - d["r"]).max() < 1e-12
