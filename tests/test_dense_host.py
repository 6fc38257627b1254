"""CPU tests of the host-side dense linear algebra of the Krylov solvers
(marie_gb300/csrc/dense.h: least squares, thin QR, LU solve, eigenpairs), built
with g++ into a small driver and checked against numpy.  No GPU."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = tmp_path_factory.mktemp("dense") / "dense_driver"
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", str(ROOT / "marie_gb300" / "csrc"),
                    str(ROOT / "tests" / "dense_driver.cpp"), "-o", str(exe)], check=True)
    return exe


def run(driver, tmp_path, cmd, *mats):
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(fin, "wb") as f:
        for m in mats:
            m = np.asarray(m, dtype=complex).reshape(m.shape[0], -1)
            np.array(m.shape, dtype=np.int32).tofile(f)
            np.asfortranarray(m).ravel(order="F").view(np.float64).tofile(f)
    subprocess.run([str(driver), cmd, str(fin), str(fout)], check=True)
    out = []
    with open(fout, "rb") as f:
        while True:
            hdr = np.fromfile(f, dtype=np.int32, count=2)
            if hdr.size < 2:
                break
            r, c = int(hdr[0]), int(hdr[1])
            v = np.fromfile(f, dtype=np.float64, count=2 * r * c).view(complex)
            out.append(v.reshape((r, c), order="F"))
    return out


def rand(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


@pytest.mark.parametrize("n", [1, 2, 7, 30, 61])
def test_eig_matches_numpy(driver, tmp_path, n):
    rng = np.random.default_rng(n)
    A = rand(rng, n, n)
    w, V = run(driver, tmp_path, "eig", A)
    w = w[:, 0]
    # eigenpairs satisfy A v = w v with unit vectors, and the spectrum is numpy's
    assert np.allclose(np.linalg.norm(V, axis=0), 1.0)
    assert np.max(np.abs(A @ V - V * w)) < 1e-10 * np.linalg.norm(A)
    ref = np.linalg.eigvals(A)
    for lam in ref:
        assert np.min(np.abs(w - lam)) < 1e-9 * np.max(np.abs(ref))


def test_eig_hessenberg_plus_rank_one(driver, tmp_path):
    # the harmonic Ritz matrix of getHarmVecs1: H_m + h^2 f e_m^T
    rng = np.random.default_rng(5)
    m = 40
    H = np.triu(rand(rng, m + 1, m), -1)
    Hm = H[:m]
    f = np.linalg.solve(Hm.conj().T, np.eye(m)[:, -1])
    M = Hm.copy()
    M[:, -1] += H[m, m - 1] ** 2 * f
    w, V = run(driver, tmp_path, "eig", M)
    assert np.max(np.abs(M @ V - V * w[:, 0])) < 1e-9 * np.linalg.norm(M)


def test_lstsq_qr_solve_rdiv(driver, tmp_path):
    rng = np.random.default_rng(9)
    A = rand(rng, 31, 24)
    b = rand(rng, 31, 1)
    (x,) = run(driver, tmp_path, "lstsq", A, b)
    np.testing.assert_allclose(x[:, 0], np.linalg.lstsq(A, b[:, 0], rcond=None)[0], rtol=1e-10, atol=1e-12)
    Q, R = run(driver, tmp_path, "qr", A)
    np.testing.assert_allclose(Q @ R, A, atol=1e-12)
    np.testing.assert_allclose(Q.conj().T @ Q, np.eye(24), atol=1e-12)
    assert np.allclose(np.tril(R, -1), 0)
    S = rand(rng, 20, 20)
    B = rand(rng, 20, 3)
    (X,) = run(driver, tmp_path, "solve", S, B)
    np.testing.assert_allclose(X, np.linalg.solve(S, B), rtol=1e-9, atol=1e-11)
    U = np.triu(rand(rng, 6, 6)) + 4 * np.eye(6)
    C = rand(rng, 9, 6)
    (Y,) = run(driver, tmp_path, "rdiv", C, U)
    np.testing.assert_allclose(Y @ U, C, atol=1e-11)
