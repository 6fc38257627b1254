"""The plan-bound mv_AN as the operator of pgmres / pgmresDR / bicgstab (the C
ABI's NULL operator) against the oracle with the same mv_AN handle."""
import numpy as np
import pytest

from oracle import vie_oracle as vo

pytestmark = pytest.mark.gpu
FREQ = 298e6


def system(L=8, dx=5e-3, radius=0.018):
    r = vo.grid(L, L, L, dx)
    er = np.ones((L, L, L), complex)
    er[np.sum(r * r, axis=3) < radius**2] = 50.0 - 30.0j
    er = np.asfortranarray(er)
    V = L * L * L
    idxS = np.flatnonzero(np.abs(er.reshape(-1, order="F") - 1) > 1e-12)
    idx = (np.concatenate([idxS, V + idxS, 2 * V + idxS]) + 1).astype(np.int64)
    Mr = np.asfortranarray(er / er)
    Mc = np.asfortranarray((er - 1) / er)
    fN = vo.getOPERATORS(r, FREQ)
    rng = np.random.default_rng(3)
    b = rng.standard_normal(idx.size) + 1j * rng.standard_normal(idx.size)
    return fN, Mr, Mc, dx**3, idx, b


@pytest.mark.parametrize("transp", ["notransp", "transp"])
def test_bound_mv_AN_in_krylov_solvers(transp):
    import marie_gb300 as mg

    fN, Mr, Mc, Gram, idx, b = system()
    op = mg.Operator.from_array(fN).bind_mv_AN(Mr, Mc, Gram, transp, idx)
    A = lambda v: vo.mv_AN(v, fN, Mr, Mc, Gram, transp, idx)
    ref = vo.pgmres(A, b, 10, 1e-10, 20)
    out = mg.pgmres(op, b, 10, 1e-10, 20)
    assert out[1] == ref[1] == 0 and out[3] == ref[3]
    np.testing.assert_allclose(out[4], ref[4], rtol=1e-6, atol=1e-14)
    assert np.linalg.norm(out[0] - ref[0]) <= 1e-8 * np.linalg.norm(ref[0])
    refb = vo.bicgstab(A, b, 1e-10, 200)
    outb = mg.bicgstab(op, b, 1e-10, 200)
    # BiCGSTAB's path follows the rounding of the FFTs (cuFFT-free device
    # transforms here, pocketfft in the oracle): same answer, counts close
    assert outb[1] == refb[1] == 0 and abs(outb[3] - refb[3]) <= 0.1 * refb[3] + 2
    assert np.linalg.norm(outb[0] - refb[0]) <= 1e-7 * np.linalg.norm(refb[0])
    refd = vo.pgmresDR(A, b, 10, 1e-10, 20, 3)
    outd = mg.pgmresDR(op, b, 10, 1e-10, 20, 3)
    assert outd[1] == refd[1] == 0 and outd[3] == refd[3]
    assert np.linalg.norm(outd[0] - refd[0]) <= 1e-8 * np.linalg.norm(refd[0])


def test_null_operator_needs_a_binding(cuda):
    import marie_gb300 as mg

    fN, Mr, Mc, Gram, idx, b = system()
    op = mg.Operator.from_array(fN)
    with pytest.raises(mg.MarieError):
        mg.pgmres(op, b, 10, 1e-8, 5)
    op.bind_mv_AN(Mr, Mc, Gram, "notransp", idx)
    with pytest.raises(mg.MarieError):
        mg.pgmres(op, b[:-3], 10, 1e-8, 5)
    with pytest.raises(ValueError):
        op.bind_mv_AN(Mr, Mc, Gram, "both", idx)


@pytest.mark.parametrize("transp", ["notransp", "transp"])
def test_apply_bound_mv_AN(cuda, transp):
    """marie_plan_apply_mv_AN: the bound mv_AN without a per-call DOF map; FP64
    gives the bits of marie_mv_AN, FP32 (epilogue in FP32 too) meets the FP32
    bar against the oracle; host and device vectors, two right-hand sides."""
    import torch

    import marie_gb300 as mg

    fN, Mr, Mc, Gram, idx, b = system(L=16, dx=3e-3, radius=0.02)
    rng = np.random.default_rng(8)
    J = np.asfortranarray(rng.standard_normal((idx.size, 2)) + 1j * rng.standard_normal((idx.size, 2)))
    op = mg.Operator.from_array(fN, precision="mixed", nrhs_max=2).bind_mv_AN(Mr, Mc, Gram, transp, idx)
    ref = np.stack([vo.mv_AN(J[:, c], fN, Mr, Mc, Gram, transp, idx) for c in range(2)], axis=1)
    scale = np.max(np.abs(ref))
    out64 = op.apply_mv_AN(J, "fp64")
    np.testing.assert_array_equal(out64, mg.mv_AN(J, op, Mr, Mc, Gram, transp, idx, precision="fp64"))
    assert np.max(np.abs(out64 - ref)) / scale < 1e-12
    out32 = op.apply_mv_AN(J, "fp32")
    assert np.max(np.abs(out32 - ref)) / scale < 1e-5
    Jd = torch.from_numpy(J[:, 0].copy()).to(cuda)
    outd = op.apply_mv_AN(Jd, "fp32")
    assert outd.is_cuda
    np.testing.assert_array_equal(outd.cpu().numpy(), out32[:, 0])
    op.close()
