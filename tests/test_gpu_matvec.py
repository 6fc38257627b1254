"""GPU parity of the circulant matvecs (mv_AN both flags, mv_L) against the
oracle restatement of mv_AN.m / mv_L.m.  Bar: FP64 within 1e-12 and FP32
within 1e-5 of max|out| (relative, max norm)."""
import numpy as np
import pytest

from oracle import vie_oracle as vo

pytestmark = pytest.mark.gpu

LENGTHS = [8, 16, 24, 32, 40, 48, 64, 80, 96, 128, 160, 192, 256, 320, 384, 512]
TOL = {"fp64": 1e-12, "fp32": 1e-5}


def problem(L, M, N, seed=0, frac=0.6, physical=False):
    rng = np.random.default_rng(seed)
    if physical:
        G = rng.standard_normal((L, M, N, 6)) + 1j * rng.standard_normal((L, M, N, 6))
        G[0, :, :, [1, 2]] = 0
        G[:, 0, :, [1, 4]] = 0
        G[:, :, 0, [2, 4]] = 0
        fN = vo.fft_operator(vo.circulant_nop(G))
    else:
        fN = rng.standard_normal((2 * L, 2 * M, 2 * N, 6)) + 1j * rng.standard_normal((2 * L, 2 * M, 2 * N, 6))
    Mr = 1 + 40 * rng.random((L, M, N)) - 20j * rng.random((L, M, N))
    Mc = (Mr - 1) / Mr
    mask = rng.random(L * M * N) < frac
    mask[0] = True
    idxS = np.nonzero(mask)[0] + 1
    V = L * M * N
    idx = np.concatenate([idxS, V + idxS, 2 * V + idxS])
    J = rng.standard_normal(idx.size) + 1j * rng.standard_normal(idx.size)
    return np.asfortranarray(fN), np.asfortranarray(Mr), np.asfortranarray(Mc), idx, J


def relerr(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b))


def shapes():
    out = []
    for n in LENGTHS:
        h = n // 2
        out += [(h, 4, 4), (4, h, 4), (4, 4, h)]
    return sorted(set(out))


@pytest.mark.parametrize("shape", shapes())
def test_mv_AN_every_fft_length_fp64(shape):
    import marie_gb300 as mg

    fN, Mr, Mc, idx, J = problem(*shape, seed=sum(shape))
    ref = vo.mv_AN(J, fN, Mr, Mc, 0.37, "notransp", idx)
    out = mg.mv_AN(J, fN, Mr, Mc, 0.37, "notransp", idx)
    assert relerr(out, ref) < TOL["fp64"]


@pytest.mark.parametrize("shape", [(4, 8, 12), (12, 20, 24), (16, 32, 40), (48, 12, 20), (80, 4, 96),
                                   (24, 160, 8), (8, 8, 256), (256, 8, 8)])
@pytest.mark.parametrize("flag", ["notransp", "transp"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_mv_AN_flags_and_precisions(shape, flag, precision):
    import marie_gb300 as mg

    fN, Mr, Mc, idx, J = problem(*shape, seed=7, physical=True)
    ref = vo.mv_AN(J, fN, Mr, Mc, 2e-7, flag, idx)
    op = mg.Operator.from_array(fN, precision="mixed")
    out = mg.mv_AN(J, op, Mr, Mc, 2e-7, flag, idx, precision=precision)
    assert relerr(out, ref) < TOL[precision]


def test_mv_L_matches_oracle():
    import marie_gb300 as mg

    L, M, N = 12, 16, 8
    fN, Mr, Mc, idx, J = problem(L, M, N, seed=3)
    full = np.arange(1, 3 * L * M * N + 1)
    Jf = np.random.default_rng(1).standard_normal(full.size) + 0j
    for ix, x in ((idx, J), (full, Jf)):
        ref = vo.mv_L(x, fN, (L, M, N), 0.5, ix)
        out = mg.mv_L(x, fN, None, 0.5, ix)
        assert relerr(out, ref) < 1e-12
        # mv_N.m: the same without the Gram term
        assert relerr(mg.mv_N(x, fN, None, ix), vo.mv_N(x, fN, (L, M, N), ix)) < 1e-12


def test_batched_rhs_and_device_pointers(cuda):
    import torch

    import marie_gb300 as mg

    L, M, N = 16, 12, 20
    fN, Mr, Mc, idx, J = problem(L, M, N, seed=11, physical=True)
    rng = np.random.default_rng(2)
    Jb = np.asfortranarray(rng.standard_normal((idx.size, 3)) + 1j * rng.standard_normal((idx.size, 3)))
    op = mg.Operator.from_array(fN, precision="fp64", nrhs_max=2)  # 3 rhs -> two chunks
    out = mg.mv_AN(Jb, op, Mr, Mc, 0.1, "notransp", idx)
    for c in range(3):
        ref = vo.mv_AN(Jb[:, c], fN, Mr, Mc, 0.1, "notransp", idx)
        assert relerr(out[:, c], ref) < 1e-12
    # device-resident inputs are used in place and give the same numbers
    td = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    outd = mg.mv_AN(td(J), op, torch.from_numpy(Mr).to(cuda), torch.from_numpy(Mc).to(cuda), 0.1, "notransp",
                    td(idx))
    outh = mg.mv_AN(J, op, Mr, Mc, 0.1, "notransp", idx)
    assert outd.is_cuda
    np.testing.assert_array_equal(outd.cpu().numpy(), outh)


def test_unsorted_sparse_idx():
    import marie_gb300 as mg

    L, M, N = 8, 8, 8
    fN, Mr, Mc, _, _ = problem(L, M, N)
    rng = np.random.default_rng(5)
    idx = rng.permutation(3 * L * M * N)[:500] + 1
    J = rng.standard_normal(idx.size) + 1j * rng.standard_normal(idx.size)
    ref = vo.mv_AN(J, fN, Mr, Mc, 0.2, "notransp", idx)
    out = mg.mv_AN(J, fN, Mr, Mc, 0.2, "notransp", idx)
    assert relerr(out, ref) < 1e-12


def test_empty_idx_and_bad_idx_errors():
    import marie_gb300 as mg

    L = M = N = 4
    fN, Mr, Mc, idx, J = problem(L, M, N)
    op = mg.Operator.from_array(fN)
    out = mg.mv_AN(np.zeros(0, complex), op, Mr, Mc, 1.0, "notransp", np.zeros(0, np.int64))
    assert out.shape == (0,)
    with pytest.raises(mg.MarieError, match="repeated"):
        mg.mv_AN(np.ones(2, complex), op, Mr, Mc, 1.0, "notransp", np.array([3, 3]))
    with pytest.raises(mg.MarieError, match="outside"):
        mg.mv_AN(np.ones(1, complex), op, Mr, Mc, 1.0, "notransp", np.array([3 * L * M * N + 1]))
    with pytest.raises(mg.MarieError):
        mg.Operator(6, 4, 4)  # padded length 12 is not built


def test_deterministic_fp64():
    import marie_gb300 as mg

    fN, Mr, Mc, idx, J = problem(16, 16, 16, seed=9)
    op = mg.Operator.from_array(fN)
    a = mg.mv_AN(J, op, Mr, Mc, 0.3, "notransp", idx)
    b = mg.mv_AN(J, op, Mr, Mc, 0.3, "notransp", idx)
    np.testing.assert_array_equal(a, b)


FUSED = [(32, 32, 4), (48, 48, 4), (64, 64, 8), (96, 96, 4), (128, 128, 4), (256, 192, 4)]


@pytest.mark.parametrize("shape", FUSED)
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_fused_xy_passes_match_oracle(shape, precision):
    """Grids with the cluster-fused x+y passes, both flags."""
    import marie_gb300 as mg

    fN, Mr, Mc, idx, J = problem(*shape, seed=3, physical=True)
    op = mg.Operator.from_array(fN, precision="mixed")
    for flag in ("notransp", "transp"):
        ref = vo.mv_AN(J, fN, Mr, Mc, 1e-7, flag, idx)
        out = mg.mv_AN(J, op, Mr, Mc, 1e-7, flag, idx, precision=precision)
        assert relerr(out, ref) < TOL[precision], flag


def test_fused_and_five_pass_paths_agree(monkeypatch):
    import marie_gb300 as mg

    fN, Mr, Mc, idx, J = problem(64, 64, 8, seed=4, physical=True)
    op_f = mg.Operator.from_array(fN)
    monkeypatch.setenv("MARIE_NO_FUSED", "1")
    op_u = mg.Operator.from_array(fN)
    a = mg.mv_AN(J, op_f, Mr, Mc, 1e-7, "notransp", idx)
    b = mg.mv_AN(J, op_u, Mr, Mc, 1e-7, "notransp", idx)
    assert relerr(a, b) < 1e-13


def test_cufft_comparison_matvec_matches_oracle(cuda):
    """The cuFFT build of the FP32 mv_AN (timed beside the hand-written one in
    bench.py) computes the same product."""
    import ctypes as C

    import torch

    import marie_gb300 as mg
    from marie_gb300 import _lib

    lib = _lib.load()
    for shape in ((12, 20, 24), (32, 32, 4)):
        fN, Mr, Mc, idx, J = problem(*shape, seed=5, physical=True)
        ref = vo.mv_AN(J, fN, Mr, Mc, 0.37, "notransp", idx)
        op = mg.Operator.from_array(fN, precision="mixed")
        out = np.zeros_like(ref)
        ms = C.c_float()
        vp = lambda a: C.c_void_p(a.ctypes.data)
        Jc, Mrf, Mcf, ix = (np.ascontiguousarray(J), np.asfortranarray(Mr), np.asfortranarray(Mc),
                            np.ascontiguousarray(idx.astype(np.int64)))
        _lib.check(lib.marie_mv_AN_cufft(op.plan, vp(Jc), vp(Mrf), vp(Mcf), 0.37, vp(ix), ix.size, vp(out),
                                         C.byref(ms)))
        assert relerr(out, ref) < 1e-5
        assert ms.value > 0
        op.close()


@pytest.mark.parametrize("shape", [(16, 16, 64), (32, 32, 4), (64, 64, 8), (12, 20, 8)])
def test_autotuner_candidates_all_match_oracle(shape):
    """Every schedule the autotuner chooses from (fused or five-pass; wide or
    narrow z radix; 8 or 4 z columns per CTA) gives the FP32 product, and the
    tuner keeps the fastest of the ones it timed."""
    import marie_gb300 as mg

    fN, Mr, Mc, idx, J = problem(*shape, seed=13, physical=True)
    ref = vo.mv_AN(J, fN, Mr, Mc, 0.2, "notransp", idx)
    op = mg.Operator.from_array(fN, precision="mixed")
    chosen, cands = op.autotune()
    assert cands and min(c[3] for c in cands) == [c[3] for c in cands if c[:3] == chosen][0]
    for f, fv, z, _ in cands:
        op.set_schedule(f, fv, z)
        out = mg.mv_AN(J, op, Mr, Mc, 0.2, "notransp", idx, precision="fp32")
        assert relerr(out, ref) < TOL["fp32"], (f, fv, z)
    op.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_transpose_is_Mc_similarity_on_device(precision):
    """N is complex symmetric, so A^T = Gram*Mr - N*Mc = Mc^-1 A Mc: the
    'transp' flag (A^T x = conj(A^H conj(x))) against 'notransp' on Mc x, for
    a random parity-symmetric circulant and for the device-assembled operator.
    Two products and a division by Mc (|Mc| >= 0.08 here): FP32 bar 1e-4."""
    import marie_gb300 as mg

    L, M, N, dx = 12, 20, 16, 5e-3  # FFT lengths 24, 40, 32
    rng = np.random.default_rng(11)
    Mr = np.asfortranarray(5 + 40 * rng.random((L, M, N)) - 20j * rng.random((L, M, N)))
    Mc = np.asfortranarray((Mr - 1) / Mr)
    V = L * M * N
    idxS = np.flatnonzero(rng.random(V) < 0.6) + 1
    idx = np.concatenate([idxS, V + idxS, 2 * V + idxS]).astype(np.int64)
    x = rng.standard_normal(idx.size) + 1j * rng.standard_normal(idx.size)
    mc = Mc.reshape(-1, order="F")[(idx - 1) % V]
    fN = problem(L, M, N, seed=4, physical=True)[0]
    tol = {"fp64": 1e-12, "fp32": 1e-4}[precision]
    for op, gram in ((mg.Operator.from_array(fN, precision="mixed"), 0.4),
                     (mg.Operator.assemble(L, M, N, dx, 298e6, precision="mixed"), dx**3)):
        ATx = np.conj(mg.mv_AN(np.conj(x), op, Mr, Mc, gram, "transp", idx, precision=precision))
        sim = mg.mv_AN(mc * x, op, Mr, Mc, gram, "notransp", idx, precision=precision) / mc
        assert relerr(sim, ATx) < tol
        op.close()
