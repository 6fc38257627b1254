"""marie_mv_AN_static, the matvec that allocates nothing (its scratch is a
static device array), against marie_mv_AN through the C ABI.  Two calls in a
row on each grid: the second reuses the array the first left behind, with a
different DOF set and flag.  Every static call runs with the library's
allocation-failure injector armed, so any device allocation inside it would
return MARIE_ENOMEM.  Bar: FP64 within 1e-12 and FP32 within 1e-5 of
max|out|, as for the matvec parity tests.  Collected last, so it runs both
after the other GPU tests and alone."""
import ctypes as C

import numpy as np
import pytest

from oracle import vie_oracle as vo

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "fp32": 1e-5}


def operator(L, M, N, seed):
    rng = np.random.default_rng(seed)
    G = rng.standard_normal((L, M, N, 6)) + 1j * rng.standard_normal((L, M, N, 6))
    G[0, :, :, [1, 2]] = 0
    G[:, 0, :, [1, 4]] = 0
    G[:, :, 0, [2, 4]] = 0
    return np.asfortranarray(vo.fft_operator(vo.circulant_nop(G)))


def case(L, M, N, seed, frac, cuda):
    import torch

    rng = np.random.default_rng(seed)
    V = L * M * N
    Mr = 1 + 40 * rng.random(V) - 20j * rng.random(V)
    Mc = (Mr - 1) / Mr
    mask = rng.random(V) < frac
    mask[seed % V] = True
    idxS = np.nonzero(mask)[0] + 1
    idx = np.concatenate([idxS, V + idxS, 2 * V + idxS]).astype(np.int64)
    J = rng.standard_normal(idx.size) + 1j * rng.standard_normal(idx.size)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    return dict(J=dev(J), Mr=dev(Mr), Mc=dev(Mc), idx=dev(idx), n=idx.size)


def call(fn, plan, c, transp, prec, out, gram=0.37):
    return fn(plan, C.c_void_p(c["J"].data_ptr()), C.c_void_p(c["Mr"].data_ptr()), C.c_void_p(c["Mc"].data_ptr()),
              gram, transp, C.c_void_p(c["idx"].data_ptr()), c["n"], C.c_void_p(out.data_ptr()), *prec)


def call_static_no_alloc(lib, plan, c, transp, prec, out):
    """The static entry point with the first device allocation set to fail."""
    lib.marie_inject_alloc_failure(1)
    try:
        return call(lib.marie_mv_AN_static, plan, c, transp, (prec,), out)
    finally:
        lib.marie_inject_alloc_failure(0)


@pytest.mark.parametrize("shape", [(16, 12, 20), (32, 32, 4), (40, 8, 24)])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_static_matvec_matches_mv_AN_on_two_calls(shape, precision, cuda):
    import torch

    import marie_gb300 as mg
    from marie_gb300 import _lib

    lib = _lib.load()
    p = _lib.MARIE_FP64 if precision == "fp64" else _lib.MARIE_FP32
    op = mg.Operator.from_array(operator(*shape, seed=sum(shape)), precision="mixed")
    calls = [(case(*shape, 1, 0.7, cuda), 0), (case(*shape, 2, 0.3, cuda), 1)]
    for c, transp in calls:
        ref = torch.zeros(c["n"], dtype=torch.complex128, device=cuda)
        out = torch.full((c["n"],), complex("nan"), dtype=torch.complex128, device=cuda)
        _lib.check(call(lib.marie_mv_AN, op.plan, c, transp, (1, p), ref))
        _lib.check(call_static_no_alloc(lib, op.plan, c, transp, p, out))
        torch.cuda.synchronize()
        r, o = ref.cpu().numpy(), out.cpu().numpy()
        assert np.all(np.isfinite(o))
        assert np.max(np.abs(o - r)) <= TOL[precision] * np.max(np.abs(r))
    op.close()


def test_static_matvec_rejects_oversize_grids_and_host_pointers(cuda):
    import torch

    import marie_gb300 as mg
    from marie_gb300 import _lib

    lib = _lib.load()
    # 64^3 in FP64 needs about 104 MB of scratch, beyond the 64 MiB array
    big = mg.Operator.from_array(operator(64, 64, 64, seed=3), precision="fp64")
    c = case(64, 64, 64, 4, 0.5, cuda)
    out = torch.zeros(c["n"], dtype=torch.complex128, device=cuda)
    st = call(lib.marie_mv_AN_static, big.plan, c, 0, (_lib.MARIE_FP64,), out)
    assert st == _lib.MARIE_EINVAL
    assert b"static array" in lib.marie_last_error()
    big.close()
    small = mg.Operator.from_array(operator(8, 8, 8, seed=5), precision="fp64")
    c = case(8, 8, 8, 6, 0.5, cuda)
    host = {k: (v.cpu() if k != "n" else v) for k, v in c.items()}
    out = torch.zeros(c["n"], dtype=torch.complex128)
    st = call(lib.marie_mv_AN_static, small.plan, host, 0, (_lib.MARIE_FP64,), out)
    assert st == _lib.MARIE_EINVAL
    assert b"device pointers" in lib.marie_last_error()
    small.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_static_matvec_follows_the_tuned_schedule(precision, cuda):
    """After marie_plan_set_schedule picks the non-default x/y and z-pass
    variants, the static entry point still matches marie_mv_AN (which runs
    them), with the allocation injector armed."""
    import torch

    import marie_gb300 as mg
    from marie_gb300 import _lib

    lib = _lib.load()
    p = _lib.MARIE_FP64 if precision == "fp64" else _lib.MARIE_FP32
    shape = (32, 32, 16)
    op = mg.Operator.from_array(operator(*shape, seed=7), precision="mixed")
    op.set_schedule(1, 1, 1)
    c = case(*shape, 8, 0.6, cuda)
    ref = torch.zeros(c["n"], dtype=torch.complex128, device=cuda)
    out = torch.full((c["n"],), complex("nan"), dtype=torch.complex128, device=cuda)
    _lib.check(call(lib.marie_mv_AN, op.plan, c, 0, (1, p), ref))
    _lib.check(call_static_no_alloc(lib, op.plan, c, 0, p, out))
    torch.cuda.synchronize()
    r, o = ref.cpu().numpy(), out.cpu().numpy()
    assert np.max(np.abs(o - r)) <= TOL[precision] * np.max(np.abs(r))
    op.close()
