"""Host buffers through the C ABI: pageable arrays of 8 MB and more travel
through the library's pinned ring (host threads fill 4 MB chunks that the
copy engine moves), pinned and smaller arrays are copied directly, device
arrays are used in place.  Every route must give the same bits as the
device-resident call, for sizes that are not whole chunks, and when several
plans transfer at once from different threads."""
import ctypes as C
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
FREQ = 298e6


def _problem(L, drop, seed):
    rng = np.random.default_rng(seed)
    V = L**3
    Mr = np.asfortranarray(1 + 40 * rng.random((L, L, L)) - 20j * rng.random((L, L, L)))
    Mc = np.asfortranarray((Mr - 1) / Mr)
    keep = np.sort(rng.permutation(V)[: V - drop]) + 1
    idx = np.concatenate([keep, V + keep, 2 * V + keep]).astype(np.int64)
    J = rng.standard_normal(idx.size) + 1j * rng.standard_normal(idx.size)
    return Mr, Mc, idx, J


def _call(op, J, Mr, Mc, idx, out, flag=0):
    from marie_gb300 import _lib

    ptr = lambda a: C.c_void_p(a.data_ptr() if hasattr(a, "data_ptr") else a.ctypes.data)
    _lib.check(op.lib.marie_mv_AN(op.plan, ptr(J), ptr(Mr), ptr(Mc), 0.25, flag, ptr(idx), len(idx), ptr(out), 1,
                                  _lib.MARIE_FP64))


def test_pageable_pinned_and_device_buffers_give_the_same_bits():
    import torch

    import marie_gb300 as mg

    L = 80
    Mr, Mc, idx, J = _problem(L, drop=12345, seed=3)  # J: 24 MB, not a whole number of 4 MB chunks
    assert J.nbytes >= 8 << 20 and J.nbytes % (4 << 20) != 0
    op = mg.Operator.assemble(L, L, L, 2e-3, FREQ, precision="fp64")
    dev = torch.device("cuda")
    Jd, Mrd, Mcd, idd = (torch.from_numpy(np.asfortranarray(a).reshape(-1, order="F")).to(dev)
                         for a in (J, Mr, Mc, idx))
    outd = torch.empty(idx.size, dtype=torch.complex128, device=dev)
    _call(op, Jd, Mrd, Mcd, idd, outd)
    ref = outd.cpu().numpy()
    # pageable in and out (the pinned ring), twice: the ring is reused
    for _ in range(2):
        out = np.full(idx.size, np.nan + 0j)
        _call(op, J, Mr, Mc, idx, out)
        np.testing.assert_array_equal(out, ref)
    # a fresh, never-touched output
    out = np.empty(idx.size, complex)
    _call(op, J, Mr, Mc, idx, out)
    np.testing.assert_array_equal(out, ref)
    # pinned host buffers are copied directly
    pin = lambda a: torch.from_numpy(np.asfortranarray(a).reshape(-1, order="F").copy()).pin_memory()
    outp = torch.zeros(idx.size, dtype=torch.complex128).pin_memory()
    _call(op, pin(J), pin(Mr), pin(Mc), pin(idx), outp)
    np.testing.assert_array_equal(outp.numpy(), ref)
    # pageable input, device output, and the reverse
    outd.zero_()
    _call(op, J, Mr, Mc, idx, outd)
    np.testing.assert_array_equal(outd.cpu().numpy(), ref)
    out = np.zeros(idx.size, complex)
    _call(op, Jd, Mrd, Mcd, idd, out)
    np.testing.assert_array_equal(out, ref)
    op.close()


def test_concurrent_plans_share_the_ring():
    import marie_gb300 as mg

    L = 64
    ops = [mg.Operator.assemble(L, L, L, 2e-3, FREQ, precision="fp64") for _ in range(3)]
    probs = [_problem(L, drop=777 * (k + 1), seed=10 + k) for k in range(3)]
    refs = []
    for op, (Mr, Mc, idx, J) in zip(ops, probs):
        out = np.empty(idx.size, complex)
        _call(op, J, Mr, Mc, idx, out, flag=1)
        refs.append(out)
    outs = [[None] * 4 for _ in ops]
    errors = []

    def run(k):
        try:
            Mr, Mc, idx, J = probs[k]
            for rep in range(4):
                out = np.empty(idx.size, complex)
                _call(ops[k], J, Mr, Mc, idx, out, flag=1)
                outs[k][rep] = out
        except Exception as e:  # reported below, on the main thread
            errors.append(e)

    threads = [threading.Thread(target=run, args=(k,)) for k in range(3)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors
    for k in range(3):
        for rep in range(4):
            np.testing.assert_array_equal(outs[k][rep], refs[k])
    for op in ops:
        op.close()
