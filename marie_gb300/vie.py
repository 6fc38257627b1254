"""Reference-facing host API of the J-VIE solve path.

Mirrors the MATLAB functions of MARIE that this path replaces, with the same
argument order, defaults and return tuples:

    getOPERATORS(r, f, op, type, singular)       src_vie/src_operators/getOPERATORS.m:1
    mv_AN(JIn0, fN, Mr, Mc, Gram, transp_flag, idx, GPU_flag)
                                                 src_vie/src_mvp/mv_AN.m:1
    mv_L(JIn0, fN, r, Gram, idx, GPU_flag)       src_vie/src_mvp/mv_L.m:1
    mv_N(JIn0, fN, r, idx, GPU_flag)             src_vie/src_mvp/mv_N.m:1
    mv_K(JIn0, fK, r, idx, GPU_flag)             src_vie/src_mvp/mv_K.m:1
    H_field_Kop(J, fK, Gram, Hinc, GPU_flag)     src_vie/src_fields/src_op/H_field_Kop.m:1
    pgmres(A, b, restart, tol, maxit, L1, L2, R1, R2, x0)
                                                 src_numeric/src_iterative/pgmres.m:70
    pgmresDR(A, b, restart, tol, maxit, ritz, L1, L2, R1, R2, x0)
                                                 src_numeric/src_iterative/pgmresDR.m:1
    bicgstab(A, b, tol, maxit, M1, M2, x0)       MATLAB built-in, JVIE_Solver.m:451-499
    JVIE_Solver(Einc, e_r, r, freq, fN, tol, form, solver, precond, max_it,
                inner_it, outer_it, ritz, gpu_flag, logfile)
                                                 src_vie/src_solver/JVIE_Solver.m:1
    Scat_Solver(Einc, Hinc, freq, r, epsilon_r, sigma_e, rho, tol, fN, fK, form,
                solver, precond, max_it, inner_it, outer_it, ritz, gpu_flag, logfile)
                                                 src_vie/src_solver/Scat_Solver.m:1
    E_field_Nop(J, fN, Gram, freq, Einc, GPU_flag)
                                                 src_vie/src_fields/src_op/E_field_Nop.m:1
    fVIEsolver_Assembly(RHBM, freq, gpu_flag)    src_vie/src_solver/fVIEsolver_Assembly.m:1
    jvie2solver(Vrhs, ..., tol, Vini)            src_vie/src_solver/jvie2solver.m:1
    PlaneWave_Excitation(r, k, omega_mu, Eo)     src_vie/src_fields/src_excitations/PlaneWave_Excitation.m:1
    Dipole_Excitation(r, k, DipJ, DipCoord)      src_vie/src_fields/src_excitations/Dipole_Excitation.m:1

Grid arrays are (L, M, N[, 3 or 6]) in column-major order, exactly the
reference's MATLAB arrays: numpy arrays (host; copied to the device per call,
like gpuArray/gather) or torch CUDA tensors with column-major strides (used in
place).  idx vectors are 1-based.  All compute runs in libmarie_vie.so on the
GPU; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import math
import time
from typing import Callable, Optional

import numpy as np

from . import _lib, solvelog
from ._lib import MARIE_FP32, MARIE_FP64, MARIE_MIXED, check

try:  # torch is only needed for device-resident arrays
    import torch
except Exception:  # pragma: no cover
    torch = None

MU0 = 4 * math.pi * 1e-7
C0 = 299792458.0
EPS0 = 1.0 / C0**2 / MU0

_PREC = {"fp64": MARIE_FP64, "fp32": MARIE_FP32, "mixed": MARIE_MIXED,
         64: MARIE_FP64, 32: MARIE_FP32, 96: MARIE_MIXED}


def EMconstants(freq):
    """EMconstants.m:13-20."""
    omega = 2 * math.pi * freq
    return dict(mu=MU0, co=C0, eo=EPS0, omega=omega, lambda_=C0 / freq, ko=2 * math.pi * freq / C0,
                omega_mu=omega * MU0, eta=3.767303134617706e+002)


# ---------------------------------------------------------------------------
# array plumbing
# ---------------------------------------------------------------------------
def _is_cuda(a) -> bool:
    return torch is not None and isinstance(a, torch.Tensor) and a.is_cuda


def _colmajor_cuda(t, dtype):
    """Column-major contiguous CUDA tensor of the same shape (no copy if already)."""
    t = t.to(dtype)
    if t.dim() <= 1:
        return t.contiguous()
    rev = list(range(t.dim() - 1, -1, -1))
    return t.permute(*rev).contiguous().permute(*rev)


def _in(a, dtype=np.complex128):
    """Pointer + keep-alive for an input array (host numpy or CUDA torch)."""
    if _is_cuda(a):
        tdt = {np.complex128: torch.complex128, np.float64: torch.float64, np.int64: torch.int64}[dtype]
        t = _colmajor_cuda(a, tdt)
        return C.c_void_p(t.data_ptr()), t
    arr = np.asfortranarray(np.asarray(a, dtype=dtype))
    return C.c_void_p(arr.ctypes.data), arr


def _out(shape, like_cuda: bool, dtype=np.complex128):
    if like_cuda:
        tdt = {np.complex128: torch.complex128, np.float64: torch.float64}[dtype]
        rev = tuple(reversed(shape))
        t = torch.empty(rev, dtype=tdt, device="cuda").permute(*range(len(shape) - 1, -1, -1))
        return C.c_void_p(t.data_ptr()), t
    arr = np.empty(shape, dtype=dtype, order="F")
    return C.c_void_p(arr.ctypes.data), arr


def release_cached_memory():
    """Returns the device memory cached by the library's pool between calls."""
    check(_lib.load().marie_release_cached_memory())


def _sync_stream(op):
    """Waits for the work queued on an Operator's plan stream."""
    torch.cuda.ExternalStream(op.lib.marie_plan_stream(op.plan)).synchronize()


def _sync():
    if torch is not None and torch.cuda.is_available():
        torch.cuda.current_stream().synchronize()


# ---------------------------------------------------------------------------
# the operator held on the device (gpuArray(fN) in JVIE_Solver.m:271)
# ---------------------------------------------------------------------------
class Operator:
    """A plan for an L x M x N grid holding the FFT-of-circulant operator fN on the
    device, in FP64 and/or FP32 (precision 'fp64', 'fp32' or 'mixed')."""

    def __init__(self, L, M, N, precision="fp64", nrhs_max=1):
        self.lib = _lib.load()
        self.L, self.M, self.N = int(L), int(M), int(N)
        self.precision = _PREC[precision]
        ph = C.c_void_p()
        check(self.lib.marie_plan_create(self.L, self.M, self.N, self.precision, int(nrhs_max), None, C.byref(ph)))
        self._plan = ph
        self.dx = None
        self.freq = None

    @property
    def plan(self):
        if self._plan is None:
            raise RuntimeError("operator closed")
        return self._plan

    @classmethod
    def from_array(cls, fN, precision="fp64", nrhs_max=1):
        Lf, Mf, Nf, q = fN.shape
        if q != 6 or Lf % 2 or Mf % 2 or Nf % 2:
            raise ValueError("fN must be 2L x 2M x 2N x 6")
        op = cls(Lf // 2, Mf // 2, Nf // 2, precision, nrhs_max)
        ptr, keep = _in(fN)
        check(op.lib.marie_set_operator(op.plan, ptr, Lf, Mf, Nf))
        del keep
        return op

    @classmethod
    def assemble(cls, L, M, N, dx, freq, precision="fp64", singular="DIRECTFN", singular_values=None, nrhs_max=1):
        """getOPERATORS(r, f, 'N') computed straight into the plan (no host copy)."""
        op = cls(L, M, N, precision, nrhs_max)
        sv, keep = _singular_arg(singular, singular_values)
        check(op.lib.marie_plan_assemble(op.plan, float(dx), float(freq), sv[0], sv[1]))
        op.dx, op.freq = dx, freq
        return op

    @classmethod
    def from_array_k(cls, fK, precision="fp64", nrhs_max=1):
        """A plan holding only the K operator (2L x 2M x 2N x 3, getOPERATORS(r, f, 'K'))."""
        Lf, Mf, Nf, q = fK.shape
        if q != 3 or Lf % 2 or Mf % 2 or Nf % 2:
            raise ValueError("fK must be 2L x 2M x 2N x 3")
        op = cls(Lf // 2, Mf // 2, Nf // 2, precision, nrhs_max)
        op.set_k(fK)
        return op

    def set_k(self, fK):
        """Upload the K operator into this plan (beside fN)."""
        ptr, keep = _in(fK)
        check(self.lib.marie_set_operator_k(self.plan, ptr, 2 * self.L, 2 * self.M, 2 * self.N))
        del keep
        return self

    def assemble_k(self, dx, freq):
        """getOPERATORS(r, f, 'K') computed straight into this plan."""
        check(self.lib.marie_plan_assemble_k(self.plan, float(dx), float(freq)))
        return self

    def autotune(self):
        """Time the FP32 matvec schedules of this grid (fused or five-pass x/y
        passes, their radix schedule; z-pass radix schedule and columns per
        CTA), keep the fastest.  Returns (chosen (fuse, fvar, zvar),
        [(fuse, fvar, zvar, ms), ...])."""
        ms = np.zeros(4 * 32)
        fuse, fvar, zvar, cnt = C.c_int(), C.c_int(), C.c_int(), C.c_int64()
        check(self.lib.marie_plan_autotune(self.plan, C.byref(fuse), C.byref(fvar), C.byref(zvar),
                                           ms.ctypes.data_as(_lib._dp), 32, C.byref(cnt)))
        cands = [(int(ms[4 * i]), int(ms[4 * i + 1]), int(ms[4 * i + 2]), float(ms[4 * i + 3]))
                 for i in range(cnt.value)]
        return (fuse.value, fvar.value, zvar.value), cands

    def set_schedule(self, fuse, fvar, zvar):
        """Pin a matvec schedule (fuse 1/0; fused radix variant 0/1; z-pass variant 0, 1 or 2)."""
        check(self.lib.marie_plan_set_schedule(self.plan, int(fuse), int(fvar), int(zvar)))
        return self

    def set_inner_precision(self, precision):
        """Krylov basis of the inner solves of a 'mixed' plan: 'fp64' (default) or 'fp32'."""
        check(self.lib.marie_plan_set_inner_precision(self.plan, {"fp32": 32, "fp64": 64}[precision]))
        return self

    def bind_mv_AN(self, Mr, Mc, Gram, transp_flag, idx):
        """Binds mv_AN(., fN, Mr, Mc, Gram, transp_flag, idx) to this plan:
        pgmres / pgmresDR / bicgstab given the Operator as A apply it on the
        device (the C ABI's NULL operator)."""
        if transp_flag not in ("notransp", "transp"):
            raise ValueError("transp_flag must be 'notransp' or 'transp'")
        mrp, mrk = _in(Mr)
        mcp, mck = _in(Mc)
        ip, ik = _in(idx, np.int64)
        n = int(np.asarray(idx).size) if not _is_cuda(idx) else int(idx.numel())
        check(self.lib.marie_plan_bind_mv_AN(self.plan, mrp, mcp, float(Gram), 1 if transp_flag == "transp" else 0,
                                             ip, n))
        return self

    def apply_mv_AN(self, J, precision="fp64"):
        """mv_AN bound with bind_mv_AN applied to J (n or n x nrhs; numpy or a
        CUDA torch tensor), without rebuilding the DOF map per call.
        precision 'fp32' runs the product in FP32 throughout."""
        cuda = _is_cuda(J)
        nrhs = 1 if J.ndim == 1 else J.shape[1]
        jp, jk = _in(J)
        op_, out = _out(J.shape, cuda)
        check(self.lib.marie_plan_apply_mv_AN(self.plan, jp, op_, nrhs, _PREC[precision]))
        if cuda:
            _sync_stream(self)
        return out

    def set_inner_restart(self, restart):
        """Restart length of the inner GMRES of a 'mixed' plan (0: the solver's inner_it)."""
        check(self.lib.marie_plan_set_inner_restart(self.plan, int(restart)))
        return self

    def set_batch_groups(self, groups):
        """Batched GMRES schedule: 2 (default: two groups on two streams, one
        group's Gram-Schmidt beside the other's matvec) or 1 (all in lockstep)."""
        check(self.lib.marie_plan_set_batch_groups(self.plan, int(groups)))
        return self

    def set_graph_refinement(self, on):
        """Refinement steps and restart cycles in conditional-graph launches
        (True, default) or driven from the host with one plain graph per cycle
        (False, the form kernel profilers can see); the results are the same."""
        check(self.lib.marie_plan_set_graph_refinement(self.plan, 1 if on else 0))
        return self

    def to_array(self):
        """The FP64 operator as a 2L x 2M x 2N x 6 numpy array."""
        ptr, arr = _out((2 * self.L, 2 * self.M, 2 * self.N, 6), False)
        check(self.lib.marie_get_plan_operator(self.plan, ptr))
        return arr

    def close(self):
        if self._plan is not None:
            self.lib.marie_plan_destroy(self._plan)
            self._plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_SINGULAR = {"DIRECTFN": b"D", "D": b"D", "CONVERGED": b"C", "C": b"C"}


def _singular_arg(singular, values):
    """singular: 'DIRECTFN' (the reference default, Np_1D = 20) or
    'CONVERGED' (a converged quadrature, not a reference method).  The
    reference's 'DEMCEM' is not built and raises."""
    if values is not None:
        v = np.asarray(values, dtype=np.complex128).reshape(5)
        arr = np.ascontiguousarray(v)
        return (b"U", C.c_void_p(arr.ctypes.data)), arr
    if singular == "DEMCEM":
        raise ValueError("singular='DEMCEM' is not built; use 'DIRECTFN' (the reference default)")
    if singular not in _SINGULAR:
        raise ValueError("singular must be 'DIRECTFN' or 'CONVERGED' (or pass singular_values)")
    return (_SINGULAR[singular], None), None


def _operator_for(fN, precision):
    if isinstance(fN, Operator):
        return fN, False
    return Operator.from_array(fN, precision=precision), True


# ---------------------------------------------------------------------------
# getOPERATORS
# ---------------------------------------------------------------------------
def getOPERATORS(r, f, op="N", type="FFTofC", singular="DIRECTFN", singular_values=None):
    """getOPERATORS.m:1-127 for op 'N' (6 components) and 'K' (3 components).
    type 'FFTofC' (default), 'C' or 'T'.

    singular='DIRECTFN' (the default, as getOPERATORS.m:39-41) evaluates the
    weakly singular self/edge/vertex integrals of N with DIRECTFN at
    Np_1D = 20 on the device (assembly_nop.m:16,96-98); 'CONVERGED' uses a
    converged quadrature instead (not a reference method); singular_values =
    [ST, EAc, EAo, VAc, VAo] overrides both."""
    lib = _lib.load()
    if op not in ("N", "K"):
        raise ValueError("op must be 'N' or 'K'")
    L, M, N = r.shape[:3]
    q = 6 if op == "N" else 3
    t = {"FFTofC": b"F", "C": b"C", "T": b"T"}[type]
    shape = (L, M, N, q) if t == b"T" else (2 * L, 2 * M, 2 * N, q)
    rp, rk = _in(r, np.float64)
    op_ptr, out = _out(shape, _is_cuda(r))
    sv, keep = _singular_arg(singular, singular_values)
    check(lib.marie_get_operators(rp, L, M, N, float(f), op.encode(), t, sv[0], sv[1], op_ptr))
    return out


def singular_integrals(ko, dx, method="DIRECTFN", np_1d=0):
    """[ST, EAc, EAo, VAc, VAo] (complex) for wavenumber ko and voxel edge dx:
    singular_st/ea/va.m with 'DIRECTFN' at Np_1D = np_1d (0: the reference's
    20), or the converged quadrature ('CONVERGED')."""
    lib = _lib.load()
    out = np.zeros(10)
    if method == "DEMCEM":
        raise ValueError("method='DEMCEM' is not built")
    code = _SINGULAR.get(method)
    if code is None:
        raise ValueError("method must be 'DIRECTFN' or 'CONVERGED'")
    check(lib.marie_singular_integrals_ex(float(ko), float(dx), code, int(np_1d), C.c_void_p(out.ctypes.data)))
    return out[0::2] + 1j * out[1::2]


def directfn(kind, vertices, ko, np_1d=20):
    """One DIRECTFN core call with its MEX gateway's arguments:
    'st' mexdirectfn_ws_st_const(r1, r2, r3, ko, Np_1D), 'ea' (r1..r4), 'va'
    (r1..r5).  Returns the complex integral."""
    lib = _lib.load()
    code = {"st": b"S", "ea": b"E", "va": b"V"}[kind]
    v = np.ascontiguousarray(np.asarray(vertices, dtype=np.float64).reshape(-1))
    if v.size != {"st": 9, "ea": 12, "va": 15}[kind]:
        raise ValueError("wrong number of vertices")
    out = np.zeros(2)
    check(lib.marie_directfn(code, C.c_void_p(v.ctypes.data), float(ko), int(np_1d), C.c_void_p(out.ctypes.data)))
    return out[0] + 1j * out[1]


# ---------------------------------------------------------------------------
# matvecs
# ---------------------------------------------------------------------------
def mv_AN(JIn0, fN, Mr, Mc, Gram, transp_flag, idx, GPU_flag=1, precision="fp64"):
    """mv_AN.m: 'notransp' -> Gram*Mr*J - Mc*N J ; 'transp' -> its Hermitian adjoint.

    JIn0 may be a vector (n,) or a batch (n, nrhs) of columns."""
    if transp_flag not in ("notransp", "transp"):
        raise ValueError("transp_flag must be 'notransp' or 'transp'")
    prec = _PREC[precision]
    opr, tmp = _operator_for(fN, "mixed" if prec == MARIE_FP32 else "fp64")
    try:
        cuda = _is_cuda(JIn0)
        n = JIn0.shape[0]
        nrhs = 1 if JIn0.ndim == 1 else JIn0.shape[1]
        jp, jk = _in(JIn0)
        mrp, mrk = _in(Mr)
        mcp, mck = _in(Mc)
        ip, ik = _in(idx, np.int64)
        op_, out = _out(JIn0.shape, cuda)
        check(opr.lib.marie_mv_AN(opr.plan, jp, mrp, mcp, float(Gram), 1 if transp_flag == "transp" else 0,
                                  ip, n, op_, nrhs, prec))
        return out
    finally:
        if tmp:
            opr.close()


def mv_L(JIn0, fN, r, Gram, idx, GPU_flag=1, precision="fp64"):
    """mv_L.m: crop(N J) - Gram*J on the entries idx."""
    prec = _PREC[precision]
    opr, tmp = _operator_for(fN, "mixed" if prec == MARIE_FP32 else "fp64")
    try:
        cuda = _is_cuda(JIn0)
        n = JIn0.shape[0]
        nrhs = 1 if JIn0.ndim == 1 else JIn0.shape[1]
        jp, jk = _in(JIn0)
        ip, ik = _in(idx, np.int64)
        op_, out = _out(JIn0.shape, cuda)
        check(opr.lib.marie_mv_L(opr.plan, jp, float(Gram), ip, n, op_, nrhs, prec))
        return out
    finally:
        if tmp:
            opr.close()


def mv_N(JIn0, fN, r, idx, GPU_flag=1, precision="fp64"):
    """mv_N.m: crop(N J) on the entries idx (marie_mv_L with Gram = 0)."""
    return mv_L(JIn0, fN, r, 0.0, idx, GPU_flag, precision)


def _k_operator_for(fK, precision):
    if isinstance(fK, Operator):
        return fK, False
    return Operator.from_array_k(fK, precision=precision), True


def mv_K(JIn0, fK, r, idx, GPU_flag=1, precision="fp64"):
    """mv_K.m: crop(IFFT(fK x FFT(J))) on the entries idx.  fK is an Operator
    holding K (Operator.assemble_k / set_k) or a 2L x 2M x 2N x 3 array."""
    prec = _PREC[precision]
    opr, tmp = _k_operator_for(fK, "mixed" if prec == MARIE_FP32 else "fp64")
    try:
        cuda = _is_cuda(JIn0)
        n = JIn0.shape[0]
        nrhs = 1 if JIn0.ndim == 1 else JIn0.shape[1]
        jp, jk = _in(JIn0)
        ip, ik = _in(idx, np.int64)
        op_, out = _out(JIn0.shape, cuda)
        check(opr.lib.marie_mv_K(opr.plan, jp, ip, n, op_, nrhs, prec))
        return out
    finally:
        if tmp:
            opr.close()


def H_field_Kop(J, fK, Gram, Hinc=None, GPU_flag=1, precision="fp64"):
    """H_field_Kop.m:46-77: Htot = Hinc + mv_K(J) / Gram."""
    opr, tmp = _k_operator_for(fK, "fp64")
    try:
        if Hinc is not None and not np.any(np.asarray(J.cpu() if _is_cuda(J) else J)):
            return Hinc
        jp, jk = _in(J)
        hp, hk = _in(Hinc) if Hinc is not None else (None, None)
        op_, out = _out(tuple(J.shape), _is_cuda(J))
        check(opr.lib.marie_h_field_kop(opr.plan, jp, float(Gram), hp, op_, _PREC[precision]))
        return out
    finally:
        if tmp:
            opr.close()


def E_field_Nop(J, fN, Gram, freq, Einc=None, GPU_flag=1, precision="fp64"):
    """E_field_Nop.m:59-84: Etot = Einc + (N J - Gram J)/(Gram j omega eps0)."""
    opr, tmp = _operator_for(fN, "fp64")
    try:
        if Einc is not None and not np.any(np.asarray(J.cpu() if _is_cuda(J) else J)):
            return Einc
        jp, jk = _in(J)
        if Einc is not None:
            ep, ek = _in(Einc)
        else:
            ep, ek = None, None
        op_, out = _out(tuple(J.shape), _is_cuda(J))
        check(opr.lib.marie_e_field_nop(opr.plan, jp, float(Gram), float(freq), ep, op_, _PREC[precision]))
        return out
    finally:
        if tmp:
            opr.close()


# ---------------------------------------------------------------------------
# pgmres with function-handle operators
# ---------------------------------------------------------------------------
class _CudaVec:
    """__cuda_array_interface__ view of a raw device vector of complex128."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<c16", "data": (ptr, False), "version": 3,
                                         "strides": None}


def _wrap_handle(fn, host_mode):
    def cb(ctx, x, y, n):
        try:
            xt = torch.as_tensor(_CudaVec(x, n), device="cuda")
            yt = torch.as_tensor(_CudaVec(y, n), device="cuda")
            if host_mode:
                res = np.asarray(fn(xt.cpu().numpy()), dtype=np.complex128).reshape(-1)
                yt.copy_(torch.from_numpy(res))
            else:
                res = fn(xt)
                yt.copy_(res.reshape(-1).to(torch.complex128))
            torch.cuda.current_stream().synchronize()
            return 0
        except Exception as e:  # surfaced as a status; the message is kept
            _wrap_handle.last_exc = e
            return -1

    return _lib.OP_FN(cb)


_wrap_handle.last_exc = None
_vec_plan = None


def _vector_plan():
    global _vec_plan
    if _vec_plan is None:
        _vec_plan = Operator(4, 4, 4, "fp64")
    return _vec_plan


def _handles(A, others, host):
    # an Operator with a bound mv_AN is passed as the NULL handle
    cbs = [_lib.OP_FN() if isinstance(A, Operator) else _wrap_handle(A, host)]
    slots = []
    for h in others:
        if h is None:
            slots.append(_lib.OP_FN())
        else:
            f = _wrap_handle(h, host)
            cbs.append(f)
            slots.append(f)
    return cbs, slots


def _call(lib_fn, *args):
    _wrap_handle.last_exc = None
    st = lib_fn(*args)
    if st != 0 and _wrap_handle.last_exc is not None:
        raise _wrap_handle.last_exc
    check(st)


def pgmres(A, b, restart=50, tol=1e-3, maxit=10, L1=None, L2=None, R1=None, R2=None, x0=None):
    """pgmres.m:70-181 on the device.  A, L1, L2, R1, R2 are function handles
    (preconditioners are applied as products, like the reference).  With a
    numpy b the handles receive and return numpy vectors; with a CUDA tensor b
    they receive and return CUDA tensors.  A may also be an Operator with a
    bound mv_AN (Operator.bind_mv_AN): the matvec then stays on the device with
    no handle round trip.  Returns (x, flag, relres, iter, resvec)."""
    restart = 50 if restart is None else restart
    tol = 1e-3 if tol is None else tol
    maxit = 10 if maxit is None else maxit
    host = not _is_cuda(b)
    opr = A if isinstance(A, Operator) else _vector_plan()
    n = b.shape[0]
    cbs, h = _handles(A, (L1, L2, R1, R2), host)
    bp, bk = _in(b)
    x0p, x0k = _in(x0) if x0 is not None else (None, None)
    xp, x = _out((n,), not host)
    flag, relres, it = C.c_int(), C.c_double(), (C.c_int * 2)()
    cap = restart * maxit + 1
    resvec = np.zeros(cap)
    rlen = C.c_int64()
    _call(opr.lib.marie_pgmres, opr.plan, cbs[0], None, bp, n, int(restart), float(tol), int(maxit),
          h[0], None, h[1], None, h[2], None, h[3], None, x0p, xp, C.byref(flag), C.byref(relres), it,
          resvec.ctypes.data_as(_lib._dp), cap, C.byref(rlen))
    return x, flag.value, relres.value, [it[0], it[1]], resvec[:rlen.value]


def pgmresDR(A, b, restart=50, tol=1e-3, maxit=10, ritz=None, L1=None, L2=None, R1=None, R2=None, x0=None):
    """pgmresDR.m (GMRES with deflated restarting by ritz harmonic Ritz
    vectors) on the device; handles and returns as pgmres."""
    restart = 50 if restart is None else restart
    tol = 1e-3 if tol is None else tol
    maxit = 10 if maxit is None else maxit
    host = not _is_cuda(b)
    opr = A if isinstance(A, Operator) else _vector_plan()
    n = b.shape[0]
    cbs, h = _handles(A, (L1, L2, R1, R2), host)
    bp, bk = _in(b)
    x0p, x0k = _in(x0) if x0 is not None else (None, None)
    xp, x = _out((n,), not host)
    flag, relres, it = C.c_int(), C.c_double(), (C.c_int * 2)()
    cap = restart * (maxit + 1) + 1
    resvec = np.zeros(cap)
    rlen = C.c_int64()
    _call(opr.lib.marie_pgmres_dr, opr.plan, cbs[0], None, bp, n, int(restart), float(tol), int(maxit),
          int(ritz) if ritz is not None else 0, h[0], None, h[1], None, h[2], None, h[3], None, x0p, xp,
          C.byref(flag), C.byref(relres), it, resvec.ctypes.data_as(_lib._dp), cap, C.byref(rlen))
    return x, flag.value, relres.value, [it[0], it[1]], resvec[:rlen.value]


def bicgstab(A, b, tol=1e-6, maxit=None, M1=None, M2=None, x0=None):
    """MATLAB's bicgstab (the solver 'B' of JVIE_Solver.m:451-499) on the
    device; M1, M2 are function handles applied as ph = M2(M1(p)).  Returns
    (x, flag, relres, iter, resvec): iter in half steps, resvec absolute."""
    tol = 1e-6 if tol is None else tol
    n = b.shape[0]
    maxit = min(n, 20) if maxit is None else maxit
    host = not _is_cuda(b)
    opr = A if isinstance(A, Operator) else _vector_plan()
    cbs, h = _handles(A, (M1, M2), host)
    bp, bk = _in(b)
    x0p, x0k = _in(x0) if x0 is not None else (None, None)
    xp, x = _out((n,), not host)
    flag, relres, it = C.c_int(), C.c_double(), C.c_double()
    cap = 2 * maxit + 1
    resvec = np.zeros(cap)
    rlen = C.c_int64()
    _call(opr.lib.marie_bicgstab, opr.plan, cbs[0], None, bp, n, float(tol), int(maxit), h[0], None, h[1], None,
          x0p, xp, C.byref(flag), C.byref(relres), C.byref(it), resvec.ctypes.data_as(_lib._dp), cap,
          C.byref(rlen))
    return x, flag.value, relres.value, it.value, resvec[:rlen.value]


# ---------------------------------------------------------------------------
# JVIE_Solver
# ---------------------------------------------------------------------------
def JVIE_Solver(Einc, e_r, r, freq, fN, tol=None, form=None, solver=None, precond=None, max_it=None, inner_it=None,
                outer_it=None, ritz=None, gpu_flag=1, logfile=None, precision=None, runlog=None):
    """JVIE_Solver.m on the device: solver 'G' (pgmres), 'D' (pgmresDR) or,
    as in the reference, anything else (the default) 'B' (bicgstab).

    fN is an Operator (or a 2L x 2M x 2N x 6 array).  precision: 'fp64' (the
    reference arithmetic), 'fp32', or 'mixed' (FP32 circulant matvec inside FP64
    Krylov iterations with FP64 iterative refinement); defaults to the
    Operator's.  Returns (Je, flag, relres, iter, resvec, solvert): iter is
    [inner, outer] for 'G' and 'D' and the half-step count for 'B'.

    logfile: the reference's solve summary is appended to this path (1:
    standard output; None: not written).  runlog: a .jsonl path that receives
    one JSON record of the solve."""
    tstart = time.perf_counter()
    tol = 1e-3 if tol is None else tol
    form = 2 if form is None else form
    solver = solver if solver in ("G", "D") else "B"
    pc = {None: b"\0", 0: b"\0", "L": b"L", "R": b"R"}.get(precond, b"\0")
    max_it = 1000 if max_it is None else max_it
    inner_it = 50 if inner_it is None or inner_it < 1 else inner_it
    outer_it = 200 if outer_it is None or outer_it < 1 else outer_it
    ritz = 5 if ritz is None or ritz < 1 else ritz
    if isinstance(fN, Operator):
        opr, tmp = fN, False
        if precision is not None and _PREC[precision] != opr.precision:
            raise ValueError("precision differs from the Operator's; build the Operator with it")
    else:
        opr, tmp = Operator.from_array(fN, precision=precision or "fp64"), True
    try:
        L, M, N = e_r.shape
        dx = float(r[1, 0, 0, 0] - r[0, 0, 0, 0]) if not _is_cuda(r) else float((r[1, 0, 0, 0] - r[0, 0, 0, 0]).item())
        cuda = _is_cuda(Einc)
        ep, ek = _in(Einc)
        erp, erk = _in(e_r)
        jp, Je = _out((L, M, N, 3), cuda)
        flag = C.c_int()
        relres = C.c_double()
        it = (C.c_double * 2)()
        cap = 1 + max(inner_it * (outer_it + 1) * 4, 2 * max_it * 4)
        resvec = np.zeros(cap)
        rlen = C.c_int64()
        solvert = C.c_double()
        check(opr.lib.marie_jvie_solve(opr.plan, ep, erp, dx, float(freq), float(tol), int(form), solver.encode(), pc,
                                       int(max_it), int(inner_it), int(outer_it), int(ritz), jp, C.byref(flag),
                                       C.byref(relres), it, resvec.ctypes.data_as(_lib._dp), cap, C.byref(rlen),
                                       C.byref(solvert)))
        iters = it[0] if solver == "B" else [int(it[0]), int(it[1])]
        resvec = resvec[:min(rlen.value, cap)]
        if logfile is not None or runlog is not None:
            _log_solve(logfile, runlog, e_r, dx, freq, solver, pc, opr, tol, max_it, inner_it, outer_it, ritz,
                       flag.value, relres.value, iters, resvec, solvert.value, time.perf_counter() - tstart)
        return Je, flag.value, relres.value, iters, resvec, solvert.value
    finally:
        if tmp:
            opr.close()


def _n_scatterer(e_r) -> int:
    """length(idxS): voxels with |e_r - 1| > 1e-12 (JVIE_Solver.m:135)."""
    if _is_cuda(e_r):
        return int(((e_r - 1).abs() > 1e-12).sum().item())
    return int(np.count_nonzero(np.abs(np.asarray(e_r) - 1) > 1e-12))


def _log_solve(logfile, runlog, e_r, dx, freq, solver, pc, opr, tol, max_it, inner_it, outer_it, ritz, flag, relres,
               iters, resvec, solvert, elapsed):
    L, M, N = e_r.shape
    ns = _n_scatterer(e_r)
    precond = pc.decode().strip("\0")
    solvelog.write_solve_log(logfile, L=L, M=M, N=N, dx=dx, n_scat=ns, freq=freq, fN_bytes=8 * L * M * N * 6 * 16,
                             solver=solver, precond=precond, inner_it=inner_it, ritz=ritz, solvert=solvert,
                             resvec=resvec, flag=flag, relres=relres, elapsed=elapsed)
    prec = {MARIE_FP64: "fp64", MARIE_FP32: "fp32", MARIE_MIXED: "mixed"}.get(opr.precision, str(opr.precision))
    solvelog.write_run_record(runlog, solvelog.run_record(L, M, N, dx, ns, freq, solver, precond, prec, tol,
                                                          inner_it, outer_it, max_it, flag, relres, iters, resvec,
                                                          solvert, elapsed))


def Scat_Solver(Einc, Hinc, freq, r, epsilon_r, sigma_e, rho, tol=None, fN=None, fK=None, form=None, solver=None,
                precond=None, max_it=None, inner_it=None, outer_it=None, ritz=None, gpu_flag=1, logfile=None,
                precision="fp64"):
    """Scat_Solver.m on the device: the J-VIE current, SAR, total E, B = mu0 H,
    global SAR and absorbed power.  fN / fK: an Operator holding them (N and
    K on one plan), or None to assemble both.  Returns (Jout, Sout, Eout, Bout,
    Gsar, Pabs, op) where op is the Operator that holds fN and fK.  logfile:
    the closing lines with the overall time are appended to it (1: standard
    output)."""
    tstart = time.perf_counter()
    tol = 1e-3 if tol is None else tol
    form = 2 if form is None else form
    solver = solver if solver in ("G", "D") else "B"
    pc = {None: b"\0", 0: b"\0", "L": b"L", "R": b"R"}.get(precond, b"\0")
    max_it = 1000 if max_it is None else max_it
    inner_it = 50 if inner_it is None or inner_it < 1 else inner_it
    outer_it = 200 if outer_it is None or outer_it < 1 else outer_it
    ritz = 5 if ritz is None or ritz < 1 else ritz
    L, M, N = epsilon_r.shape
    dx = float(r[1, 0, 0, 0] - r[0, 0, 0, 0]) if not _is_cuda(r) else float((r[1, 0, 0, 0] - r[0, 0, 0, 0]).item())
    if isinstance(fN, Operator):
        opr = fN
        if isinstance(fK, np.ndarray):
            opr.set_k(fK)
    else:
        opr = Operator(L, M, N, precision)
        if fN is not None:
            ptr, keep = _in(fN)
            check(opr.lib.marie_set_operator(opr.plan, ptr, 2 * L, 2 * M, 2 * N))
        if fK is not None:
            opr.set_k(fK)
    cuda = _is_cuda(Einc)
    ep, ek = _in(Einc)
    hp, hk = _in(Hinc) if Hinc is not None else (None, None)
    epsp, epsk = _in(epsilon_r, np.float64)
    sp_, sk = _in(sigma_e, np.float64)
    rp_, rk = _in(rho, np.float64)
    jp, Jout = _out((L, M, N, 3), cuda)
    spo, Sout = _out((L, M, N), cuda, np.float64)
    eo, Eout = _out((L, M, N, 3), cuda)
    bo, Bout = _out((L, M, N, 3), cuda)
    gsar, pabs = C.c_double(), C.c_double()
    check(opr.lib.marie_scat_solver(opr.plan, ep, hp, dx, float(freq), epsp, sp_, rp_, float(tol), int(form),
                                    solver.encode(), pc, int(max_it), int(inner_it), int(outer_it), int(ritz), jp, spo,
                                    eo, bo, C.byref(gsar), C.byref(pabs)))
    solvelog.write_overall_log(logfile, time.perf_counter() - tstart)
    return Jout, Sout, Eout, Bout, gsar.value, pabs.value, opr


def JVIE_Solver_batch(Einc, e_r, r, freq, fN, tol=None, form=None, precond=None, inner_it=None, outer_it=None):
    """JVIE_Solver for several excitations of one body solved together.

    Einc: (L, M, N, 3, nexc) column-major.  The excitations advance in lockstep
    (one batched matvec per GMRES step, one graph launch per restart cycle).
    Returns (Je (L, M, N, 3, nexc), flag[nexc], relres[nexc], iter[nexc, 2], solvert)."""
    tol = 1e-3 if tol is None else tol
    form = 2 if form is None else form
    pc = {None: b"\0", 0: b"\0", "L": b"L", "R": b"R"}.get(precond, b"\0")
    inner_it = 50 if inner_it is None or inner_it < 1 else inner_it
    outer_it = 200 if outer_it is None or outer_it < 1 else outer_it
    opr, tmp = (fN, False) if isinstance(fN, Operator) else (Operator.from_array(fN), True)
    try:
        L, M, N = e_r.shape
        nexc = Einc.shape[4]
        dx = float(r[1, 0, 0, 0] - r[0, 0, 0, 0]) if not _is_cuda(r) else float((r[1, 0, 0, 0] - r[0, 0, 0, 0]).item())
        cuda = _is_cuda(Einc)
        ep, ek = _in(Einc)
        erp, erk = _in(e_r)
        jp, Je = _out((L, M, N, 3, nexc), cuda)
        flag = np.zeros(nexc, np.int32)
        relres = np.zeros(nexc)
        it = np.zeros(2 * nexc, np.int32)
        solvert = C.c_double()
        check(opr.lib.marie_jvie_solve_batch(opr.plan, ep, nexc, erp, dx, float(freq), int(form), pc, float(tol),
                                             int(inner_it), int(outer_it), jp,
                                             flag.ctypes.data_as(_lib._ip), relres.ctypes.data_as(_lib._dp),
                                             it.ctypes.data_as(_lib._ip), C.byref(solvert)))
        return Je, flag, relres, it.reshape(nexc, 2), solvert.value
    finally:
        if tmp:
            opr.close()


def JVIE_Solver_bodies(bodies, freq, tol=None, form=None, precond=None, inner_it=None, outer_it=None):
    """Several bodies of uneven grid size solved concurrently.

    bodies: list of (Einc (L,M,N,3,nexc), e_r (L,M,N), r, Operator).  Returns a
    list of (Je, flag, relres, iter) per body and the wall time."""
    tol = 1e-3 if tol is None else tol
    form = 2 if form is None else form
    pc = {None: b"\0", 0: b"\0", "L": b"L", "R": b"R"}.get(precond, b"\0")
    inner_it = 50 if inner_it is None or inner_it < 1 else inner_it
    outer_it = 200 if outer_it is None or outer_it < 1 else outer_it
    nb = len(bodies)
    keep, Ep, Erp, Jp, outs = [], [], [], [], []
    nexc = np.zeros(nb, np.int64)
    dxs = np.zeros(nb)
    plans = (C.c_void_p * nb)()
    for b, (Einc, e_r, r, op) in enumerate(bodies):
        L, M, N = e_r.shape
        nexc[b] = Einc.shape[4]
        dxs[b] = float(r[1, 0, 0, 0] - r[0, 0, 0, 0])
        ep, ek = _in(Einc)
        erp, erk = _in(e_r)
        jp, Je = _out((L, M, N, 3, int(nexc[b])), _is_cuda(Einc))
        keep += [ek, erk]
        Ep.append(ep.value)
        Erp.append(erp.value)
        Jp.append(jp.value)
        outs.append(Je)
        plans[b] = op.plan.value
    tot = int(nexc.sum())
    flag = np.zeros(tot, np.int32)
    relres = np.zeros(tot)
    it = np.zeros(2 * tot, np.int32)
    solvert = C.c_double()
    arr = lambda v: (C.c_void_p * nb)(*v)
    lib = _lib.load()
    check(lib.marie_jvie_solve_bodies(nb, plans, arr(Ep), nexc.ctypes.data_as(_lib._i64p), arr(Erp),
                                      dxs.ctypes.data_as(_lib._dp), float(freq), int(form), pc, float(tol),
                                      int(inner_it), int(outer_it), arr(Jp), flag.ctypes.data_as(_lib._ip),
                                      relres.ctypes.data_as(_lib._dp), it.ctypes.data_as(_lib._ip),
                                      C.byref(solvert)))
    res, o = [], 0
    for b in range(nb):
        k = int(nexc[b])
        res.append((outs[b], flag[o:o + k], relres[o:o + k], it.reshape(-1, 2)[o:o + k]))
        o += k
    return res, solvert.value


# ---------------------------------------------------------------------------
# the J-VIE solve as the inner solver of the coil solvers
# ---------------------------------------------------------------------------
# grid sizes L (per axis) whose 2L the FFT engine transforms
SUPPORTED_L = (4, 8, 12, 16, 20, 24, 32, 40, 48, 64, 80, 96, 128, 160, 192, 256)


def supported_size(n):
    """The smallest grid size >= n per axis that the matvec transforms (2n in
    the FFT engine's length list); larger grids are extended with air."""
    for L in SUPPORTED_L:
        if L >= n:
            return L
    raise ValueError(f"grid dimension {n} exceeds the largest supported size {SUPPORTED_L[-1]}")


def jvie2solver(Vrhs, fN, idx, Mr, Mc, Gram, tol, Vini=None, max_it=1000):
    """jvie2solver.m:1-79: BiCGSTAB (max_it iterations, no preconditioner, x0 =
    Vini) on mv_AN(J, fN, Mr, Mc, Gram, 'notransp', idx); an all-zero Vrhs is
    returned unchanged.  fN: an Operator (or a 2L x 2M x 2N x 6 array).  Returns
    (Vsol, flag, relres, iter, solvert); iter counts half steps."""
    opr, tmp = _operator_for(fN, "fp64")
    try:
        n = int(np.asarray(idx).size) if not _is_cuda(idx) else int(idx.numel())
        ip, ik = _in(idx, np.int64)
        mrp, mrk = _in(Mr)
        mcp, mck = _in(Mc)
        bp, bk = _in(Vrhs)
        xp, xk = _in(Vini) if Vini is not None else (None, None)
        op_, out = _out((n,), _is_cuda(Vrhs))
        flag = C.c_int()
        relres = C.c_double()
        it = C.c_double()
        solvert = C.c_double()
        check(opr.lib.marie_jvie2solver(opr.plan, ip, n, mrp, mcp, float(Gram), bp, float(tol), int(max_it), xp, op_,
                                        C.byref(flag), C.byref(relres), C.byref(it), C.byref(solvert)))
        return out, flag.value, relres.value, it.value, solvert.value
    finally:
        if tmp:
            opr.close()


def _crop_box(r, e_r, dx):
    """Index ranges of fVIEsolver_Assembly.m:82-94: the grid lines within one
    voxel of the non-air voxels' bounding box."""
    nonair = np.abs(e_r - 1) > 1e-12
    ranges = []
    for a in range(3):
        coord = r[..., a][nonair]
        lo, hi = coord.min() - dx, coord.max() + dx
        line = np.moveaxis(r[..., a], a, 0)[:, 0, 0]
        ranges.append(np.flatnonzero((line >= lo) & (line <= hi)))
    return ranges


def fVIEsolver_Assembly(RHBM, freq, gpu_flag=1, precision="fp64"):
    """fVIEsolver_Assembly.m:1-210: prepares a body for repeated J-VIE solves.

    RHBM: dict with r (L,M,N,3), epsilon_r, sigma_e (L,M,N) and optionally fN
    (an Operator or array for the full grid) and freqfN.  The domain is cropped
    to one voxel around the non-air bounding box when that is below 70 % of the
    voxels, or when no operator for this frequency is given (then the operator
    is assembled on the device); the cropped grid is then extended with air to
    the next size the FFT engine transforms (the matvec on the non-air DOFs is
    unchanged by air padding).  Returns (fVIEsolver, Gram, tau3, Scoord, op):
    fVIEsolver(Vrhs, tol, Vini) -> Vsol solves the form-2 system on the DOFs in
    the order of Scoord (tau3 turns incident fields at those voxels into the
    right-hand side); op is the Operator that holds fN on the device."""
    omega = 2 * np.pi * freq
    r = np.asarray(RHBM["r"], dtype=np.float64)
    e_r = np.asarray(RHBM["epsilon_r"]) - 1j * np.asarray(RHBM["sigma_e"]) / (EPS0 * omega)
    dx = float(r[1, 0, 0, 0] - r[0, 0, 0, 0])
    Gram = dx**3
    L, M, N = e_r.shape
    ND = L * M * N
    idxS = np.flatnonzero(np.abs(e_r.reshape(-1, order="F") - 1) > 1e-12)
    Scoord = np.stack([r[..., a].reshape(-1, order="F")[idxS] for a in range(3)], axis=1)
    ix, iy, iz = _crop_box(r, e_r, dx)
    Lf, Mf, Nf = len(ix), len(iy), len(iz)
    fN = RHBM.get("fN")
    if Lf * Mf * Nf < 0.7 * ND or fN is None or RHBM.get("freqfN") != freq:
        e_r = e_r[np.ix_(ix, iy, iz)]
        Ls, Ms, Ns = supported_size(Lf), supported_size(Mf), supported_size(Nf)
        e_pad = np.ones((Ls, Ms, Ns), complex, order="F")
        e_pad[:Lf, :Mf, :Nf] = e_r
        e_r = e_pad
        op = Operator.assemble(Ls, Ms, Ns, dx, freq, precision=precision)
    else:
        op = fN if isinstance(fN, Operator) else Operator.from_array(fN, precision=precision)
    e_r = np.asfortranarray(e_r)
    Lc, Mc_, Nc = e_r.shape
    NDc = Lc * Mc_ * Nc
    idxS = np.flatnonzero(np.abs(e_r.reshape(-1, order="F") - 1) > 1e-12)
    idxS3 = np.concatenate([idxS, NDc + idxS, 2 * NDc + idxS]).astype(np.int64) + 1
    Mr = np.asfortranarray(e_r / e_r)
    Mcoef = np.asfortranarray((e_r - 1.0) / e_r)
    tau = (1j * omega * EPS0 * Mcoef).reshape(-1, order="F")[idxS]
    tau3 = np.concatenate([tau, tau, tau])
    if torch is not None and torch.cuda.is_available():
        # the per-body arrays stay on the device between solves
        idx_d = torch.from_numpy(idxS3).cuda()
        Mr_d = _colmajor_cuda_from_numpy(Mr)
        Mc_d = _colmajor_cuda_from_numpy(Mcoef)
    else:
        idx_d, Mr_d, Mc_d = idxS3, Mr, Mcoef

    def fVIEsolver(Vrhs, tol, Vini=None):
        return jvie2solver(Vrhs, op, idx_d, Mr_d, Mc_d, Gram, tol, Vini)[0]

    return fVIEsolver, Gram, tau3, Scoord, op


def _colmajor_cuda_from_numpy(a):
    t = torch.from_numpy(np.ascontiguousarray(a.transpose(*range(a.ndim - 1, -1, -1)))).cuda()
    return t.permute(*range(a.ndim - 1, -1, -1))


# ---------------------------------------------------------------------------
# excitations
# ---------------------------------------------------------------------------
def PlaneWave_Excitation(r, k, omega_mu, Eo):
    """PlaneWave_Excitation.m:39-95 -> (E, H), voxel-averaged plane wave."""
    lib = _lib.load()
    L, M, N = r.shape[:3]
    rp, rk = _in(r, np.float64)
    kk = np.ascontiguousarray(np.asarray(k, dtype=np.float64).reshape(3))
    eo = np.asarray(Eo, dtype=np.complex128).reshape(3)
    eov = np.ascontiguousarray(np.stack([eo.real, eo.imag], axis=1).reshape(-1))
    ptr, E = _out((L, M, N, 3), _is_cuda(r))
    check(lib.marie_plane_wave(rp, L, M, N, C.c_void_p(kk.ctypes.data), C.c_void_p(eov.ctypes.data), ptr))
    Ho = np.cross(kk, eo) / omega_mu
    c = int(np.argmax(np.abs(eo)))
    base = E[..., c] / eo[c]
    if _is_cuda(r):
        H = torch.stack([base * complex(Ho[i]) for i in range(3)], dim=3)
    else:
        H = np.stack([base * Ho[i] for i in range(3)], axis=3)
    return E, H


def Dipole_Excitation(r, k, DipJ, DipCoord):
    """Dipole_Excitation.m:39-54 (E field of electric dipoles via E_field_DGF.m).
    DipJ: (ndip, 3) complex moments, DipCoord: (ndip, 3) positions.  Returns E
    (the magnetic field is not on this path)."""
    lib = _lib.load()
    L, M, N = r.shape[:3]
    Jd = np.asarray(DipJ, dtype=np.complex128).reshape(-1, 3)
    pos = np.ascontiguousarray(np.asarray(DipCoord, dtype=np.float64).reshape(-1, 3))
    jv = np.ascontiguousarray(np.stack([Jd.real, Jd.imag], axis=2).reshape(-1))
    rp, rk = _in(r, np.float64)
    ptr, E = _out((L, M, N, 3), _is_cuda(r))
    check(lib.marie_dipole_field(rp, L, M, N, float(k), C.c_void_p(jv.ctypes.data), C.c_void_p(pos.ctypes.data),
                                 Jd.shape[0], ptr))
    return E
