"""Differentiable J-VIE objectives: d(objective)/d(per-voxel eps_r, sigma).

The gradient comes from the hand-written adjoint solve in libmarie_vie.so
(`marie_jvie_adjoint_grad`): a forward J-VIE solve, the objective, one adjoint
solve with the same J-VIE operator (the E-field system's transpose is the
reference's form-1 operator, N being symmetric) and a fused gradient kernel.
`JVIEObjective` wraps it as a torch.autograd.Function.

Objectives (sums over the non-air voxels):
    'power'   F = sum 0.5 * sigma * |E|^2        (absorbed power density sum)
    'misfit'  F = sum |E - E_target|^2
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from ._lib import check
from .vie import EPS0, Operator, _in, _is_cuda, _out

try:
    import torch
except Exception:  # pragma: no cover
    torch = None

_OBJ = {"power": 0, "misfit": 1}


def complex_permittivity(eps_r, sigma, freq):
    """e_r = eps_r - j sigma / (eps0 omega)  (Scat_Solver.m:144)."""
    omega = 2 * math.pi * freq
    return eps_r - 1j * sigma / (EPS0 * omega)


def adjoint_gradient(op: Operator, Einc, e_r, dx, freq, objective="power", E_target=None, tol=1e-8, inner_it=50,
                     outer_it=200):
    """Returns (F, dF_deps (L,M,N), dF_dsigma (L,M,N), flags (fwd, adj), iters (fwd, adj))."""
    L, M, N = e_r.shape
    cuda = _is_cuda(Einc)
    ep, ek = _in(Einc)
    erp, erk = _in(e_r)
    if E_target is not None:
        tp, tk = _in(E_target)
    else:
        tp, tk = None, None
    gep, ge = _out((L, M, N), cuda, np.float64)
    gsp, gs = _out((L, M, N), cuda, np.float64)
    F = C.c_double()
    flags = (C.c_int * 2)()
    iters = (C.c_int * 2)()
    check(op.lib.marie_jvie_adjoint_grad(op.plan, ep, erp, float(dx), float(freq), _OBJ[objective], tp, float(tol),
                                         int(inner_it), int(outer_it), C.byref(F), gep, gsp, flags, iters))
    return F.value, ge, gs, (flags[0], flags[1]), (iters[0], iters[1])


if torch is not None:

    class JVIEObjective(torch.autograd.Function):
        """F(eps_r, sigma) for a fixed incident field; backward returns the
        adjoint gradients (the forward call computes them together with F)."""

        @staticmethod
        def forward(ctx, eps_r, sigma, op, Einc, dx, freq, objective, E_target, tol):
            e_r = complex_permittivity(eps_r.detach().to(torch.float64), sigma.detach().to(torch.float64), freq)
            F, ge, gs, flags, iters = adjoint_gradient(op, Einc, e_r, dx, freq, objective, E_target, tol)
            if flags[0] or flags[1]:
                raise RuntimeError(f"J-VIE solve did not converge (forward/adjoint flags {flags})")
            ge = torch.as_tensor(ge, device=eps_r.device)
            gs = torch.as_tensor(gs, device=sigma.device)
            ctx.save_for_backward(ge, gs)
            return torch.tensor(F, dtype=torch.float64, device=eps_r.device)

        @staticmethod
        def backward(ctx, gF):
            ge, gs = ctx.saved_tensors
            return gF * ge, gF * gs, None, None, None, None, None, None, None

    def jvie_objective(eps_r, sigma, op, Einc, dx, freq, objective="power", E_target=None, tol=1e-8):
        """Differentiable objective over column-major (L, M, N) eps_r / sigma tensors."""
        return JVIEObjective.apply(eps_r, sigma, op, Einc, dx, freq, objective, E_target, tol)
