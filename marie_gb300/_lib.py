"""ctypes binding of libmarie_vie.so (the C ABI in include/marie_vie.h).

The library is the only compute path: there is no CPU fallback.  Loading fails
loudly when the shared object is missing or does not export every declared
symbol.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libmarie_vie.so"

MARIE_OK = 0
MARIE_EINVAL = -1
MARIE_ENOMEM = -2
MARIE_ECUDA = -3
MARIE_ENOCONV = -4
MARIE_EBREAKDOWN = -5
MARIE_ETIMEOUT = -6
MARIE_EUNSUPPORTED = -7
MARIE_ENOOP = -8

MARIE_FP64 = 64
MARIE_FP32 = 32
MARIE_MIXED = 96

_dp = C.POINTER(C.c_double)
_i64p = C.POINTER(C.c_int64)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p

OP_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64)

# name -> (restype, argtypes); must list every function declared in include/marie_vie.h
SIGNATURES = {
    "marie_last_error": (C.c_char_p, []),
    "marie_version": (C.c_int, []),
    "marie_plan_create": (C.c_int, [C.c_int64, C.c_int64, C.c_int64, C.c_int, C.c_int64, _vp, C.POINTER(_vp)]),
    "marie_plan_destroy": (C.c_int, [_vp]),
    "marie_plan_stream": (_vp, [_vp]),
    "marie_get_operators": (C.c_int, [_vp, C.c_int64, C.c_int64, C.c_int64, C.c_double, C.c_char, C.c_char,
                                      C.c_char, _vp, _vp]),
    "marie_singular_integrals": (C.c_int, [C.c_double, C.c_double, _vp]),
    "marie_singular_integrals_ex": (C.c_int, [C.c_double, C.c_double, C.c_char, C.c_int, _vp]),
    "marie_directfn": (C.c_int, [C.c_char, _vp, C.c_double, C.c_int, _vp]),
    "marie_set_operator": (C.c_int, [_vp, _vp, C.c_int64, C.c_int64, C.c_int64]),
    "marie_plan_assemble": (C.c_int, [_vp, C.c_double, C.c_double, C.c_char, _vp]),
    "marie_get_plan_operator": (C.c_int, [_vp, _vp]),
    "marie_set_operator_k": (C.c_int, [_vp, _vp, C.c_int64, C.c_int64, C.c_int64]),
    "marie_plan_assemble_k": (C.c_int, [_vp, C.c_double, C.c_double]),
    "marie_mv_K": (C.c_int, [_vp, _vp, _vp, C.c_int64, _vp, C.c_int64, C.c_int]),
    "marie_h_field_kop": (C.c_int, [_vp, _vp, C.c_double, _vp, _vp, C.c_int]),
    "marie_mv_AN": (C.c_int, [_vp, _vp, _vp, _vp, C.c_double, C.c_int, _vp, C.c_int64, _vp, C.c_int64, C.c_int]),
    "marie_mv_AN_static": (C.c_int, [_vp, _vp, _vp, _vp, C.c_double, C.c_int, _vp, C.c_int64, _vp, C.c_int]),
    "marie_mv_AN_cufft": (C.c_int, [_vp, _vp, _vp, _vp, C.c_double, _vp, C.c_int64, _vp, C.POINTER(C.c_float)]),
    "marie_mv_L": (C.c_int, [_vp, _vp, C.c_double, _vp, C.c_int64, _vp, C.c_int64, C.c_int]),
    "marie_pgmres": (C.c_int, [_vp, OP_FN, _vp, _vp, C.c_int64, C.c_int, C.c_double, C.c_int,
                               OP_FN, _vp, OP_FN, _vp, OP_FN, _vp, OP_FN, _vp,
                               _vp, _vp, _ip, _dp, _ip, _dp, C.c_int64, _i64p]),
    "marie_pgmres_dr": (C.c_int, [_vp, OP_FN, _vp, _vp, C.c_int64, C.c_int, C.c_double, C.c_int, C.c_int,
                                  OP_FN, _vp, OP_FN, _vp, OP_FN, _vp, OP_FN, _vp,
                                  _vp, _vp, _ip, _dp, _ip, _dp, C.c_int64, _i64p]),
    "marie_bicgstab": (C.c_int, [_vp, OP_FN, _vp, _vp, C.c_int64, C.c_double, C.c_int, OP_FN, _vp, OP_FN, _vp,
                                 _vp, _vp, _ip, _dp, _dp, _dp, C.c_int64, _i64p]),
    "marie_jvie_solve": (C.c_int, [_vp, _vp, _vp, C.c_double, C.c_double, C.c_double, C.c_int, C.c_char, C.c_char,
                                   C.c_int, C.c_int, C.c_int, C.c_int, _vp, _ip, _dp, _dp, _dp, C.c_int64, _i64p,
                                   _dp]),
    "marie_scat_solver": (C.c_int, [_vp, _vp, _vp, C.c_double, C.c_double, _vp, _vp, _vp, C.c_double, C.c_int,
                                    C.c_char, C.c_char, C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp,
                                    _dp, _dp]),
    "marie_jvie_solve_bodies": (C.c_int, [C.c_int, _vp, _vp, _vp, _vp, _vp, C.c_double, C.c_int, C.c_char,
                                          C.c_double, C.c_int, C.c_int, _vp, _ip, _dp, _ip, _dp]),
    "marie_jvie_adjoint_grad": (C.c_int, [_vp, _vp, _vp, C.c_double, C.c_double, C.c_int, _vp, C.c_double, C.c_int,
                                          C.c_int, _dp, _vp, _vp, _ip, _ip]),
    "marie_jvie2solver": (C.c_int, [_vp, _vp, C.c_int64, _vp, _vp, C.c_double, _vp, C.c_double, C.c_int, _vp, _vp,
                                    _ip, _dp, _dp, _dp]),
    "marie_jvie_solve_batch": (C.c_int, [_vp, _vp, C.c_int64, _vp, C.c_double, C.c_double, C.c_int, C.c_char,
                                         C.c_double, C.c_int, C.c_int, _vp, _ip, _dp, _ip, _dp]),
    "marie_e_field_nop": (C.c_int, [_vp, _vp, C.c_double, C.c_double, _vp, _vp, C.c_int]),
    "marie_plane_wave": (C.c_int, [_vp, C.c_int64, C.c_int64, C.c_int64, _vp, _vp, _vp]),
    "marie_launch_count": (C.c_int64, []),
    "marie_graph_loops": (C.c_int64, []),
    "marie_release_cached_memory": (C.c_int, []),
    "marie_plan_autotune": (C.c_int, [_vp, _ip, _ip, _ip, _dp, C.c_int64, _i64p]),
    "marie_plan_set_schedule": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int]),
    "marie_plan_set_inner_precision": (C.c_int, [_vp, C.c_int]),
    "marie_plan_set_inner_restart": (C.c_int, [_vp, C.c_int]),
    "marie_plan_set_batch_groups": (C.c_int, [_vp, C.c_int]),
    "marie_plan_apply_mv_AN": (C.c_int, [_vp, _vp, _vp, C.c_int64, C.c_int]),
    "marie_plan_set_graph_refinement": (C.c_int, [_vp, C.c_int]),
    "marie_plan_bind_mv_AN": (C.c_int, [_vp, _vp, _vp, C.c_double, C.c_int, _vp, C.c_int64]),
    "marie_inject_alloc_failure": (None, [C.c_int64]),
    "marie_inject_tile_timeout": (None, [C.c_int64]),
    "marie_plan_profile": (C.c_int, [_vp, C.c_int, _dp, _i64p]),
    "marie_dipole_field": (C.c_int, [_vp, C.c_int64, C.c_int64, C.c_int64, C.c_double, _vp, _vp, C.c_int64,
                                     _vp]),
}


class MarieError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"marie status {code}: {msg}")
        self.code = code


_lib = None


def load(path: Path | str | None = None):
    """Load libmarie_vie.so and bind every C-ABI symbol.  Raises if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                          "(the CUDA library is the only implementation; there is no fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)  # AttributeError if a symbol is not exported
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(status: int) -> None:
    if status != MARIE_OK:
        msg = load().marie_last_error().decode(errors="replace")
        raise MarieError(status, msg)
