"""GB300-native J-VIE solve path of MARIE (getOPERATORS -> mv_AN -> pgmres).

The compute lives in libmarie_vie.so (hand-written sm_103a CUDA behind the C ABI
in include/marie_vie.h); this package is the reference-facing host API.
"""
from ._lib import MARIE_FP32, MARIE_FP64, MARIE_MIXED, MarieError, load  # noqa: F401
from .vie import (EMconstants, E_field_Nop, JVIE_Solver, JVIE_Solver_batch, JVIE_Solver_bodies, Operator,  # noqa: F401,E501
                  Scat_Solver,
                  PlaneWave_Excitation, Dipole_Excitation, H_field_Kop, bicgstab, getOPERATORS, mv_AN, mv_K, mv_L, mv_N,
                  pgmres, pgmresDR, singular_integrals, directfn, fVIEsolver_Assembly, jvie2solver, supported_size,
                  release_cached_memory)
from .bodies import Import_RHBM  # noqa: F401
from .opcache import OperatorCache, ScheduleCache  # noqa: F401

__all__ = ["EMconstants", "E_field_Nop", "JVIE_Solver", "JVIE_Solver_batch", "Operator", "PlaneWave_Excitation",
           "Scat_Solver",
           "Dipole_Excitation", "H_field_Kop", "bicgstab", "getOPERATORS", "mv_AN", "mv_K", "mv_L", "mv_N", "pgmres", "pgmresDR",
           "singular_integrals", "directfn", "fVIEsolver_Assembly", "jvie2solver", "supported_size", "Import_RHBM",
           "release_cached_memory", "OperatorCache", "ScheduleCache",
           "MarieError", "load"]
