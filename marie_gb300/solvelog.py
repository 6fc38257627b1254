"""The solve log of JVIE_Solver and a JSON-lines record of each solve.

JVIE_Solver.m writes a fixed summary to its `logfile` (appended; standard
output when the argument is empty or the file cannot be opened,
JVIE_Solver.m:115-122): the domain (:159-166), the estimated matvec peak memory
(:246-250), one line naming the solver and one with its time, iteration count,
flag and residues (:324-335, :395-406, :464-475), and the elapsed time of the
whole call (:515-516).  `write_solve_log` writes the same lines with the same
formats.  Here an empty `logfile` writes nothing (a library call does not
print); `logfile=1` is MATLAB's fid 1, standard output.

`write_run_record` appends one JSON object per solve to a `.jsonl` file: the
grid, the DOFs, the solver settings, the result (flag, relres, iterations,
residual history length) and the times, for run-to-run comparison of a deployment.
"""
from __future__ import annotations

import json
import sys
from typing import Optional, Sequence


def _solver_line(solver: str, precond: str, inner_it: int, ritz: int) -> str:
    """The solver-name line of JVIE_Solver.m for the GPU branch (:328, :348,
    :368 GMRES; :399, :419, :439 deflated GMRES; :468, :479 BiCGSTAB)."""
    pc = {"R": "w/ Right preconditioner", "L": "w/ Left preconditioner"}.get(precond, "wo/ preconditioner")
    if solver == "G":
        return "\n GPU GMRES solver (%d restart), %s" % (inner_it, pc)
    if solver == "D":
        return "\n GPU GMRES solver (%d restart, deflated %d), %s \n" % (inner_it, ritz, pc)
    return "\n GPU BICGSTAB solver, %s" % ("w/ preconditioner" if precond in ("L", "R") else "wo/ preconditioner")


def format_solve_log(L: int, M: int, N: int, dx: float, n_scat: int, freq: float, fN_bytes: int, solver: str,
                     precond: str, inner_it: int, ritz: int, solvert: float, resvec: Sequence[float], flag: int,
                     relres: float, elapsed: float) -> str:
    """The text JVIE_Solver.m writes to its log for one solve.  n_scat is the
    number of non-air voxels (length(idxS)); fN_bytes the bytes of the
    2L x 2M x 2N x 6 complex operator (whos('fN').bytes)."""
    nD = L * M * N
    out = []
    out.append("\n ----------------------------------------------------------")
    out.append("\n Domain:                %dx%dx%d voxels" % (L, M, N))
    out.append("\n Resolution:            %.2fmm" % (dx * 1000))
    out.append("\n # DOFS:                %d" % (3 * nD))
    out.append("\n # DOFS in Scatterer:   %d" % (3 * n_scat))
    out.append("\n Operating Frequency:   %.2f MHz" % (freq / 1e6))
    out.append("\n")
    out.append("\n ----------------------------------------------------------")
    out.append("\n Estimated MVP Peak Memory %.3f MB.\n" % (4 * fN_bytes / (1024 * 1024)))
    out.append(_solver_line(solver, precond, inner_it, ritz))
    last = float(resvec[-1]) if len(resvec) else float("nan")
    out.append(" Time  = %.2f [sec] for %d iterations, flag %d, residue %g, relative residue %g \n"
               % (solvert, len(resvec), flag, last, relres))
    out.append(" VIE Solve finished. Elapsed Time  = %.2f [sec] \n" % elapsed)
    return "".join(out)


def _emit(logfile, text: str) -> None:
    if logfile is None or logfile == "":
        return
    if logfile == 1:
        sys.stdout.write(text)
        return
    try:
        with open(logfile, "a") as fh:
            fh.write(text)
    except OSError:
        # JVIE_Solver.m:118-121: a log file that cannot be opened falls back to fid 1
        sys.stdout.write(text)


def write_solve_log(logfile, **fields) -> None:
    """Appends format_solve_log(**fields) to logfile (a path, or 1 for
    standard output; None writes nothing)."""
    if logfile is None or logfile == "":
        return
    _emit(logfile, format_solve_log(**fields))


def write_overall_log(logfile, toverall: float) -> None:
    """Scat_Solver.m:238-241: the closing lines with the overall time."""
    _emit(logfile, "\n --------------------------------------------------------------"
                   "\n Overall Scattering Problem:      \tElapsed time  = %.2f [sec]"
                   "\n --------------------------------------------------------------"
                   "\n --------------------------------------------------------------\n" % toverall)


def run_record(L: int, M: int, N: int, dx: float, n_scat: int, freq: float, solver: str, precond: str,
               precision: str, tol: float, inner_it: int, outer_it: int, max_it: int, flag: int, relres: float,
               iters, resvec: Sequence[float], solvert: float, elapsed: float) -> dict:
    """One solve as a JSON-serialisable dict (resvec_len: entries of the
    residual history the solver returned)."""
    it = [int(i) for i in iters] if isinstance(iters, (list, tuple)) else float(iters)
    return {
        "grid": [int(L), int(M), int(N)], "dx": float(dx), "freq": float(freq),
        "dofs": 3 * L * M * N, "dofs_scatterer": 3 * int(n_scat),
        "solver": solver, "precond": precond or None, "precision": precision, "tol": float(tol),
        "inner_it": int(inner_it), "outer_it": int(outer_it), "max_it": int(max_it),
        "flag": int(flag), "relres": float(relres), "iter": it, "resvec_len": len(resvec),
        "solve_s": float(solvert), "elapsed_s": float(elapsed),
    }


def write_run_record(path: Optional[str], record: dict) -> None:
    """Appends record as one JSON line to path (None writes nothing)."""
    if path is None:
        return
    with open(path, "a") as fh:
        fh.write(json.dumps(record, sort_keys=True) + "\n")
