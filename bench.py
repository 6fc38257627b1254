"""Benchmark of the J-VIE solve path on one or more GPUs.

Workload (single body, mixed precision): a 128^3 grid at 2 mm holding a seeded
phantom of 12 random ellipsoids (eps_r ~ U[5,80], sigma ~ U[0.02,2] S/m) inside
a 20 x 15 x 25 cm outer ellipsoid, 298 MHz, x-polarised plane wave travelling
+z; J-VIE form 2, GMRES restart 50, tolerance 1e-6 on the true FP64 relative
residual.  A step is one full solve: RHS set-up on the device, the solve, and
the scatter of J back onto the grid (the operator fN is assembled once per
frequency, outside the timed region, and reported separately).

Arms:
  default          FP32 circulant matvec inside GMRES with an FP64 Krylov
                   basis, FP64 residuals and refinement (inputs resident in
                   HBM for `value`; host buffers through the C ABI for `e2e`);
                   the plain FP64 solve, the FP32-basis variant and the matvec
                   times are measured beside it, and the other workloads (c1
                   Mie sphere, c3 batched dipoles and uneven bodies, c4 64^3
                   adjoint gradient, c5 256x192x160 body) as extra keys.
  --impl reference the reference's CPU path (the numpy/scipy restatement of
                   mv_AN + pgmres, complex128, scipy.fft on all host cores),
                   one GMRES iteration per step, reported as solves/s.

Multi-GPU (--gpus N): the script re-runs itself as N processes under
torch.distributed.run when it is not already inside one.  Each rank solves its
own body (seed = rank) for the headline, and its share of the c3 excitations
and bodies; NCCL only takes the timing maximum and gathers the per-unit
results ("weak" scaling, replicas of independent objects, no data-path
collective).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "VIE solves/s & matvec ms @128^3, FP32+FP64-refined vs FP64 on GB300, 1e-6 residual"
FREQ = 298e6
L = M = N = 128
DX = 2e-3
N_ELL = 12
TOL = 1e-6
RESTART = 50
WORKLOAD = ("single body 128^3 @2mm, 12-ellipsoid phantom, 298 MHz plane wave, J-VIE form 2, "
            "GMRES(50) restarts, solved to 1e-6 FP64 relative residual")


def headline_config(er, world):
    """The c2 workload as both arms report it (the problem, not the method)."""
    return {"workload": WORKLOAD, "grid": [L, M, N], "fft_grid": [2 * L, 2 * M, 2 * N],
            "dofs": int(3 * np.count_nonzero(np.abs(er - 1) > 1e-12)),
            "l2": "working set (fN 0.8 GB + spectra 0.3 GB) > L2", "parallelism": f"replicas x{world}"}
# FP64 GMRES iterations of this workload (seed 0), measured by the FP64 arm on
# GB300 (iter = [20, 5]: four full cycles of 50 and 20 steps; the CPU
# restatement takes the same iterations by parity); used only to scale the CPU
# arm's per-iteration time to solves/s.
FP64_ITERATIONS_C2 = 220
# DRAM traffic of one z-pass launch (k_zmul<float,256>) at this workload, read
# from the committed ncu summary of that kernel.
ZMUL_PROFILE = ROOT / "profiles" / "k_zmul_f32_128cube.md"


def zmul_traffic():
    """dram__bytes_read.sum + dram__bytes_write.sum per launch, or None."""
    try:
        for line in ZMUL_PROFILE.read_text().splitlines():
            if line.startswith("traffic_bytes_per_launch:"):
                return int(line.split(":")[1].split()[0])
    except OSError:
        pass
    return None


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d["hbm_gbs"], "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.path = Path(tempfile.gettempdir()) / f"marie_bench_clocks_{os.getpid()}_{index}.csv"

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}",
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().strip().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_problem(seed):
    from marie_gb300 import phantoms

    r, er, scale = phantoms.ellipsoids(L, M, N, DX, N_ELL, seed, FREQ)
    return r, er


def dist_init():
    from marie_gb300 import replicas

    return replicas.init("nccl")


def reduce_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_gpu(args, world, rank, local):
    import ctypes as C

    import torch

    import marie_gb300 as mg
    from marie_gb300 import _lib, vie

    torch.cuda.set_device(local)
    lib = _lib.load()
    r, er = make_problem(seed=rank)
    em = mg.EMconstants(FREQ)
    E, _ = mg.PlaneWave_Excitation(r, [0, 0, em["ko"]], em["omega_mu"], [1, 0, 0])
    dev = torch.device("cuda", local)
    t_asm0 = time.perf_counter()
    op = mg.Operator.assemble(L, M, N, DX, FREQ, precision="mixed")
    torch.cuda.synchronize()
    t_asm = time.perf_counter() - t_asm0

    def colmajor(a):
        t = torch.from_numpy(np.ascontiguousarray(np.asarray(a).transpose(*range(a.ndim - 1, -1, -1))))
        return t.to(dev).permute(*range(a.ndim - 1, -1, -1))

    Ed, erd = colmajor(E), colmajor(er)
    stream = torch.cuda.ExternalStream(lib.marie_plan_stream(op.plan))

    def solve(opr, Ein, e_r, rr):
        return mg.JVIE_Solver(Ein, e_r, rr, FREQ, opr, tol=TOL, form=2, inner_it=RESTART, outer_it=200, solver="G")

    if args.solve_only:
        # profiling entry: the mixed solves of the timed region and nothing else,
        # with the schedule the autotuner picks for this grid on an idle GPU
        # (fused x+y passes, default radix schedules; a tuning run under a
        # profiler would time the candidates serialised and could pick another)
        op.set_schedule(1, 0, 0)
        # refinement steps and restart cycles driven from the host (plain
        # graphs): ncu does not profile kernels inside conditional graphs;
        # the kernels and their results are those of the one-launch solve.
        # --graph-form keeps the one-launch form (for ncu --graph-profiling graph)
        op.set_graph_refinement(args.graph_form)
        for _ in range(args.warmup + args.steps):
            res = solve(op, Ed, erd, r)
        torch.cuda.synchronize()
        return {"solve_only": True, "flag": res[1], "relres": res[2], "iter": res[3]} if rank == 0 else {}

    # schedule autotuner (outside the timed region): fused / five-pass x-y
    # passes and their radix schedule, z-pass radix schedule and columns per CTA
    tuned, tune_cands = op.autotune()
    # the stated precision split: FP32 matvec, Arnoldi in FP64 (the default)
    op.set_inner_precision("fp64")

    # --- timed region: mixed-precision solves, inputs resident in HBM --------
    for _ in range(args.warmup):
        res = solve(op, Ed, erd, r)
    barrier(world)
    torch.cuda.synchronize()
    n0 = lib.marie_launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            res = solve(op, Ed, erd, r)
        ev1.record(stream)
        ev1.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    launches = lib.marie_launch_count() - n0
    elapsed = ev0.elapsed_time(ev1) / 1e3
    elapsed_max = reduce_max(elapsed, world)
    Jm, flag_m, relres_m, iter_m, resvec_m, _ = res
    ms_per_step = elapsed_max / args.steps * 1e3
    value = world * args.steps / elapsed_max

    # --- e2e: the same solves through the reference-facing C ABI
    # (marie_jvie_solve, the call a MEX gateway makes) with host buffers: the
    # excitation and e_r copied in and Je copied out by the library every
    # solve, into a host output allocated per solve as a gateway allocates its
    # mxArray; right after the device-resident timing so that both see the
    # same GPU state
    Eh, erh = np.asfortranarray(E), np.asfortranarray(er)
    rv_cap = 1 + RESTART * 201 * 4
    rv = np.zeros(rv_cap)

    def solve_cabi():
        Jh = np.empty((L, M, N, 3), dtype=np.complex128, order="F")
        flag, relres, rlen, st = C.c_int(), C.c_double(), C.c_int64(), C.c_double()
        it = (C.c_double * 2)()
        _lib.check(lib.marie_jvie_solve(op.plan, C.c_void_p(Eh.ctypes.data), C.c_void_p(erh.ctypes.data), DX, FREQ,
                                        TOL, 2, b"G", b"\0", 1000, RESTART, 200, 5, C.c_void_p(Jh.ctypes.data),
                                        C.byref(flag), C.byref(relres), it, rv.ctypes.data_as(_lib._dp), rv_cap,
                                        C.byref(rlen), C.byref(st)))
        return Jh, flag.value, relres.value, st.value

    solve_cabi()
    barrier(world)
    torch.cuda.synchronize()
    ne2e = max(1, args.steps)
    e2e_ms, e2e_lib_ms = [], []
    with Clocks(local) as clk_e2e:
        t0 = time.perf_counter()
        for _ in range(ne2e):
            t1 = time.perf_counter()
            Jh, fh, rh, lib_s = solve_cabi()
            e2e_ms.append(round(1e3 * (time.perf_counter() - t1), 2))
            e2e_lib_ms.append(round(1e3 * lib_s, 2))  # inside marie_jvie_solve, staging included
            assert fh == 0 and rh <= TOL, (fh, rh)
            del Jh
        t_e2e = (time.perf_counter() - t0) / ne2e
    t_e2e = reduce_max(t_e2e, world)

    out = {}
    if rank == 0:
        # --- FP64 arm (the reference arithmetic on the GPU) -------------------
        op64 = mg.Operator.from_array(op.to_array(), precision="fp64")
        t0 = time.perf_counter()
        J64, flag64, relres64, it64, resvec64, _ = solve(op64, Ed, erd, r)
        torch.cuda.synchronize()
        t64 = time.perf_counter() - t0
        n_it64 = len(resvec64) - 1
        field_err = float((torch.linalg.norm(Jm - J64) / torch.linalg.norm(J64)).item())

        # --- the same mixed solve with an FP32 Krylov basis in the inner solves
        # (an opt-in that departs from the stated split), CUDA events
        op.set_inner_precision("fp32")
        solve(op, Ed, erd, r)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        n32 = max(1, min(args.steps, 3))
        e0.record(stream)
        for _ in range(n32):
            Ji, fi, ri, iti, resi, _ = solve(op, Ed, erd, r)
        e1.record(stream)
        e1.synchronize()
        t32 = e0.elapsed_time(e1) / 1e3 / n32
        inner32 = {"flag": fi, "relres": ri, "iter": iti, "matvecs": len(resi) - 1, "seconds": round(t32, 4),
                   "solves_per_s": round(1 / t32, 4), "speedup_vs_fp64": round(t64 / t32, 3),
                   "field_rel_err_vs_fp64": float((torch.linalg.norm(Ji - J64) / torch.linalg.norm(J64)).item())}
        op.set_inner_precision("fp64")
        del Ji

        # --- the other solvers of JVIE_Solver, mixed precision, one solve each
        variants = {}
        for sv in ("B", "D"):
            t0 = time.perf_counter()
            Jv, fv, rv, itv, resv, _ = mg.JVIE_Solver(Ed, erd, r, FREQ, op, tol=TOL, form=2, solver=sv,
                                                      inner_it=RESTART, outer_it=200)
            torch.cuda.synchronize()
            tv = time.perf_counter() - t0
            variants["bicgstab" if sv == "B" else "pgmresDR"] = {
                "flag": fv, "relres": rv, "iter": itv, "seconds": round(tv, 4),
                "field_rel_err_vs_fp64_gmres": float((torch.linalg.norm(Jv - J64) / torch.linalg.norm(J64)).item())}

        # --- matvec times on the solver's DOFs ------------------------------
        mv = matvec_times(mg, op, op64, er, lib)

        V = L * M * N
        hbm, kind = peaks()
        dom = mv["dominant"]
        out = {
            "metric": METRIC, "value": round(value, 4), "unit": "solves/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_per_step, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c64 matvec + inner krylov / c128 refinement",
            "data": "synthetic (seeded ellipsoid phantom, plane wave)",
            "config": headline_config(er, world),
            "method": "mixed precision: inner GMRES with the FP32 matvec and an FP64 Krylov basis "
                      "(Arnoldi, Givens and residual estimates in FP64; restart 20), FP64 true residuals and "
                      "refinement (GMRES-IR); the whole solve is one CUDA graph launch (nested conditional "
                      "WHILE nodes)",
            "solve": {"mixed": {"flag": flag_m, "relres": relres_m, "iter": iter_m,
                                "matvecs": len(resvec_m) - 1, "solves_per_s": round(value / world, 4)},
                      "fp64": {"flag": flag64, "relres": relres64, "iter": it64, "iterations": n_it64,
                               "seconds": round(t64, 4), "solves_per_s": round(1 / t64, 4)},
                      "speedup_mixed_vs_fp64": round(t64 / (ms_per_step / 1e3), 3),
                      "field_rel_err_mixed_vs_fp64": field_err, "mixed_inner_fp32_basis": inner32,
                      "mixed_other_solvers": variants},
            "matvec_ms": {"fp32": mv["fp32_ms"], "fp64": mv["fp64_ms"], "fp32_passes_ms": mv["fp32_passes"],
                          "fp64_passes_ms": mv["fp64_passes"], "fp32_cufft_comparison": mv["fp32_cufft_ms"],
                          "fp32_bound": mv["fp32_bound_ms"], "fp64_bound": mv["fp64_bound_ms"],
                          "note": "fp32/fp64: marie_mv_AN per call, which rebuilds the DOF map and coefficients; "
                                  "*_bound: marie_plan_apply_mv_AN, the solver's matvec (map and coefficients "
                                  "bound once; FP32 epilogue in FP32)"},
            "assembly_s": round(t_asm, 3),
            "autotune": {"chosen": {"fused_xy": tuned[0], "xy_variant": tuned[1], "z_variant": tuned[2]},
                         "candidates_ms": [{"fused_xy": f, "xy_variant": fv, "z_variant": z, "ms": round(ms, 4)}
                                           for f, fv, z, ms in tune_cands]},
            "roofline": {"bound": "hbm", "kernel": dom["name"], "achieved": round(dom["gbs"], 1), "peak": hbm,
                         "unit": "GB/s", "frac": round(dom["gbs"] / hbm, 4),
                         "traffic": zmul_traffic() if dom["name"] == "z_multiply" else None,
                         "peak_kind": kind, "alg_bytes_per_launch": dom["bytes"]},
            "matvec_roofline": {"alg_bytes": mv["alg_bytes"], "gbs": round(mv["alg_bytes"] / (mv["fp32_ms"] / 1e3) / 1e9, 1),
                                "frac": round(mv["alg_bytes"] / (mv["fp32_ms"] / 1e3) / 1e9 / hbm, 4),
                                "bound_gbs": round(mv["alg_bytes"] / (mv["fp32_bound_ms"] / 1e3) / 1e9, 1),
                                "bound_frac": round(mv["alg_bytes"] / (mv["fp32_bound_ms"] / 1e3) / 1e9 / hbm, 4)},
            "e2e": {"value": round(world / t_e2e, 4), "unit": "solves/s", "h2d_bytes_per_step": 4 * V * 16,
                    "d2h_bytes_per_step": 3 * V * 16, "per_solve_ms": e2e_ms, "library_ms": e2e_lib_ms,
                    "clocks": clk_e2e.summary()},
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
        }
        if world == 1 and not args.no_cpu:
            out["cpu_baseline"] = cpu_baseline(n_it64, budget_s=args.cpu_budget)
    return out


def matvec_times(mg, op, op64, er, lib):
    """FP32 and FP64 matvec times (CUDA events, averaged) on the solver's DOFs."""
    import ctypes as C

    import torch

    V = L * M * N
    idxS = np.nonzero(np.abs(er.reshape(-1, order="F") - 1) > 1e-12)[0] + 1
    idx = np.concatenate([idxS, V + idxS, 2 * V + idxS]).astype(np.int64)
    n = idx.size
    dev = torch.device("cuda")
    Mr = torch.ones(V, dtype=torch.complex128, device=dev)
    erf = torch.from_numpy(er.reshape(-1, order="F")).to(dev)
    Mc = (erf - 1) / erf
    idx_d = torch.from_numpy(idx).to(dev)
    J = torch.randn(n, dtype=torch.complex128, device=dev)
    out = torch.empty_like(J)
    res = {}
    for name, opr, prec in (("fp32", op, 32), ("fp64", op64, 64)):
        st = torch.cuda.ExternalStream(lib.marie_plan_stream(opr.plan))
        reps = 20 if prec == 32 else 5

        def call():
            s = lib.marie_mv_AN(opr.plan, C.c_void_p(J.data_ptr()), C.c_void_p(Mr.data_ptr()),
                                C.c_void_p(Mc.data_ptr()), 8e-9, 0, C.c_void_p(idx_d.data_ptr()), n,
                                C.c_void_p(out.data_ptr()), 1, prec)
            assert s == 0, lib.marie_last_error()

        for _ in range(3):
            call()
        # per-pass profile
        pm = (C.c_double * 5)()
        cnt = C.c_int64()
        lib.marie_plan_profile(opr.plan, 1, pm, C.byref(cnt))
        for _ in range(reps):
            call()
        lib.marie_plan_profile(opr.plan, 0, pm, C.byref(cnt))
        passes = [round(x, 4) for x in pm]
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            call()
        e1.record(st)
        e1.synchronize()
        res[name + "_ms"] = round(e0.elapsed_time(e1) / reps, 4)
        res[name + "_passes"] = passes
        # the same product with the DOF map and coefficients bound to the plan
        # once (marie_plan_apply_mv_AN: the solver's matvec, no per-call set-up;
        # FP32 with its epilogue in FP32 as in the inner solves)
        opr.bind_mv_AN(Mr, Mc, 8e-9, "notransp", idx_d)

        def apply():
            s = lib.marie_plan_apply_mv_AN(opr.plan, C.c_void_p(J.data_ptr()), C.c_void_p(out.data_ptr()), 1, prec)
            assert s == 0, lib.marie_last_error()

        for _ in range(3):
            apply()
        st.synchronize()
        e0.record(st)
        for _ in range(reps):
            apply()
        e1.record(st)
        e1.synchronize()
        res[name + "_bound_ms"] = round(e0.elapsed_time(e1) / reps, 4)
    # the same FP32 matvec through cuFFT (padded arrays, full operator), for comparison
    ms = C.c_float()
    cf = []
    for _ in range(3 + 10):
        s = lib.marie_mv_AN_cufft(op.plan, C.c_void_p(J.data_ptr()), C.c_void_p(Mr.data_ptr()),
                                  C.c_void_p(Mc.data_ptr()), 8e-9, C.c_void_p(idx_d.data_ptr()), n,
                                  C.c_void_p(out.data_ptr()), C.byref(ms))
        assert s == 0, lib.marie_last_error()
        cf.append(ms.value)
    res["fp32_cufft_ms"] = round(float(np.median(cf[3:])), 4)
    # algorithmic bytes (complex64 spectra), per pass and per matvec
    S = 8
    Lp, Mp = 2 * L, 2 * M
    fN_oct = 6 * (L + 1) * (M + 1) * (N + 1) * S
    x_spec = 3 * Lp * M * N * S     # 3 x N x M x 2L
    y_spec = 3 * Lp * Mp * N * S    # 3 x N x 2M x 2L
    vec = n * 16
    pass_bytes = [vec + x_spec, x_spec + y_spec, 2 * y_spec + fN_oct, y_spec + x_spec, x_spec + 4 * vec]
    names = ["x_forward", "y_forward", "z_multiply", "y_inverse", "x_inverse"]
    k = int(np.argmax(res["fp32_passes"]))
    res["dominant"] = {"name": names[k], "bytes": pass_bytes[k],
                       "gbs": pass_bytes[k] / (res["fp32_passes"][k] / 1e3) / 1e9}
    res["alg_bytes"] = S * 56 * V + fN_oct
    return res


# ---------------------------------------------------------------------------
# CPU arm (the oracle restatement of mv_AN + pgmres)
# ---------------------------------------------------------------------------
def cpu_iteration_time(budget_s=20.0):
    """Seconds per GMRES iteration of the CPU restatement at 128^3 (one mv_AN
    with scipy.fft on every host core, plus the CGS step at the mean basis size
    of GMRES(50)).  fN values do not change the FFT cost, so a seeded random
    operator of the right shape stands in for the assembled one."""
    from oracle import vie_oracle as vo

    workers = os.cpu_count() or 1
    r, er = make_problem(0)
    V = L * M * N
    rng = np.random.default_rng(0)
    fN = (rng.standard_normal((2 * L, 2 * M, 2 * N, 6)) + 1j * rng.standard_normal((2 * L, 2 * M, 2 * N, 6)))
    Mr = np.ones((L, M, N), complex)
    Mc = (er - 1) / er
    idxS = np.nonzero(np.abs(er.reshape(-1, order="F") - 1) > 1e-12)[0] + 1
    idx = np.concatenate([idxS, V + idxS, 2 * V + idxS])
    n = idx.size
    J = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    vo.mv_AN(J, fN, Mr, Mc, DX**3, "notransp", idx, workers)  # warm-up / plan
    t0 = time.perf_counter()
    reps = 0
    while True:
        vo.mv_AN(J, fN, Mr, Mc, DX**3, "notransp", idx, workers)
        reps += 1
        if time.perf_counter() - t0 > budget_s * 0.7 or reps >= 10:
            break
    t_mv = (time.perf_counter() - t0) / reps
    k = RESTART // 2
    Vb = rng.standard_normal((n, k)) + 1j * rng.standard_normal((n, k))
    t0 = time.perf_counter()
    h = Vb.conj().T @ J
    w = J - Vb @ h
    np.linalg.norm(w)
    t_cgs = time.perf_counter() - t0
    return t_mv + t_cgs, workers, reps, t_mv, t_cgs


def cpu_baseline(iterations, budget_s=20.0):
    t_it, workers, reps, t_mv, t_cgs = cpu_iteration_time(budget_s)
    solves = 1.0 / (t_it * iterations) if iterations else None
    return {"value": solves, "unit": "solves/s", "cores": workers, "kind": "port",
            "sample": f"{reps} oracle mv_AN calls at 128^3 (complex128, scipy.fft workers={workers}) "
                      f"+ one CGS step at 25 basis vectors = {t_it:.3f} s/iteration, x {iterations} "
                      f"FP64 GMRES iterations of this workload"}


def run_reference(args, world, rank):
    if rank != 0:
        return None
    iters = FP64_ITERATIONS_C2
    times = []
    for i in range(args.warmup + args.steps):
        t_it, workers, reps, t_mv, t_cgs = cpu_iteration_time(budget_s=args.cpu_budget / max(1, args.steps))
        if i >= args.warmup:
            times.append(t_it)
    t = statistics.mean(times)
    value = 1.0 / (t * iters) if iters else 1.0 / t
    unit = "solves/s" if iters else "GMRES iterations/s"
    return {"metric": METRIC, "value": value, "unit": unit, "impl": "reference", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": headline_config(make_problem(0)[1], world),
            "method": "FP64 pgmres with the FFT mv_AN, restated on the CPU (numpy / scipy.fft)",
            "cpu_baseline": {"value": value, "unit": unit, "cores": workers, "kind": "port",
                             "sample": f"one GMRES iteration (mv_AN + CGS) per step, scaled by {iters} "
                                       f"iterations per solve"},
            "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ---------------------------------------------------------------------------
# the other workloads: extra keys of the main line (world 1), or their own line
# with --config cX
# ---------------------------------------------------------------------------
def _timed(fn, steps, warmup):
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = None
    for _ in range(steps):
        out = fn()
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) / steps, out


def config_c1(steps, warmup):
    """32^3 Mie sphere (r 7.5 cm, eps_r 50, sigma 0.5 S/m, 5 mm), plane wave,
    GMRES(50) to 1e-6: FP64 and mixed solves (the Mie comparison itself is a
    test against the analytic series)."""
    import marie_gb300 as mg
    from marie_gb300 import phantoms

    em = mg.EMconstants(FREQ)
    Lc, dx, R = 32, 5e-3, 0.075
    r, er = phantoms.sphere(Lc, Lc, Lc, dx, R, 50.0, 0.5, FREQ)
    E, _ = mg.PlaneWave_Excitation(r, [0, 0, em["ko"]], em["omega_mu"], [1, 0, 0])
    res = {"workload": "32^3 sphere r 7.5 cm, eps_r 50, sigma 0.5 S/m, 5 mm, plane wave, GMRES(50), tol 1e-6"}
    for prec in ("fp64", "mixed"):
        op = mg.Operator.assemble(Lc, Lc, Lc, dx, FREQ, precision=prec)
        t, out = _timed(lambda: mg.JVIE_Solver(E, er, r, FREQ, op, tol=1e-6, solver="G"), steps, warmup)
        res[prec] = {"seconds": round(t, 5), "iter": out[3], "relres": out[2], "matvecs": len(out[4]) - 1}
        op.close()
    return res


def config_c3(steps, warmup, world=1, rank=0):
    """16 z-directed dipoles on a 0.15 m cylinder around the 128^3 body, one
    lockstep batch per rank (its share of the 16); three uneven bodies 48^3,
    64^3, 96^3 (seeds 1-3) with 4 dipoles each, its share of the bodies
    solved concurrently.  Throughput = all units / max time over ranks."""
    import torch

    import marie_gb300 as mg
    from marie_gb300 import phantoms, replicas

    em = mg.EMconstants(FREQ)
    res = {"workload": "16 dipoles (4 azimuths x z in {-5,0,5,10} cm, rho 0.15 m) on the 128^3 body; "
                       "bodies 48^3/64^3/96^3 (seeds 1-3) x 4 dipoles"}
    r, er = make_problem(0)
    pos = phantoms.dipole_ring(0.15, [-0.05, 0.0, 0.05, 0.10], 4)
    mine = replicas.shard(len(pos), rank, world)
    units = []
    t_b = 0.0
    if mine:
        Eb = np.asfortranarray(np.stack([np.asarray(mg.Dipole_Excitation(r, em["ko"], np.array([[0, 0, 1.0]]),
                                                                         pos[e][None])) for e in mine], axis=4))
        op = mg.Operator.assemble(L, M, N, DX, FREQ, precision="mixed", nrhs_max=len(mine))
        t_b, out = _timed(lambda: mg.JVIE_Solver_batch(Eb, er, r, FREQ, op, tol=TOL), steps, warmup)
        units = [(e, int(out[1][i]), float(out[2][i]), [int(x) for x in out[3][i]]) for i, e in enumerate(mine)]
        del Eb
        op.close()
    dev = torch.device("cuda", torch.cuda.current_device())
    t_max = replicas.max_over_ranks(t_b, world, dev)
    allu = replicas.gather_results(units, world)
    res["batch16"] = {"seconds": round(t_max, 4), "excitation_solves_per_s": round(len(pos) / t_max, 4),
                      "flags": [u[1] for u in allu], "max_relres": max(u[2] for u in allu),
                      "iters": [u[3] for u in allu], "units_solved": [u[0] for u in allu]}
    specs = ((1, 48), (2, 64), (3, 96))
    mine_b = replicas.shard(len(specs), rank, world)
    bodies, t_u, ub = [], 0.0, []
    for i in mine_b:
        seed, Lb = specs[i]
        rb, erb, _ = phantoms.ellipsoids(Lb, Lb, Lb, DX, N_ELL, seed, FREQ)
        pb = phantoms.dipole_ring(0.15, [0.0], 4)
        Eb = np.asfortranarray(np.stack([np.asarray(mg.Dipole_Excitation(rb, em["ko"], np.array([[0, 0, 1.0]]),
                                                                         p[None])) for p in pb], axis=4))
        bodies.append((Eb, erb, rb, mg.Operator.assemble(Lb, Lb, Lb, DX, FREQ, precision="mixed", nrhs_max=4)))
    if bodies:
        t_u, out = _timed(lambda: mg.JVIE_Solver_bodies(bodies, FREQ, tol=TOL), steps, warmup)
        ub = [(specs[i][1], [int(f) for f in o[1]]) for i, o in zip(mine_b, out[0])]
    t_umax = replicas.max_over_ranks(t_u, world, dev)
    allb = replicas.gather_results(ub, world)
    res["bodies_48_64_96x4"] = {"seconds": round(t_umax, 4), "excitation_solves_per_s": round(12 / t_umax, 4),
                                "flags": [b[1] for b in allb], "bodies_solved": [b[0] for b in allb]}
    for b in bodies:
        b[3].close()
    return res


def config_c4(steps, warmup):
    """64^3 phantom at 3 mm, plane wave: absorbed-power adjoint gradient, FP64
    and mixed precision, and the difference between the two gradients."""
    import marie_gb300 as mg
    from marie_gb300 import phantoms
    from marie_gb300.autograd import adjoint_gradient

    em = mg.EMconstants(FREQ)
    Lc, dx = 64, 3e-3
    r, er, _ = phantoms.ellipsoids(Lc, Lc, Lc, dx, N_ELL, 0, FREQ)
    E, _ = mg.PlaneWave_Excitation(r, [0, 0, em["ko"]], em["omega_mu"], [1, 0, 0])
    res = {"workload": "64^3 ellipsoid phantom at 3 mm, plane wave, absorbed-power gradient w.r.t. eps_r and sigma"}
    grads = {}
    for prec in ("fp64", "mixed"):
        op = mg.Operator.assemble(Lc, Lc, Lc, dx, FREQ, precision=prec)
        t, out = _timed(lambda: adjoint_gradient(op, E, er, dx, FREQ, "power", None, TOL), steps, warmup)
        res[prec] = {"seconds_per_gradient": round(t, 4), "F": out[0], "flags": out[3], "iters": out[4]}
        grads[prec] = out[1:3]
        op.close()
    res["grad_rel_diff_mixed_vs_fp64"] = [float(np.linalg.norm(a - b) / np.linalg.norm(a))
                                          for a, b in zip(grads["fp64"], grads["mixed"])]
    return res


def config_c5():
    """256x192x160 at 2 mm (512x384x320 FFT), 40 ellipsoids, 8 dipoles on a
    0.2 m cylinder: assembly, the 8 excitations in one batch, and the
    absorbed-power gradient of the summed excitation."""
    import marie_gb300 as mg
    from marie_gb300 import phantoms
    from marie_gb300.autograd import adjoint_gradient

    em = mg.EMconstants(FREQ)
    Lc, Mc, Nc = 256, 192, 160
    r, er, _ = phantoms.ellipsoids(Lc, Mc, Nc, DX, 40, 0, FREQ)
    pos = phantoms.dipole_ring(0.2, [-0.05, 0.05], 4)
    Es = [np.asarray(mg.Dipole_Excitation(r, em["ko"], np.array([[0, 0, 1.0]]), p[None])) for p in pos]
    Eb = np.asfortranarray(np.stack(Es, axis=4))
    res = {"workload": "256x192x160 at 2 mm, 40 ellipsoids, 8 dipoles (rho 0.2 m), batch + summed-excitation "
                       "gradient"}
    t0 = time.perf_counter()
    op = mg.Operator.assemble(Lc, Mc, Nc, DX, FREQ, precision="mixed", nrhs_max=8)
    res["assembly_s"] = round(time.perf_counter() - t0, 3)
    t, out = _timed(lambda: mg.JVIE_Solver_batch(Eb, er, r, FREQ, op, tol=TOL), 1, 0)
    res["batch8"] = {"seconds": round(t, 4), "flags": out[1].tolist(), "max_relres": float(out[2].max()),
                     "iters": out[3].tolist()}
    del Eb, out
    Esum = np.asfortranarray(sum(Es))
    t, g = _timed(lambda: adjoint_gradient(op, Esum, er, DX, FREQ, "power", None, TOL), 1, 0)
    res["gradient"] = {"seconds": round(t, 4), "F": g[0], "flags": g[3], "iters": g[4]}
    op.close()
    return res


def run_configs(which, world, rank):
    """The other workloads as a dict of per-config results; a failure is
    recorded under its config instead of ending the run."""
    import torch

    import marie_gb300 as mg

    out = {}
    for c in which:
        try:
            if c == "c3":
                out[c] = config_c3(1, 1, world, rank)
            elif rank == 0:
                out[c] = {"c1": lambda: config_c1(3, 1), "c4": lambda: config_c4(1, 1), "c5": config_c5}[c]()
        except Exception as exc:  # noqa: BLE001 - reported in the JSON line
            out[c] = {"error": f"{type(exc).__name__}: {exc}"}
        torch.cuda.synchronize()
        mg.release_cached_memory()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="marie", choices=["marie", "reference"])
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--solve-only", action="store_true", help="run the mixed solves only (for profilers)")
    ap.add_argument("--graph-form", action="store_true",
                    help="with --solve-only: the one-launch (conditional graph) form of the solve")
    ap.add_argument("--configs", default="c1,c3,c4,c5",
                    help="other workloads reported as extra keys of the main line ('' for none)")
    ap.add_argument("--config", default="c2", choices=["c1", "c2", "c3", "c4", "c5"])
    args = ap.parse_args()
    from marie_gb300 import replicas

    if args.gpus > 1 and not replicas.under_launcher():
        sys.exit(replicas.relaunch(args.gpus, __file__, sys.argv[1:]))
    world, rank, local = dist_init()
    if args.impl == "marie":
        import torch

        torch.cuda.set_device(local)
    if args.config != "c2":
        res = run_configs([args.config], world, rank)
        if rank == 0:
            print(json.dumps({"config": args.config, "n_gpus": world, **res[args.config]}, default=float))
        replicas.finish(world)
        return
    if args.impl == "reference":
        out = run_reference(args, world, rank)
    else:
        out = run_gpu(args, world, rank, local)
        which = [c for c in args.configs.split(",") if c] if not args.solve_only else []
        if world > 1:
            which = [c for c in which if c == "c3"]
        if which:
            extra = run_configs(which, world, rank)
            if rank == 0 and out:
                out["configs"] = extra
    if rank == 0 and out:
        print(json.dumps(out, default=float))
    replicas.finish(world)


if __name__ == "__main__":
    main()
