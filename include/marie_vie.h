/*
 * marie_vie.h -- C ABI of the GB300 J-VIE solve path.
 *
 * Drop-in boundary for the FFT-accelerated current-based volume integral
 * equation (J-VIE) path of MARIE: operator assembly (getOPERATORS), the
 * circulant matvec (mv_AN / mv_L) and restarted GMRES (pgmres), plus the
 * JVIE_Solver driver that strings them together.  Every entry point takes plain
 * pointers and sizes; no C++ or torch types cross this boundary.
 *
 * Conventions (same as the reference MATLAB arrays):
 *   - complex data is interleaved (re, im) doubles, i.e. double2;
 *   - grid arrays are column-major: x fastest, then y, then z, then component;
 *   - idx vectors are 1-based int64 linear indices into an L x M x N x 3 array
 *     (the MATLAB vector idxS3), translated on the device;
 *   - a pointer argument may be host memory (copied, as gpuArray/gather do) or
 *     device memory (used in place); the library tells them apart itself;
 *   - every call returns MARIE_OK (0) or a negative status; marie_last_error()
 *     gives the message of the last failure on the calling thread.
 *
 * A plan binds one grid size, one CUDA stream and the device memory of the
 * operator; calls on one plan are serialised on that stream.
 */
#ifndef MARIE_VIE_H
#define MARIE_VIE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define MARIE_OK 0
#define MARIE_EINVAL (-1)      /* bad argument, shape or index                */
#define MARIE_ENOMEM (-2)      /* device allocation failed                   */
#define MARIE_ECUDA (-3)       /* CUDA runtime error                         */
#define MARIE_ENOCONV (-4)     /* reserved: non-convergence is reported by flag */
#define MARIE_EBREAKDOWN (-5)  /* Arnoldi breakdown with a non-finite residual */
#define MARIE_ETIMEOUT (-6)    /* a bounded device wait ran out              */
#define MARIE_EUNSUPPORTED (-7) /* FFT length or configuration not built     */
#define MARIE_ENOOP (-8)       /* plan has no operator (set or assemble first) */

/* arithmetic of the circulant matvec */
#define MARIE_FP64 64
#define MARIE_FP32 32
#define MARIE_MIXED 96 /* FP32 matvec inside FP64 GMRES with FP64 refinement */

typedef struct marie_plan marie_plan;

/* y = A(x) on device vectors of length n (nrhs = 1).  Returns a status. */
typedef int (*marie_op_fn)(void* ctx, const double* x, double* y, int64_t n);

const char* marie_last_error(void);
int marie_version(void);

/* Create a plan for an L x M x N voxel grid (FFT grid 2L x 2M x 2N).
 * precision: MARIE_FP64, MARIE_FP32 or MARIE_MIXED; nrhs_max bounds batched
 * calls; stream is a cudaStream_t (NULL = a stream owned by the plan). */
int marie_plan_create(int64_t L, int64_t M, int64_t N, int precision, int64_t nrhs_max,
                      void* stream, marie_plan** plan);
int marie_plan_destroy(marie_plan* plan);
/* Device stream of the plan (a cudaStream_t). */
void* marie_plan_stream(marie_plan* plan);

/* Replaces getOPERATORS(r, f, op, type, singular)
 * (src_vie/src_operators/getOPERATORS.m:1-127) for op = 'N' (6 components)
 * and op = 'K' (3 components [Kx, Ky, Kz], assembly_kop.m; singular unused).
 *   r:       L x M x N x 3 voxel centres (uniform spacing; dx = r[1]-r[0])
 *   type:    'F' FFT of the circulant (2L x 2M x 2N x 6, the default 'FFTofC'),
 *            'C' circulant (2L x 2M x 2N x 6), 'T' Toeplitz (L x M x N x 6)
 *   singular:'D' (the reference default 'DIRECTFN', getOPERATORS.m:39-41)
 *            computes the weakly singular self/edge/vertex integrals on the
 *            device with DIRECTFN at Np_1D = 20 (assembly_nop.m:16,96-98);
 *            'C' uses a converged 4-D quadrature instead (not a reference
 *            method; differs from DIRECTFN@20 by up to 3.4e-5 relative);
 *            'U' uses the five values in singular_values = {ST, EAc, EAo,
 *            VAc, VAo} (complex).  'E' ('DEMCEM') is not built: MARIE_EINVAL.
 *   op_out:  complex output, host or device.
 * Component order [xx, xy, xz, yy, yz, zz] as vector_projection.m:15-22. */
int marie_get_operators(const double* r, int64_t L, int64_t M, int64_t N, double f, char op,
                        char type, char singular, const double* singular_values, double* op_out);

/* The five singular integrals {ST, EAc, EAo, VAc, VAo} (complex, out10 =
 * 5 x (re, im)) for cubic voxels of edge dx and wavenumber ko: replaces
 * singular_st.m / singular_ea.m / singular_va.m with method 'DIRECTFN' at
 * Np_1D = 20, as assembly_nop.m:96-98 calls them. */
int marie_singular_integrals(double ko, double dx, double* out10);
/* The same with the method ('D' DIRECTFN, 'C' converged quadrature) and its
 * order np_1d (0: 20 for 'D', 32 for 'C'; DIRECTFN takes 1..64). */
int marie_singular_integrals_ex(double ko, double dx, char method, int np_1d, double* out10);
/* One call of a DIRECTFN core for constant basis functions on a triangle
 * pair, with the MEX gateway's arguments (vertices: 3 x kind-count doubles):
 *   kind 'S': mexdirectfn_ws_st_const(r1, r2, r3, ko, Np_1D)
 *             (mexcubatures/directfn_ws_st_const_mex.cpp:47)
 *   kind 'E': mexdirectfn_ws_ea_const(r1, r2, r3, r4, ko, Np_1D)
 *             (directfn_ws_ea_const_mex.cpp:50: second triangle (r4, r2, r1))
 *   kind 'V': mexdirectfn_ws_va_const(r1, r2, r3, r4, r5, ko, Np_1D)
 *             (directfn_ws_va_const_mex.cpp:51: second triangle (r4, r5, r1))
 * out2 = (re, im).  Np_1D in 1..64. */
int marie_directfn(char kind, const double* vertices, double ko, int np_1d, double* out2);

/* Upload an FFT-of-circulant operator fN (2L x 2M x 2N x 6 complex), as
 * gpuArray(fN) in JVIE_Solver.m:271.  Converted to the plan's precisions. */
int marie_set_operator(marie_plan* plan, const double* fN, int64_t Lf, int64_t Mf, int64_t Nf);
/* Assemble the operator on the device for this plan's grid (no host copy). */
int marie_plan_assemble(marie_plan* plan, double dx, double freq, char singular,
                        const double* singular_values);
/* The K operator of getOPERATORS(r, f, 'K') for mv_K / H_field_Kop, uploaded
 * (2L x 2M x 2N x 3 complex, as gpuArray(fK)) or assembled on the device. */
int marie_set_operator_k(marie_plan* plan, const double* fK, int64_t Lf, int64_t Mf, int64_t Nf);
int marie_plan_assemble_k(marie_plan* plan, double dx, double freq);
/* Copy the plan's FP64 operator out (2L x 2M x 2N x 6 complex, host or device). */
int marie_get_plan_operator(marie_plan* plan, double* fN_out);

/* Replaces mv_AN(JIn0, fN, Mr, Mc, Gram, transp_flag, idx, GPU_flag)
 * (src_vie/src_mvp/mv_AN.m:1-146) with the plan's operator.
 *   JIn0, JOut: n_idx x nrhs complex (columns contiguous)
 *   Mr, Mc:     L x M x N complex
 *   transp:     0 = 'notransp', 1 = 'transp' (Hermitian adjoint)
 *   idx:        n_idx 1-based indices into L x M x N x 3 (no duplicates)
 *   precision:  MARIE_FP64 or MARIE_FP32 (arithmetic of the circulant part) */
int marie_mv_AN(marie_plan* plan, const double* JIn0, const double* Mr, const double* Mc,
                double Gram, int transp, const int64_t* idx, int64_t n_idx, double* JOut,
                int64_t nrhs, int precision);

/* No counterpart in the reference: marie_mv_AN (one right-hand side) that
 * allocates nothing, for callers that cannot let a library allocate device
 * memory when they ask for a matvec (a host whose device memory belongs to
 * another allocator, such as MATLAB's gpuArray pool or a serving runtime's
 * fixed arena, or a loop that must not block in cudaMalloc).  Its scratch is a
 * 64 MiB static device array that every GPU loading this library holds until
 * exit; grids needing more (about 204-252 bytes per voxel in FP32, 396 in FP64)
 * are rejected with MARIE_EINVAL.  Device pointers only.  The call runs on the
 * plan's device and stream (the caller's current device is restored) with the
 * plan's matvec schedule and blocks the host until that stream is done (it
 * reads the kernels' error flag), so it cannot be captured into a CUDA graph.
 * Calls share the array, so calls that overlap on the GPU race. */
int marie_mv_AN_static(marie_plan* plan, const double* JIn0, const double* Mr,
                       const double* Mc, double Gram, int transp, const int64_t* idx,
                       int64_t n_idx, double* JOut, int precision);

/* Replaces mv_L(JIn0, fN, r, Gram, idx, GPU_flag) (src_vie/src_mvp/mv_L.m:1-97):
 * JOut = crop(N J) - Gram*J on the entries idx. */
int marie_mv_L(marie_plan* plan, const double* JIn0, double Gram, const int64_t* idx,
               int64_t n_idx, double* JOut, int64_t nrhs, int precision);

/* Replaces mv_K(JIn0, fK, r, idx, GPU_flag) (src_vie/src_mvp/mv_K.m:1-93) with
 * the plan's K operator: JOut = crop(IFFT(fK x FFT(J))) on the entries idx,
 * the cross product [K3 J2 - K2 J3, K1 J3 - K3 J1, K2 J1 - K1 J2]. */
int marie_mv_K(marie_plan* plan, const double* JIn0, const int64_t* idx, int64_t n_idx,
               double* JOut, int64_t nrhs, int precision);

/* Binds mv_AN(., fN, Mr, Mc, Gram, transp_flag, idx) (src_vie/src_mvp/mv_AN.m:1)
 * to the plan, the handle fA = @(J) mv_AN(J, ...) that JVIE_Solver.m:211-297
 * passes to its solvers: marie_pgmres, marie_pgmres_dr and marie_bicgstab
 * called with a NULL operator apply it on the device.  Arguments as
 * marie_mv_AN; the plan keeps device copies of the DOF map and coefficients
 * until the next bind or marie_plan_destroy. */
int marie_plan_bind_mv_AN(marie_plan* plan, const double* Mr, const double* Mc, double Gram, int transp,
                          const int64_t* idx, int64_t n_idx);
/* JOut = mv_AN(JIn0) with the mv_AN bound to the plan (one call of the handle
 * fA of JVIE_Solver.m:211-297): no DOF map or coefficients are rebuilt per
 * call, unlike marie_mv_AN.  JIn0, JOut: n_idx x nrhs complex, host or device.
 * precision MARIE_FP32 runs the whole product in FP32 (transforms and the
 * epilogue Gram*Mr*J - Mc*(N J), the matvec of the mixed-precision inner
 * solves); MARIE_FP64 in FP64.  With device output the call returns without
 * waiting for the plan's stream (a bounded-wait timeout is then reported by
 * the next call that synchronises the plan); with host output it returns
 * after the copy. */
int marie_plan_apply_mv_AN(marie_plan* plan, const double* JIn0, double* JOut, int64_t nrhs, int precision);

/* Replaces pgmres(A, b, restart, tol, maxit, L1, L2, R1, R2, x0)
 * (src_numeric/src_iterative/pgmres.m:70-181, pgmres_iter.m:22-150): restarted
 * GMRES with classical Gram-Schmidt, function-handle preconditioners applied as
 * products, true residual recomputed at the end.  All vectors are device or
 * host (n complex); A/L1/L2/R1/R2 receive device vectors.  NULL L1..R2 = none;
 * NULL A = the mv_AN bound to the plan (marie_plan_bind_mv_AN), applied on the
 * device without a callback.  NULL x0 = zero start.  Outputs: x, flag (0
 * converged / 1 not), relres, iter = {inner, outer}, resvec (relative, length
 * written to *resvec_len). */
int marie_pgmres(marie_plan* plan, marie_op_fn A, void* A_ctx, const double* b, int64_t n,
                 int restart, double tol, int maxit, marie_op_fn L1, void* L1_ctx,
                 marie_op_fn L2, void* L2_ctx, marie_op_fn R1, void* R1_ctx, marie_op_fn R2,
                 void* R2_ctx, const double* x0, double* x, int* flag, double* relres,
                 int* iter, double* resvec, int64_t resvec_cap, int64_t* resvec_len);

/* Replaces pgmresDR(A, b, restart, tol, maxit, ritz, L1, L2, R1, R2, x0)
 * (src_numeric/src_iterative/pgmresDR.m:1-282, pgmresDR_iter.m:1-142,
 * getHarmVecs1.m, getHarmVecs2.m): GMRES(restart) that deflates ritz harmonic
 * Ritz vectors of each cycle into the next (ritz < 1: min(10, restart/2);
 * restart + ritz <= 127).  Arguments and outputs as marie_pgmres. */
int marie_pgmres_dr(marie_plan* plan, marie_op_fn A, void* A_ctx, const double* b, int64_t n,
                    int restart, double tol, int maxit, int ritz, marie_op_fn L1, void* L1_ctx,
                    marie_op_fn L2, void* L2_ctx, marie_op_fn R1, void* R1_ctx, marie_op_fn R2,
                    void* R2_ctx, const double* x0, double* x, int* flag, double* relres,
                    int* iter, double* resvec, int64_t resvec_cap, int64_t* resvec_len);

/* Replaces MATLAB's bicgstab(A, b, tol, maxit, M1, M2, x0), the solver 'B'
 * of JVIE_Solver.m:451-499 (a MATLAB built-in, outside the reference
 * sources): BiCGSTAB with MATLAB's outputs.  Vectors device or host (n
 * complex); A/M1/M2 receive device vectors, M1/M2 applied as ph = M2(M1(p)),
 * NULL = none (NULL A: the plan's bound mv_AN); NULL x0 = zero start.  flag 0 converged / 1 maxit / 2
 * preconditioner output not finite / 3 stagnation / 4 breakdown; iter in half
 * steps; resvec the absolute residual norms (initial, then one per half
 * step). */
int marie_bicgstab(marie_plan* plan, marie_op_fn A, void* A_ctx, const double* b, int64_t n,
                   double tol, int maxit, marie_op_fn M1, void* M1_ctx, marie_op_fn M2,
                   void* M2_ctx, const double* x0, double* x, int* flag, double* relres,
                   double* iter, double* resvec, int64_t resvec_cap, int64_t* resvec_len);

/* Replaces JVIE_Solver(Einc, e_r, r, freq, fN, tol, form, solver, precond,
 * max_it, inner_it, outer_it, ritz, gpu_flag) (src_vie/src_solver/
 * JVIE_Solver.m:1-521) with the plan's operator.  Einc: L x M x N x 3, e_r:
 * L x M x N (complex), dx the voxel edge (r enters only through dx).
 * Arguments are clamped as JVIE_Solver.m:71-122 does: tol outside
 * [1e-15, 1) -> 1e-3; form 1 or 2; solver 'G' (pgmres with restart
 * inner_it and outer_it cycles), 'D' (pgmresDR, deflating ritz harmonic Ritz
 * vectors) or anything else 'B' (bicgstab with max_it iterations); precond 0,
 * 'L' or 'R' (bicgstab takes either as its M1).  With a MARIE_MIXED plan the
 * circulant part of every Krylov matvec runs in FP32 inside FP64 iterations,
 * refined by FP64 true residuals until relres <= tol.  Je: L x M x N x 3.
 * iter: 2 doubles, {inner, outer} for 'G' and 'D', {iterations, 0} for 'B'
 * (half steps count 0.5).  resvec as the solver returns it: relative for 'G'
 * and 'D', absolute for 'B'. */
int marie_jvie_solve(marie_plan* plan, const double* Einc, const double* e_r, double dx,
                     double freq, double tol, int form, char solver, char precond, int max_it,
                     int inner_it, int outer_it, int ritz, double* Je, int* flag, double* relres,
                     double* iter, double* resvec, int64_t resvec_cap, int64_t* resvec_len,
                     double* solvert);

/* Several bodies of uneven grid size (one plan each), each with nexc[b]
 * excitations, solved concurrently.  On MARIE_MIXED plans of one device the
 * refinements of all bodies are branches of ONE graph launch (each body's
 * set-up, right-hand sides and results on its plan's stream); otherwise every
 * body's batch runs on its plan's stream from its own host thread.  Outputs
 * are concatenated over bodies (flag, relres: sum(nexc); iter: 2 per
 * excitation).  The reference solves one body at a time. */
int marie_jvie_solve_bodies(int nbody, marie_plan* const* plans, const double* const* Einc,
                            const int64_t* nexc, const double* const* e_r, const double* dx,
                            double freq, int form, char precond, double tol, int inner_it,
                            int outer_it, double* const* Je, int* flag, double* relres, int* iter,
                            double* solvert);

/* Adjoint gradient of a body-field objective with respect to the per-voxel
 * eps_r and sigma (no counterpart in the reference, which has no derivatives;
 * it reuses the J-VIE operator: K^T of the E-field system is the reference's
 * form-1 operator).  objective 0: F = sum 0.5 sigma |E|^2 (absorbed power);
 * 1: F = sum |E - E_target|^2 (E_target: L x M x N x 3).  Sums over the
 * non-air voxels.  Outputs F, dF_deps and dF_dsigma (L x M x N, zero in air),
 * flags {forward, adjoint} and iteration counts {forward, adjoint}. */
int marie_jvie_adjoint_grad(marie_plan* plan, const double* Einc, const double* e_r, double dx,
                            double freq, int objective, const double* E_target, double tol,
                            int inner_it, int outer_it, double* F, double* dF_deps,
                            double* dF_dsigma, int* flags, int* iters);

/* Replaces jvie2solver(Vrhs, fVIE, fVIEGPU, tol, Vini)
 * (src_vie/src_solver/jvie2solver.m:1), the inner J-VIE solve that
 * fVIEsolver_Assembly.m:196 hands to the coil solvers: BiCGSTAB (MATLAB
 * semantics, max_it iterations, no preconditioner, x0 = Vini or zero) on the
 * operator mv_AN(J, fN, Mr, Mc, Gram, 'notransp', idx) of the plan.  An
 * all-zero Vrhs is returned as the solution.  idx: 1-based DOF indices into
 * 3LMN (n_idx of them); Mr, Mc: L x M x N complex; Vrhs, Vini, Vsol: n_idx
 * complex, host or device.  A MARIE_MIXED plan refines FP32-matvec solves
 * with FP64 residuals.  flag / relres / iter (half steps) as bicgstab. */
int marie_jvie2solver(marie_plan* plan, const int64_t* idx, int64_t n_idx, const double* Mr, const double* Mc,
                      double Gram, const double* Vrhs, double tol, int max_it, const double* Vini, double* Vsol,
                      int* flag, double* relres, double* iter, double* solvert);

/* JVIE_Solver for nexc excitations of one body solved together: Einc and Je
 * are nexc consecutive L x M x N x 3 arrays; the solves advance in lockstep,
 * one batched matvec per GMRES step for each of two groups of excitations (see
 * marie_plan_set_batch_groups).  On a MARIE_MIXED plan the whole refinement is
 * one graph launch (marie_plan_set_graph_refinement).  Per excitation:
 * flag[e], relres[e], iter[2e..2e+1].  The reference solves excitations one at
 * a time (JVIE_Solver.m is called per port/excitation). */
int marie_jvie_solve_batch(marie_plan* plan, const double* Einc, int64_t nexc, const double* e_r,
                           double dx, double freq, int form, char precond, double tol, int inner_it,
                           int outer_it, double* Je, int* flag, double* relres, int* iter,
                           double* solvert);

/* Replaces H_field_Kop(J, fK, Gram, Hinc, GPU_flag) (src_vie/src_fields/src_op/
 * H_field_Kop.m:46-77): Htot = Hinc + mv_K(J) / Gram with the plan's K
 * operator.  J, Hinc (may be NULL), Htot: L x M x N x 3 complex. */
int marie_h_field_kop(marie_plan* plan, const double* J, double Gram, const double* Hinc,
                      double* Htot, int precision);

/* Replaces Scat_Solver(Einc, Hinc, freq, r, epsilon_r, sigma_e, rho, tol, fN, fK,
 * form, solver, precond, max_it, inner_it, outer_it, ritz, gpu_flag)
 * (src_vie/src_solver/Scat_Solver.m:1-241) on the plan: e_r = eps_r -
 * j sigma/(eps0 omega), the JVIE_Solver current Jout, SAR Sout = |J|^2 /
 * (2 sigma rho) (0 where |2 sigma rho| <= 1e-10), the total field Eout
 * (E_field_Nop), Bout = mu0 H_field_Kop(Jout, fK, Gram, Hinc), Gsar = sum Sout
 * Gram and Pabs = 0.5 Re sum Eout . conj(Jout) Gram.  The plan's N and K
 * operators are assembled first when it holds none (Scat_Solver.m:155-160).
 * eps_r, sigma_e, rho: L x M x N real; Einc, Hinc (may be NULL), Jout, Eout,
 * Bout: L x M x N x 3 complex; Sout: L x M x N real; NULL outputs are skipped
 * (Jout is required). */
int marie_scat_solver(marie_plan* plan, const double* Einc, const double* Hinc, double dx,
                      double freq, const double* eps_r, const double* sigma_e, const double* rho,
                      double tol, int form, char solver, char precond, int max_it, int inner_it,
                      int outer_it, int ritz, double* Jout, double* Sout, double* Eout, double* Bout,
                      double* Gsar, double* Pabs);

/* Replaces E_field_Nop(J, fN, Gram, freq, Einc) (src_vie/src_fields/src_op/
 * E_field_Nop.m:59-84): Etot = Einc + (N J - Gram J)/(Gram*j*omega*eps0).
 * J, Einc (may be NULL), Etot: L x M x N x 3 complex. */
int marie_e_field_nop(marie_plan* plan, const double* J, double Gram, double freq,
                      const double* Einc, double* Etot, int precision);

/* Incident fields on the grid (L x M x N x 3 complex):
 * PlaneWave_Excitation.m:39-95 (voxel-averaged, k = wavevector, Eo = polarisation)
 * and Dipole_Excitation.m / E_field_DGF.m:36-99 (point-sampled electric dipoles,
 * ndip dipoles with moments Jd[ndip][3] complex and positions pos[ndip][3]). */
int marie_plane_wave(const double* r, int64_t L, int64_t M, int64_t N, const double* k,
                     const double* Eo, double* E);
int marie_dipole_field(const double* r, int64_t L, int64_t M, int64_t N, double ko,
                       const double* Jd, const double* pos, int64_t ndip, double* E);

/* Comparison build (no counterpart in the reference): the FP32 'notransp'
 * mv_AN through cuFFT (zero-padded arrays, batched 3-D transforms, full
 * operator), the sequence of mv_AN.m:101-131 on a gpuArray.  *ms returns the
 * device time of the matvec proper (padding to epilogue).  Keeps its cuFFT plan
 * and buffers with the plan after the first call. */
int marie_mv_AN_cufft(marie_plan* plan, const double* JIn0, const double* Mr, const double* Mc,
                      double Gram, const int64_t* idx, int64_t n_idx, double* JOut, float* ms);

/* Instrumentation (no counterpart in the reference, which times with tic/toc):
 * number of kernels this library has launched since load, and per-pass device
 * times of the matvec.  marie_plan_profile(plan, enable, pass_ms, count)
 * returns the mean milliseconds of the five matvec passes (x forward, y
 * forward, z multiply, y inverse, x inverse) over the matvecs run since the
 * previous call, then resets and switches recording on or off. */
int64_t marie_launch_count(void);
/* Number of device-driven GMRES calls (the solvers' restart cycles) whose
 * cycles after the first ran as one graph launch: a conditional WHILE node
 * repeating one cycle and its device-side close (no counterpart in the
 * reference; a diagnostic like marie_launch_count). */
int64_t marie_graph_loops(void);
/* Per-call device buffers come from a library-owned memory pool per device
 * that keeps freed blocks for the next call (no reference counterpart).  This
 * returns the cached blocks to the device (after synchronising it); plans and
 * their operators are unaffected. */
int marie_release_cached_memory(void);
/* Schedule autotuner (no counterpart in the reference): times the plan's FP32
 * matvec for every candidate schedule (fuse: fused x+y cluster passes or the
 * five-pass form; fvar: default or narrow radix schedule of the fused x/y
 * transforms, or clusters of half the size; zvar: z pass with the default schedule, the narrow radix
 * schedule, or 4 instead of 8 columns per CTA), keeps the fastest on the plan
 * and returns it in *fuse / *fvar / *zvar.  ms receives {fuse, fvar, zvar,
 * milliseconds} per candidate (up to cap candidates, *count written).  A plan
 * without an FP32 operator is left as it is (*count = 0). */
int marie_plan_autotune(marie_plan* plan, int* fuse, int* fvar, int* zvar, double* ms, int64_t cap,
                        int64_t* count);
/* Pin a schedule as marie_plan_autotune would choose it. */
int marie_plan_set_schedule(marie_plan* plan, int fuse, int fvar, int zvar);
/* Krylov basis precision of the inner solves of a MARIE_MIXED plan's GMRES
 * refinement (no counterpart in the reference): MARIE_FP64 (the default: the
 * Arnoldi orthogonalisation in FP64 around the FP32 matvec) or MARIE_FP32 (an
 * opt-in: FP32 basis, dots and updates with FP64 reductions across threads;
 * FP64 Hessenberg and rotations).  The outer residuals and the returned
 * solution are FP64 either way. */
int marie_plan_set_inner_precision(marie_plan* plan, int precision);
/* Restart length of those inner GMRES solves (no counterpart in the
 * reference): 0 (the default) uses 20 (at most the caller's inner_it) with the
 * FP64 basis, whose FP64 Gram-Schmidt makes shorter cycles faster, and the
 * caller's inner_it with the FP32 basis; 1..127 overrides it for the inner
 * solves only.  Plain FP64 / FP32 solves and the outer semantics (restart of
 * the caller, tolerance on the FP64 true residual) are unaffected. */
int marie_plan_set_inner_restart(marie_plan* plan, int restart);
/* Batched GMRES schedule (no counterpart in the reference): 2 (the default)
 * splits the excitations of a batch into two groups on two streams whose
 * matvecs alternate, so that one group's FP64 Gram-Schmidt can run beside the
 * other group's FP32 matvec; 1 steps all excitations together.  Per system the
 * arithmetic is the same either way: the results are identical. */
int marie_plan_set_batch_groups(marie_plan* plan, int groups);
/* Control of the device-driven loops (no counterpart in the reference): 1
 * (the default) runs a MARIE_MIXED plan's GMRES solve -- every refinement
 * step with its inner restart cycles, FP64 residuals and tolerance updates --
 * as one launch of a CUDA graph with nested conditional WHILE nodes, the
 * device deciding every step, and the restart cycles of other GMRES solves in
 * one conditional-graph launch; 0 drives the refinement steps and the restart
 * cycles from the host, one plain CUDA graph per cycle (the form whose kernels
 * a profiler that replays kernels, such as ncu, can see: it does not profile
 * kernels inside graphs with conditional nodes).  The arithmetic and the
 * results are the same. */
int marie_plan_set_graph_refinement(marie_plan* plan, int on);
/* Host-side fault injection for tests (no reference counterpart): the nth
 * device allocation from now on fails with MARIE_ENOMEM (0 switches it off). */
void marie_inject_alloc_failure(int64_t nth);
/* Test of the bounded waits (no reference counterpart): the next n z passes
 * that load their operator tile by bulk copy arm its barrier for 16 bytes more
 * than the copy delivers and wait 5 ms instead of 2 s; the pass then finishes
 * with a wrong product and the entry point returns MARIE_ETIMEOUT (the plan
 * stays usable).  Nothing faults or hangs: the copy itself completes. */
void marie_inject_tile_timeout(int64_t n);
int marie_plan_profile(marie_plan* plan, int enable, double* pass_ms, int64_t* count);

#ifdef __cplusplus
}
#endif
#endif /* MARIE_VIE_H */
