// JVIE_Solver (src_vie/src_solver/JVIE_Solver.m:1-521) on the device, for one
// excitation (solvers 'G' pgmres, 'D' pgmresDR, 'B' bicgstab) or a batch of
// excitations of one body (lockstep pgmres):
//   set-up (JVIE_Solver.m:131-156, 242-244): non-air voxel compaction, the
//   local DOF order [idxS; V+idxS; 2V+idxS], the right-hand sides
//   Gram*j*omega*eps0*Mc*Einc, the form-2 scaling, the preconditioner
//   coefficients (1/Mr, 1/Mr - 1), then pgmres (restart inner_it, outer_it
//   cycles) and the scatter Je(idxS3) = x (:513-514).
// Arithmetic: MARIE_FP64 plans solve with the FP64 matvec (the reference
// arithmetic); MARIE_MIXED plans run GMRES-IR: the inner pgmres uses the FP32
// circulant matvec (Krylov basis, Arnoldi, Givens and the diagonal Gram*Mr
// term in FP64) and the outer loop refines with FP64 true residuals until
// ||b - A x|| / ||b|| <= tol.  The single-excitation solvers 'B' and 'D' refine
// the same way around an FP32-matvec bicgstab / pgmresDR.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <string>
#include <thread>
#include <vector>

#include "plan.h"

namespace marie {

// Restart length of the inner GMRES of mixed-precision refinement with an FP64
// Krylov basis (when the plan sets none).  Its Gram-Schmidt costs ~0.016 ms
// per basis vector per step at 128^3 on the FP64 pipe, so shorter cycles win
// although they take more matvecs: measured on the 128^3 phantom, restart
// 12 / 20 / 30 / 50 gave 224 / 224 / 241 / 262 ms per solve (303 / 273 / 261 /
// 236 matvecs).  With the FP32 basis the time is flat in the restart and the
// caller's inner_it is kept.
constexpr int kInnerRestart64 = 20;

// EMconstants.m:13-20
static constexpr double MU0 = 4e-7 * M_PI;
static constexpr double C0 = 299792458.0;
static inline double eps0() { return 1.0 / (C0 * C0 * MU0); }

static inline int grid_n(long long n) { return grid_stride_blocks(n, 8); }

// ---------------------------------------------------------------------------
// non-air voxel compaction: idxS = find(abs(Mc(:)) > 1e-12), in order
// ---------------------------------------------------------------------------
static constexpr int CMP_BLOCKS = 1024;

__device__ __forceinline__ bool non_air(const double2* er, long long v) {
  const double2 e = er[v];
  return hypot(e.x - 1.0, e.y) > 1e-12;
}

__global__ void k_count_nonair(const double2* __restrict__ er, long long V, int* __restrict__ counts) {
  const long long chunk = (V + gridDim.x - 1) / gridDim.x;
  const long long i0 = blockIdx.x * chunk, i1 = i0 + chunk < V ? i0 + chunk : V;
  int c = 0;
  for (long long i = i0 + threadIdx.x; i < i1; i += blockDim.x) c += non_air(er, i) ? 1 : 0;
  __shared__ int s[32];
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s[w];
    counts[blockIdx.x] = t;
  }
}

// writes idxS (0-based voxel ids) in increasing order; offsets = exclusive scan of counts
__global__ void k_write_nonair(const double2* __restrict__ er, long long V, const int* __restrict__ offsets,
                               int* __restrict__ idxS) {
  const long long chunk = (V + gridDim.x - 1) / gridDim.x;
  const long long i0 = blockIdx.x * chunk, i1 = i0 + chunk < V ? i0 + chunk : V;
  __shared__ int wsum[32];
  __shared__ int base;
  if (threadIdx.x == 0) base = offsets[blockIdx.x];
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (long long s0 = i0; s0 < i1; s0 += blockDim.x) {
    const long long i = s0 + threadIdx.x;
    const bool f = (i < i1) && non_air(er, i);
    const unsigned bal = __ballot_sync(0xffffffffu, f);
    const int before = __popc(bal & ((1u << lane) - 1u));
    if (lane == 0) wsum[wid] = __popc(bal);
    __syncthreads();
    int woff = 0, tot = 0;
    for (int w = 0; w < nw; ++w) {
      if (w < wid) woff += wsum[w];
      tot += wsum[w];
    }
    if (f) idxS[base + woff + before] = (int)i;
    __syncthreads();
    if (threadIdx.x == 0) base += tot;
    __syncthreads();
  }
}

// Per-DOF set-up for nS non-air voxels (DOF k = c*nS + s):
//   idx3[k] = c*V + idxS[s] + 1                       (JVIE_Solver.m:148)
//   f[k]    = Gram * j*omega*eps0 * Mc (/ Mr, form 2)  (rhs = f .* Einc, :151-156, :243)
//   a = Gram*Mr, b = Mc (form 2: Mc/Mr and Mr = 1)      (:242-244)
//   pa = Gram/Mr, pb = 1/Mr - 1                         (preconditioner, :276-278)
__global__ void k_jvie_coef(const int* __restrict__ idxS, long long nS, long long V, const double2* __restrict__ er,
                            double Gram, double omega_eps0, int form, int64_t* __restrict__ idx3,
                            double2* __restrict__ f, double2* __restrict__ a, double2* __restrict__ b,
                            double2* __restrict__ pa, double2* __restrict__ pb) {
  const long long n = 3 * nS;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const long long c = k / nS, s = k - c * nS;
    const long long v = idxS[s];
    idx3[k] = c * V + v + 1;
    double2 mr = er[v];
    double2 mc = mk<double2>(mr.x - 1.0, mr.y);
    double2 fk = mk<double2>(-Gram * omega_eps0 * mc.y, Gram * omega_eps0 * mc.x);  // Gram*j*omega*eps0*Mc
    if (form != 1) {
      const double den = mr.x * mr.x + mr.y * mr.y;
      const double2 inv_mr = mk<double2>(mr.x / den, -mr.y / den);
      mc = cmul(mc, inv_mr);
      fk = cmul(fk, inv_mr);
      mr = mk<double2>(1.0, 0.0);
    }
    f[k] = fk;
    a[k] = mk<double2>(Gram * mr.x, Gram * mr.y);
    b[k] = mc;
    const double den = mr.x * mr.x + mr.y * mr.y;
    const double2 imr = mk<double2>(mr.x / den, -mr.y / den);
    pa[k] = mk<double2>(Gram * imr.x, Gram * imr.y);
    pb[k] = mk<double2>(imr.x - 1.0, imr.y);
  }
}

// rhs_e[k] = f[k] * Einc_e[idx3[k]-1] for every excitation e
__global__ void k_jvie_rhs(const double2* __restrict__ f, const int64_t* __restrict__ idx3, long long n,
                           const double2* __restrict__ E, long long es, double2* __restrict__ rhs) {
  const int e = blockIdx.y;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    rhs[e * n + k] = cmul(f[k], E[e * es + idx3[k] - 1]);
}

__global__ void k_scatter_dofs(const double2* __restrict__ x, const int64_t* __restrict__ idx3, long long n,
                               double2* __restrict__ out, long long os) {
  const int e = blockIdx.y;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    out[e * os + idx3[k] - 1] = x[e * n + k];
}

// y_s = a .* x_s for systems with stop[s] >= step
__global__ void k_diag_b(const double2* __restrict__ a, const double2* __restrict__ x, long long xs,
                         double2* __restrict__ y, long long ys, long long n, const int* __restrict__ stop, int step) {
  const int s = blockIdx.y;
  if (stop && stop[s] < step) return;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    y[s * ys + k] = cmul(a[k], x[s * xs + k]);
}

__global__ void k_diag_b32(const float2* __restrict__ a, const float2* __restrict__ x, long long xs,
                           float2* __restrict__ y, long long ys, long long n, const int* __restrict__ stop, int step) {
  const int s = blockIdx.y;
  if (stop && stop[s] < step) return;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    y[s * ys + k] = cmul(a[k], x[s * xs + k]);
}

// FP32 copies of the four per-DOF coefficient arrays
__global__ void k_coef_f32(const double2* __restrict__ a, const double2* __restrict__ b,
                           const double2* __restrict__ pa, const double2* __restrict__ pb, long long n,
                           float2* __restrict__ af, float2* __restrict__ bf, float2* __restrict__ paf,
                           float2* __restrict__ pbf) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    af[k] = cvt<float2>(a[k]);
    bf[k] = cvt<float2>(b[k]);
    paf[k] = cvt<float2>(pa[k]);
    pbf[k] = cvt<float2>(pb[k]);
  }
}

__global__ void k_any_nonzero(const double2* __restrict__ b, long long n, int* __restrict__ nonzero) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    if (b[k].x != 0.0 || b[k].y != 0.0) *nonzero = 1;
}

// y_s = b_s - y_s, x_s += d_s   (for systems with flag[s])
__global__ void k_sub_b(const double2* __restrict__ b, double2* __restrict__ y, long long n,
                        const int* __restrict__ flag) {
  const int s = blockIdx.y;
  if (!flag[s]) return;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    y[s * n + k] = csub(b[s * n + k], y[s * n + k]);
}
__global__ void k_add_b(const double2* __restrict__ d, double2* __restrict__ x, long long n,
                        const int* __restrict__ flag) {
  const int s = blockIdx.y;
  if (!flag[s]) return;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    x[s * n + k] = cadd(x[s * n + k], d[s * n + k]);
}

struct JvieState {
  long long nS = 0, n = 0;
  DBuf idxS, idx3, inv, f, a, b, pa, pb;
  DBuf af, bf, paf, pbf;  // FP32 copies of a, b, pa, pb (plans with an FP32 operator)
};

static int jvie_setup(marie_plan* p, const double2* er, double dx, double freq, int form, JvieState& S) {
  cudaStream_t st = p->stream;
  const long long V = p->d.V;
  DBuf counts;
  MARIE_TRY(counts.alloc(CMP_BLOCKS * sizeof(int), st));
  k_count_nonair<<<CMP_BLOCKS, 256, 0, st>>>(er, V, counts.as<int>());
  count_launch();
  std::vector<int> hc(CMP_BLOCKS);
  MARIE_CUDA_TRY(cudaMemcpyAsync(hc.data(), counts.p, CMP_BLOCKS * sizeof(int), cudaMemcpyDeviceToHost, st));
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  long long tot = 0;
  for (int i = 0; i < CMP_BLOCKS; ++i) {
    const int c = hc[i];
    hc[i] = (int)tot;
    tot += c;
  }
  S.nS = tot;
  S.n = 3 * tot;
  if (tot == 0) return MARIE_OK;
  MARIE_CUDA_TRY(cudaMemcpyAsync(counts.p, hc.data(), CMP_BLOCKS * sizeof(int), cudaMemcpyHostToDevice, st));
  MARIE_TRY(S.idxS.alloc(tot * sizeof(int), st));
  k_write_nonair<<<CMP_BLOCKS, 256, 0, st>>>(er, V, counts.as<int>(), S.idxS.as<int>());
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  const long long n = S.n;
  MARIE_TRY(S.idx3.alloc(n * sizeof(int64_t), st));
  MARIE_TRY(S.f.alloc(n * sizeof(double2), st));
  MARIE_TRY(S.a.alloc(n * sizeof(double2), st));
  MARIE_TRY(S.b.alloc(n * sizeof(double2), st));
  MARIE_TRY(S.pa.alloc(n * sizeof(double2), st));
  MARIE_TRY(S.pb.alloc(n * sizeof(double2), st));
  MARIE_TRY(S.inv.alloc(3 * V * sizeof(int), st));
  const double Gram = dx * dx * dx;
  const double omega = 2.0 * M_PI * freq;
  k_jvie_coef<<<grid_n(n), 256, 0, st>>>(S.idxS.as<int>(), tot, V, er, Gram, omega * eps0(), form,
                                         S.idx3.as<int64_t>(), S.f.as<double2>(), S.a.as<double2>(),
                                         S.b.as<double2>(), S.pa.as<double2>(), S.pb.as<double2>());
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  if (p->fN32) {
    MARIE_TRY(S.af.alloc(n * sizeof(float2), st));
    MARIE_TRY(S.bf.alloc(n * sizeof(float2), st));
    MARIE_TRY(S.paf.alloc(n * sizeof(float2), st));
    MARIE_TRY(S.pbf.alloc(n * sizeof(float2), st));
    k_coef_f32<<<grid_n(n), 256, 0, st>>>(S.a.as<double2>(), S.b.as<double2>(), S.pa.as<double2>(),
                                          S.pb.as<double2>(), n, S.af.as<float2>(), S.bf.as<float2>(),
                                          S.paf.as<float2>(), S.pbf.as<float2>());
    count_launch();
    MARIE_CUDA_TRY(cudaGetLastError());
  }
  MARIE_TRY(build_inverse_index(p, S.idx3.as<int64_t>(), n, S.inv.as<int>()));
  return MARIE_OK;
}

static int any_nonzero(marie_plan* p, const double2* b, long long n, bool* nz) {
  DBuf f;
  MARIE_TRY(f.alloc(sizeof(int), p->stream));
  MARIE_CUDA_TRY(cudaMemsetAsync(f.p, 0, sizeof(int), p->stream));
  k_any_nonzero<<<grid_n(n), 256, 0, p->stream>>>(b, n, f.as<int>());
  count_launch();
  int h = 0;
  MARIE_CUDA_TRY(cudaMemcpyAsync(&h, f.p, sizeof(int), cudaMemcpyDeviceToHost, p->stream));
  MARIE_CUDA_TRY(cudaStreamSynchronize(p->stream));
  *nz = (h != 0);
  return MARIE_OK;
}

// mv_AN on the solver's DOFs for a batch of systems, coefficients (a, b).  A
// b that is identically zero leaves only the diagonal Gram*Mr product (the
// circulant term is multiplied by zero in mv_AN.m:127-131), so no FFT runs.
static BatchOp make_bop(marie_plan* p, int prec, const JvieState& S, const double2* a, const double2* b,
                        bool diag_only, const float2* af = nullptr, const float2* bf = nullptr) {
  const long long n = S.n;
  const int* inv = S.inv.as<int>();
  BatchOp op;
  if (prec == MARIE_FP32 && af && bf) {
    op.apply32 = [p, n, inv, af, bf, diag_only](const float2* in, long long is, float2* out, long long os, int ns,
                                                const int* stop, int step) -> int {
      if (diag_only) {
        k_diag_b32<<<dim3(grid_n(n), ns), 256, 0, p->stream>>>(af, in, is, out, os, n, stop, step);
        count_launch();
        MARIE_CUDA_TRY(cudaGetLastError());
        return MARIE_OK;
      }
      Prologue pro{nullptr, 0};
      Epilogue ep{};
      ep.af = af;
      ep.bf = bf;
      return run_matvec32(p, in, is, out, os, n, ns, inv, pro, ep, stop, step);
    };
  }
  // the FP32 operator on FP64 vectors (an FP64 Krylov basis) runs its
  // epilogue in FP32 with the coefficient copies af, bf, when given
  const float2* af_epi = prec == MARIE_FP32 ? af : nullptr;
  const float2* bf_epi = prec == MARIE_FP32 ? bf : nullptr;
  op.apply = [p, prec, n, inv, a, b, af_epi, bf_epi, diag_only](const double2* in, long long is, double2* out,
                                                                long long os, int ns, const int* stop,
                                                                int step) -> int {
    if (diag_only) {
      k_diag_b<<<dim3(grid_n(n), ns), 256, 0, p->stream>>>(a, in, is, out, os, n, stop, step);
      count_launch();
      MARIE_CUDA_TRY(cudaGetLastError());
      return MARIE_OK;
    }
    Prologue pro{nullptr, 0};
    Epilogue ep{};
    ep.a = a;
    ep.b = b;
    ep.af = af_epi;
    ep.bf = bf_epi;
    return run_matvec(p, prec, in, is, out, os, n, ns, inv, pro, ep, stop, step);
  };
  return op;
}

struct SolveOut {
  std::vector<GmresResult> r;
  BicgResult b;      // solver 'B'
  char solver = 'G';
};

// Krylov choice of JVIE_Solver.m:86-93, 300-499 for one excitation.
struct SolverArgs {
  char solver = 'G';  // 'G', 'D' or 'B'
  int max_it = 1000;  // bicgstab iterations
  int ritz = 5;       // pgmresDR deflation vectors
};

// Work of several bodies gathered for one graph launch: their refinement
// jobs, the steps that follow each job (run in order after the launch), and
// the buffers those steps need.
struct Deferred {
  std::vector<std::unique_ptr<RefineJob>> jobs;
  bool launched = false;  // the jobs' graph ran
  std::vector<std::function<int()>> after;
  std::vector<std::shared_ptr<void>> keep;
};

static int solve_systems(marie_plan* p, const JvieState& S, const double2* Bv, int S_exc, double2* X, char precond,
                         double tol, int inner_it, int outer_it, SolveOut& out, Deferred* dfr = nullptr);
static int solve_single(marie_plan* p, const JvieState& S, const double2* Bv, double2* X, char precond, double tol,
                        int inner_it, int outer_it, const SolverArgs& sa, SolveOut& out,
                        const double2* x0 = nullptr);

// Solves the S excitations E (3V x S, column stride es) of one body.
// With dfr, a mixed-precision 'G' solve leaves its refinement to dfr's
// shared graph launch and the DOF scatter to dfr's steps after it.
static int jvie_solve_core(marie_plan* p, const double2* E, long long es, int S_exc, const double2* er, double dx,
                           double freq, int form, char precond, double tol, int inner_it, int outer_it, double2* Je,
                           long long js, SolveOut& out, const SolverArgs& sa = SolverArgs(), Deferred* dfr = nullptr) {
  cudaStream_t st = p->stream;
  const long long V = p->d.V;
  auto Sp = std::make_shared<JvieState>();
  JvieState& S = *Sp;
  MARIE_TRY(jvie_setup(p, er, dx, freq, form, S));
  for (int e = 0; e < S_exc; ++e) MARIE_CUDA_TRY(cudaMemsetAsync(Je + e * js, 0, 3 * V * sizeof(double2), st));
  out.r.assign(S_exc, GmresResult());
  out.solver = sa.solver;
  if (S.n == 0) {
    for (auto& r : out.r) {
      r.flag = 0;
      r.relres = 0;
    }
    out.b.flag = 0;
    out.b.relres = 0;
    return MARIE_OK;
  }
  const long long n = S.n;
  auto rhs = std::make_shared<DBuf>(), x = std::make_shared<DBuf>();
  MARIE_TRY(rhs->alloc((size_t)S_exc * n * sizeof(double2), st));
  MARIE_TRY(x->alloc((size_t)S_exc * n * sizeof(double2), st));
  k_jvie_rhs<<<dim3(grid_n(n), S_exc), 256, 0, st>>>(S.f.as<double2>(), S.idx3.as<int64_t>(), n, E, es,
                                                      rhs->as<double2>());
  count_launch();
  if (sa.solver == 'G')
    MARIE_TRY(solve_systems(p, S, rhs->as<double2>(), S_exc, x->as<double2>(), precond, tol, inner_it, outer_it, out,
                            dfr));
  else
    MARIE_TRY(solve_single(p, S, rhs->as<double2>(), x->as<double2>(), precond, tol, inner_it, outer_it, sa, out));
  auto scatter = [p, Sp, x, n, S_exc, Je, js]() -> int {
    k_scatter_dofs<<<dim3(grid_n(n), S_exc), 256, 0, p->stream>>>(x->as<double2>(), Sp->idx3.as<int64_t>(), n, Je,
                                                                   js);
    count_launch();
    MARIE_CUDA_TRY(cudaGetLastError());
    return MARIE_OK;
  };
  if (!dfr) return scatter();
  dfr->keep.push_back(Sp);
  dfr->keep.push_back(rhs);
  dfr->keep.push_back(x);
  dfr->after.push_back(scatter);
  return MARIE_OK;
}

// Solves A2 x_e = B_e (form-2 J-VIE operator of the state S) for S_exc
// right-hand sides: FP64 pgmres, or GMRES-IR on a MARIE_MIXED plan.
static int solve_systems(marie_plan* p, const JvieState& S, const double2* Bv, int S_exc, double2* X, char precond,
                         double tol, int inner_it, int outer_it, SolveOut& out, Deferred* dfr) {
  cudaStream_t st = p->stream;
  const long long n = S.n;
  out.r.assign(S_exc, GmresResult());
  bool pb_nz = true;
  MARIE_TRY(any_nonzero(p, S.pb.as<double2>(), n, &pb_nz));
  const int prec_main = (p->precision == MARIE_FP32) ? MARIE_FP32 : MARIE_FP64;
  BatchOp A64 = make_bop(p, prec_main, S, S.a.as<double2>(), S.b.as<double2>(), false);
  BatchOp P64 = make_bop(p, prec_main, S, S.pa.as<double2>(), S.pb.as<double2>(), !pb_nz);
  const BatchOp* L1 = precond == 'L' ? &P64 : nullptr;
  const BatchOp* R1 = precond == 'R' ? &P64 : nullptr;
  if (p->precision != MARIE_MIXED) {
    MARIE_TRY(gmres_batch(p, A64, L1, R1, Bv, n, n, S_exc, inner_it, tol, outer_it, X, n, out.r, true, nullptr,
                          true));
  } else {
    // GMRES-IR: FP32-matvec pgmres on the residual, FP64 true residual and correction
    BatchOp A32 = make_bop(p, MARIE_FP32, S, S.a.as<double2>(), S.b.as<double2>(), false, S.af.as<float2>(),
                           S.bf.as<float2>());
    BatchOp P32 = make_bop(p, MARIE_FP32, S, S.pa.as<double2>(), S.pb.as<double2>(), !pb_nz, S.paf.as<float2>(),
                           S.pbf.as<float2>());
    const int max_refine = 20;
    // restart of the inner solves: the plan's setting, else with an FP64
    // basis kInnerRestart64 (its Gram-Schmidt is FP64-pipe-bound, so
    // shorter cycles win despite more matvecs), else the caller's inner_it
    const int m_in = p->inner_restart > 0 ? p->inner_restart
                     : p->inner_prec == MARIE_FP64 ? std::min(inner_it, kInnerRestart64)
                                                   : inner_it;
    const bool fp32b = p->inner_prec == MARIE_FP32;
    SolveOut* outp = &out;
    // The refinement driven from the host: the form selected by the plan, and
    // the fallback of the graph launch (it starts from x = 0 again).
    auto host_refine = [p, A32, P32, A64, precond, Bv, X, n, S_exc, tol, m_in, outer_it, max_refine, fp32b,
                        outp]() -> int {
      cudaStream_t st = p->stream;
      SolveOut& out = *outp;
      const BatchOp* L1m = precond == 'L' ? &P32 : nullptr;
      const BatchOp* R1m = precond == 'R' ? &P32 : nullptr;
      DBuf rb, db, flags, nrm;
      MARIE_TRY(rb.alloc((size_t)S_exc * n * sizeof(double2), st));
      MARIE_TRY(db.alloc((size_t)S_exc * n * sizeof(double2), st));
      MARIE_TRY(flags.alloc(S_exc * sizeof(int), st));
      MARIE_TRY(nrm.alloc((S_exc + batch_norm_scratch(S_exc)) * sizeof(double), st));
      double2* Rr = rb.as<double2>();
      double2* D = db.as<double2>();
      MARIE_CUDA_TRY(cudaMemsetAsync(X, 0, (size_t)S_exc * n * sizeof(double2), st));
      MARIE_CUDA_TRY(cudaMemcpyAsync(Rr, Bv, (size_t)S_exc * n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
      std::vector<double> bn(S_exc), rn(S_exc);
      // the norms of the graph-launched refinement (same kernels, same bits)
      double* nrm_d = nrm.as<double>();
      auto norms = [&](const double2* V, const int* mask, std::vector<double>& h) -> int {
        MARIE_TRY(batch_norms_dev(p, V, n, n, S_exc, mask, nrm_d + S_exc, nrm_d));
        MARIE_CUDA_TRY(cudaMemcpyAsync(h.data(), nrm_d, S_exc * sizeof(double), cudaMemcpyDeviceToHost, st));
        MARIE_CUDA_TRY(cudaStreamSynchronize(st));
        return MARIE_OK;
      };
      MARIE_TRY(norms(Bv, nullptr, bn));
      rn = bn;
      std::vector<int> act(S_exc), inner_total(S_exc, 0), last_p(S_exc, 0);
      for (int e = 0; e < S_exc; ++e) {
        out.r[e].relres = rn[e] / bn[e];
        out.r[e].resvec.push_back(out.r[e].relres);
      }
      std::vector<double> inner_tols(S_exc, 0.5), rn_new(S_exc);
      for (int it = 0; it < max_refine; ++it) {
        bool any = false;
        double inner_tol = 0.5;
        for (int e = 0; e < S_exc; ++e) {
          act[e] = out.r[e].relres > tol ? 1 : 0;
          if (act[e]) {
            any = true;
            // half of what is still missing, not below the FP32 floor; each
            // system of a batch stops its inner solve at its own tolerance
            inner_tols[e] = std::min(0.5, std::max(0.5 * tol * bn[e] / rn[e], 1e-5));
            inner_tol = std::min(inner_tol, inner_tols[e]);
          }
        }
        if (!any) break;
        MARIE_TRACE("refinement step");
        std::vector<GmresResult> ri;
        MARIE_TRY(gmres_batch(p, A32, L1m, R1m, Rr, n, n, S_exc, m_in, inner_tol, outer_it, D, n, ri, true, &act,
                              false, p->inner_prec == MARIE_FP32, &inner_tols));
        MARIE_CUDA_TRY(cudaMemcpyAsync(flags.p, act.data(), S_exc * sizeof(int), cudaMemcpyHostToDevice, st));
        k_add_b<<<dim3(grid_n(n), S_exc), 256, 0, st>>>(D, X, n, flags.as<int>());
        count_launch();
        // r = b - A64 x (FP64) for the systems that moved
        MARIE_TRY(A64.apply(X, n, Rr, n, S_exc, flags.as<int>(), 1));
        k_sub_b<<<dim3(grid_n(n), S_exc), 256, 0, st>>>(Bv, Rr, n, flags.as<int>());
        count_launch();
        MARIE_CUDA_TRY(cudaGetLastError());
        MARIE_TRY(norms(Rr, flags.as<int>(), rn_new));
        for (int e = 0; e < S_exc; ++e) {
          if (!act[e]) continue;
          for (size_t i = 1; i < ri[e].resvec.size(); ++i) out.r[e].resvec.push_back(ri[e].resvec[i] * rn[e] / bn[e]);
          inner_total[e] += ri[e].iter[1];
          last_p[e] = ri[e].iter[0];
          rn[e] = rn_new[e];
          out.r[e].relres = rn[e] / bn[e];
          out.r[e].resvec.push_back(out.r[e].relres);
        }
      }
      for (int e = 0; e < S_exc; ++e) {
        out.r[e].flag = out.r[e].relres <= tol ? 0 : 1;
        out.r[e].iter[0] = last_p[e];
        out.r[e].iter[1] = inner_total[e];
      }
      return MARIE_OK;
    };
    if (p->graph_refine) {
      // the whole refinement in one graph launch
      RefineOps ops;
      ops.add = [p, n, S_exc](const double2* D, double2* Xv, const int* fl) -> int {
        k_add_b<<<dim3(grid_n(n), S_exc), 256, 0, p->stream>>>(D, Xv, n, fl);
        count_launch();
        MARIE_CUDA_TRY(cudaGetLastError());
        return MARIE_OK;
      };
      ops.residual = [p, n, S_exc, A64, Bv](const double2* Xv, double2* R, const int* fl) -> int {
        MARIE_TRY(A64.apply(Xv, n, R, n, S_exc, fl, 1));
        k_sub_b<<<dim3(grid_n(n), S_exc), 256, 0, p->stream>>>(Bv, R, n, fl);
        count_launch();
        MARIE_CUDA_TRY(cudaGetLastError());
        return MARIE_OK;
      };
      auto job = std::make_unique<RefineJob>();
      bool ok = false;
      MARIE_TRY(job->prepare(p, A32, precond == 'L' ? &P32 : nullptr, precond == 'R' ? &P32 : nullptr, ops, Bv, n,
                             S_exc, m_in, tol, outer_it, max_refine, fp32b, X, &ok));
      if (ok && dfr) {
        // one launch with the other bodies' refinements; the results (or the
        // host-driven refinement, if that graph could not run) afterwards
        RefineJob* jp = job.get();
        dfr->jobs.push_back(std::move(job));
        dfr->after.push_back([dfr, jp, outp, host_refine]() -> int {
          return dfr->launched ? jp->finish(outp->r) : host_refine();
        });
        return MARIE_OK;
      }
      if (ok) {
        std::vector<RefineJob*> one{job.get()};
        bool ran = false;
        MARIE_TRY(launch_refine_jobs(one, p->stream, &ran));
        if (ran) return job->finish(out.r);
      }
    }
    return host_refine();
  }
  return MARIE_OK;
}

static DevOp single(const BatchOp& op, long long n) {
  return [op, n](const double2* x, double2* y) -> int { return op.apply(x, n, y, n, 1, nullptr, 0); };
}

// One excitation with bicgstab ('B', JVIE_Solver.m:451-499: the preconditioner,
// 'L' or 'R' alike, is bicgstab's M1) or pgmresDR ('D', :400-446).  MARIE_MIXED
// plans refine: FP32-matvec solves of A d = r, x += d, FP64 r = b - A x.
static int solve_single(marie_plan* p, const JvieState& S, const double2* Bv, double2* X, char precond, double tol,
                        int inner_it, int outer_it, const SolverArgs& sa, SolveOut& out, const double2* x0) {
  cudaStream_t st = p->stream;
  const long long n = S.n;
  bool pb_nz = true;
  MARIE_TRY(any_nonzero(p, S.pb.as<double2>(), n, &pb_nz));
  const int prec_main = (p->precision == MARIE_FP32) ? MARIE_FP32 : MARIE_FP64;
  const DevOp A64 = single(make_bop(p, prec_main, S, S.a.as<double2>(), S.b.as<double2>(), false), n);
  const DevOp P64 = single(make_bop(p, prec_main, S, S.pa.as<double2>(), S.pb.as<double2>(), !pb_nz), n);
  auto run = [&](const DevOp& A, const DevOp& P, const double2* b, double t, const double2* xs, double2* x,
                 BicgResult& rb, GmresResult& rg) -> int {
    if (sa.solver == 'B') return bicgstab(p, A, precond ? &P : nullptr, nullptr, b, n, t, sa.max_it, xs, x, rb);
    const DevOp* L1 = precond == 'L' ? &P : nullptr;
    const DevOp* R1 = precond == 'R' ? &P : nullptr;
    return gmres_dr(p, A, L1, nullptr, R1, nullptr, b, n, inner_it, t, outer_it, sa.ritz, xs, x, rg);
  };
  if (p->precision != MARIE_MIXED) {
    GmresResult rg;
    MARIE_TRY(run(A64, P64, Bv, tol, x0, X, out.b, rg));
    out.r[0] = rg;
    return MARIE_OK;
  }
  const DevOp A32 = single(make_bop(p, MARIE_FP32, S, S.a.as<double2>(), S.b.as<double2>(), false), n);
  const DevOp P32 = single(make_bop(p, MARIE_FP32, S, S.pa.as<double2>(), S.pb.as<double2>(), !pb_nz), n);
  DBuf rb, db, one;
  MARIE_TRY(rb.alloc((size_t)n * sizeof(double2), st));
  MARIE_TRY(db.alloc((size_t)n * sizeof(double2), st));
  MARIE_TRY(one.alloc(sizeof(int), st));
  const int on = 1;
  MARIE_CUDA_TRY(cudaMemcpyAsync(one.p, &on, sizeof(int), cudaMemcpyHostToDevice, st));
  double2* Rr = rb.as<double2>();
  double2* D = db.as<double2>();
  if (x0) {
    // start from x0: r = b - A x0 in FP64
    MARIE_CUDA_TRY(cudaMemcpyAsync(X, x0, (size_t)n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    MARIE_TRY(A64(X, Rr));
    k_sub_b<<<dim3(grid_n(n), 1), 256, 0, st>>>(Bv, Rr, n, one.as<int>());
    count_launch();
    MARIE_CUDA_TRY(cudaGetLastError());
  } else {
    MARIE_CUDA_TRY(cudaMemsetAsync(X, 0, (size_t)n * sizeof(double2), st));
    MARIE_CUDA_TRY(cudaMemcpyAsync(Rr, Bv, (size_t)n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
  }
  double bn = 0;
  MARIE_TRY(dev_norm2(p, Bv, n, &bn));
  double rn = bn;
  if (x0) MARIE_TRY(dev_norm2(p, Rr, n, &rn));
  BicgResult& B = out.b;
  GmresResult& G = out.r[0];
  B = BicgResult();
  G = GmresResult();
  B.resvec.push_back(rn);
  G.resvec.push_back(bn > 0 ? rn / bn : 0.0);
  double biter = 0;
  int inner_total = 0, last_p = 0, last_flag = 1;
  for (int it = 0; it < 20 && rn > tol * bn; ++it) {
    // half of what is still missing, not below the FP32 floor
    const double inner_tol = std::max(0.5 * tol * bn / rn, 1e-5);
    BicgResult ib;
    GmresResult ig;
    MARIE_TRY(run(A32, P32, Rr, inner_tol, nullptr, D, ib, ig));
    k_add_b<<<dim3(grid_n(n), 1), 256, 0, st>>>(D, X, n, one.as<int>());
    count_launch();
    MARIE_TRY(A64(X, Rr));
    k_sub_b<<<dim3(grid_n(n), 1), 256, 0, st>>>(Bv, Rr, n, one.as<int>());
    count_launch();
    MARIE_CUDA_TRY(cudaGetLastError());
    const double rprev = rn;
    MARIE_TRY(dev_norm2(p, Rr, n, &rn));
    if (sa.solver == 'B') {
      for (size_t i = 1; i < ib.resvec.size(); ++i) B.resvec.push_back(ib.resvec[i]);
      B.resvec.push_back(rn);
      biter += ib.iter;
      last_flag = ib.flag;
    } else {
      for (size_t i = 1; i < ig.resvec.size(); ++i) G.resvec.push_back(ig.resvec[i] * rprev / bn);
      G.resvec.push_back(rn / bn);
      inner_total += ig.iter[1];
      last_p = ig.iter[0];
    }
    if (!std::isfinite(rn)) return set_error(MARIE_EBREAKDOWN, "non-finite residual in the refinement");
  }
  const int fl = rn <= tol * bn ? 0 : (sa.solver == 'B' && last_flag > 1 ? last_flag : 1);
  B.flag = G.flag = fl;
  B.relres = G.relres = bn > 0 ? rn / bn : 0.0;
  B.iter = biter;
  G.iter[0] = last_p;
  G.iter[1] = inner_total;
  return MARIE_OK;
}

// adjoint-gradient kernels (adjoint.cu)
__global__ void k_adj_fields(const double2* __restrict__ J, const int64_t* __restrict__ idx3, long long n,
                             long long V, const double2* __restrict__ er, double omega_eps0, int objective,
                             const double2* __restrict__ Et, double2* __restrict__ E, double2* __restrict__ w,
                             double* __restrict__ Fpart);
__global__ void k_adj_grad(const double2* __restrict__ q, const double2* __restrict__ E, const int* __restrict__ idxS,
                           long long nS, const double2* __restrict__ er, double omega_eps0, int objective,
                           double* __restrict__ g_eps, double* __restrict__ g_sig);

// Forward solve, objective, adjoint solve with the same J-VIE operator, and
// the fused gradient (derivation in adjoint.cu).  g_eps, g_sig: L x M x N.
int jvie_adjoint_core(marie_plan* p, const double2* Einc, const double2* er, double dx, double freq, int objective,
                      const double2* Et, double tol, int inner_it, int outer_it, double* F, double* g_eps,
                      double* g_sig, int* flags, int* iters) {
  cudaStream_t st = p->stream;
  const long long V = p->d.V;
  JvieState S;
  MARIE_TRY(jvie_setup(p, er, dx, freq, 2, S));
  MARIE_CUDA_TRY(cudaMemsetAsync(g_eps, 0, V * sizeof(double), st));
  MARIE_CUDA_TRY(cudaMemsetAsync(g_sig, 0, V * sizeof(double), st));
  *F = 0;
  if (S.n == 0) return MARIE_OK;
  const long long n = S.n;
  const double omega_eps0 = 2.0 * M_PI * freq * eps0();
  DBuf rhs, J, E, w, lam, q, Fp;
  MARIE_TRY(rhs.alloc(n * sizeof(double2), st));
  MARIE_TRY(J.alloc(n * sizeof(double2), st));
  MARIE_TRY(E.alloc(n * sizeof(double2), st));
  MARIE_TRY(w.alloc(n * sizeof(double2), st));
  MARIE_TRY(lam.alloc(n * sizeof(double2), st));
  MARIE_TRY(q.alloc(n * sizeof(double2), st));
  const int nb = grid_n(n);
  MARIE_TRY(Fp.alloc(nb * sizeof(double), st));
  k_jvie_rhs<<<dim3(nb, 1), 256, 0, st>>>(S.f.as<double2>(), S.idx3.as<int64_t>(), n, Einc, 0, rhs.as<double2>());
  count_launch();
  SolveOut fwd, adj;
  MARIE_TRY(solve_systems(p, S, rhs.as<double2>(), 1, J.as<double2>(), 0, tol, inner_it, outer_it, fwd));
  k_adj_fields<<<nb, 256, 0, st>>>(J.as<double2>(), S.idx3.as<int64_t>(), n, V, er, omega_eps0, objective, Et,
                                   E.as<double2>(), w.as<double2>(), Fp.as<double>());
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  std::vector<double> hF(nb);
  MARIE_CUDA_TRY(cudaMemcpyAsync(hF.data(), Fp.p, nb * sizeof(double), cudaMemcpyDeviceToHost, st));
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  double Fs = 0;
  for (double v : hF) Fs += v;
  *F = Fs;
  // adjoint solve A lambda = w (rows divided by eps_c, like the forward form 2)
  MARIE_TRY(solve_systems(p, S, w.as<double2>(), 1, lam.as<double2>(), 0, tol, inner_it, outer_it, adj));
  // q = (Gram - N) lambda in FP64
  Prologue pro{nullptr, 0};
  Epilogue ep{};
  ep.a_s = mk<double2>(dx * dx * dx, 0.0);
  ep.b_s = mk<double2>(1.0, 0.0);
  const int prec = p->fN64 ? MARIE_FP64 : MARIE_FP32;
  MARIE_TRY(run_matvec(p, prec, lam.as<double2>(), q.as<double2>(), n, 1, S.inv.as<int>(), pro, ep));
  k_adj_grad<<<grid_n(S.nS), 256, 0, st>>>(q.as<double2>(), E.as<double2>(), S.idxS.as<int>(), S.nS, er, omega_eps0,
                                           objective, g_eps, g_sig);
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  if (flags) {
    flags[0] = fwd.r[0].flag;
    flags[1] = adj.r[0].flag;
  }
  if (iters) {
    iters[0] = (int)fwd.r[0].resvec.size() - 1;
    iters[1] = (int)adj.r[0].resvec.size() - 1;
  }
  return MARIE_OK;
}

static int clamp_args(double& tol, int& form, char& precond, int& inner_it, int& outer_it) {
  // JVIE_Solver.m:71-122 argument clamps
  if (tol < 1e-15 || tol >= 1) tol = 1e-3;
  if (form != 1) form = 2;
  if (precond != 'L' && precond != 'R') precond = 0;
  if (inner_it < 1) inner_it = 50;
  if (outer_it < 1) outer_it = 200;
  if (inner_it > 127) return set_error(MARIE_EINVAL, "inner_it (GMRES restart) above 127 is not built");
  return MARIE_OK;
}

// solver ('G', 'D', else 'B'), max_it (default 1000), ritz (default 5):
// JVIE_Solver.m:86-93, 99-101, 108-110
static void clamp_solver(SolverArgs& sa, int inner_it) {
  if (sa.solver != 'G' && sa.solver != 'D') sa.solver = 'B';
  if (sa.max_it < 1) sa.max_it = 1000;
  if (sa.ritz < 1) sa.ritz = 5;
  // pgmresDR.m:55-60
  if (sa.ritz > inner_it - 1) sa.ritz = inner_it - 1;
}

// Scat_Solver post-processing (Scat_Solver.m:177-229) in one pass over the
// voxels: SAR S = sum_c |J_c|^2 / (2 sigma rho) where |2 sigma rho| > 1e-10
// (zero elsewhere), and per-block partial sums of S and of Re(E . conj(J)).
__global__ void k_sar_power(const double2* __restrict__ J, const double2* __restrict__ E,
                            const double* __restrict__ sigma, const double* __restrict__ rho, long long V,
                            double* __restrict__ S, double* __restrict__ part) {
  double ssum = 0, psum = 0;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
    double jj = 0, ej = 0;
    for (int c = 0; c < 3; ++c) {
      const double2 j = J[c * V + v], e = E[c * V + v];
      jj = fma(j.x, j.x, fma(j.y, j.y, jj));
      ej = fma(e.x, j.x, fma(e.y, j.y, ej));  // Re(e conj(j))
    }
    const double denom = 2.0 * sigma[v] * rho[v];
    const double sv = fabs(denom) > 1e-10 ? jj / denom : 0.0;
    S[v] = sv;
    ssum += sv;
    psum += ej;
  }
  __shared__ double ws[2][32];
  for (int o = 16; o > 0; o >>= 1) {
    ssum += __shfl_xor_sync(0xffffffffu, ssum, o);
    psum += __shfl_xor_sync(0xffffffffu, psum, o);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    ws[0][wid] = ssum;
    ws[1][wid] = psum;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    double t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += ws[threadIdx.x][w];
    part[threadIdx.x * gridDim.x + blockIdx.x] = t;
  }
}

// e_r = eps_r - j sigma / (eps0 omega) (Scat_Solver.m:144)
__global__ void k_complex_permittivity(const double* __restrict__ eps_r, const double* __restrict__ sigma,
                                       double eps0_omega, long long V, double2* __restrict__ er) {
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x)
    er[v] = mk<double2>(eps_r[v], -sigma[v] / eps0_omega);
}

__global__ void k_scale_field(double2* __restrict__ x, double s, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    x[i] = mk<double2>(x[i].x * s, x[i].y * s);
}

}  // namespace marie

using namespace marie;


// The bodies of marie_jvie_solve_bodies with their refinements in ONE graph
// launch: each body's set-up, right-hand sides and refinement start run on
// its plan's stream; the refinement loops of all bodies are independent
// branches of one graph launched once; then each body's results, DOF scatter
// and host copies.
static int solve_bodies_one_launch(int nbody, marie_plan* const* plans, const double* const* Einc,
                                   const int64_t* nexc, const double* const* e_r, const double* dx, double freq,
                                   int form, char precond, double tol, int inner_it, int outer_it, double* const* Je,
                                   int* flag, double* relres, int* iter) {
  Deferred dfr;
  long long off = 0;
  for (int b = 0; b < nbody; ++b) {
    marie_plan* p = plans[b];
    auto fail = [&](int code) {
      const std::string m = marie_last_error();
      return set_error(code, "body %d: %s", b, m.c_str());
    };
    if (!Einc[b] || !e_r[b] || !Je[b] || nexc[b] < 1) return set_error(MARIE_EINVAL, "body %d: NULL argument", b);
    if (!p->has_op) return set_error(MARIE_ENOOP, "body %d: plan has no operator", b);
    if (!(dx[b] > 0) || !(freq > 0)) return set_error(MARIE_EINVAL, "body %d: dx and freq must be positive", b);
    double tb = tol;
    int fb = form, ib = inner_it, ob = outer_it;
    char pb = precond;
    int s = clamp_args(tb, fb, pb, ib, ob);
    if (s != MARIE_OK) return fail(s);
    cudaStream_t st = p->stream;
    const long long V = p->d.V;
    const size_t jbytes = (size_t)nexc[b] * 3 * V * sizeof(double2);
    auto tE = std::make_shared<DBuf>(), tER = std::make_shared<DBuf>(), tJe = std::make_shared<DBuf>();
    const void *E_d, *er_d;
    void* Je_d;
    if ((s = stage_in(Einc[b], jbytes, st, *tE, &E_d)) != MARIE_OK) return fail(s);
    if ((s = stage_in(e_r[b], V * sizeof(double2), st, *tER, &er_d)) != MARIE_OK) return fail(s);
    if ((s = stage_out(Je[b], jbytes, st, *tJe, &Je_d)) != MARIE_OK) return fail(s);
    auto pf = std::make_shared<HostPrefault>();
    pf->start(Je[b], jbytes);
    auto so = std::make_shared<SolveOut>();
    s = jvie_solve_core(p, (const double2*)E_d, 3 * V, (int)nexc[b], (const double2*)er_d, dx[b], freq, fb, pb, tb,
                        ib, ob, (double2*)Je_d, 3 * V, *so, SolverArgs(), &dfr);
    if (s != MARIE_OK) return fail(s);
    dfr.keep.push_back(tE);
    dfr.keep.push_back(tER);
    dfr.keep.push_back(tJe);
    dfr.keep.push_back(pf);
    dfr.keep.push_back(so);
    void* Jh = Je[b];
    const long long ne = nexc[b], o = off;
    dfr.after.push_back([p, pf, so, Jh, Je_d, jbytes, ne, o, flag, relres, iter]() -> int {
      pf->join();
      MARIE_TRY(finish_out(Jh, Je_d, jbytes, p->stream));
      MARIE_CUDA_TRY(cudaStreamSynchronize(p->stream));
      for (long long e = 0; e < ne; ++e) {
        if (flag) flag[o + e] = so->r[e].flag;
        if (relres) relres[o + e] = so->r[e].relres;
        if (iter) {
          iter[2 * (o + e)] = so->r[e].iter[0];
          iter[2 * (o + e) + 1] = so->r[e].iter[1];
        }
      }
      return check_kernel_status(p);
    });
    off += nexc[b];
  }
  if (!dfr.jobs.empty()) {
    std::vector<RefineJob*> jobs;
    for (auto& j : dfr.jobs) jobs.push_back(j.get());
    bool ran = false;
    MARIE_TRY(launch_refine_jobs(jobs, plans[0]->stream, &ran));
    dfr.launched = ran;
  }
  for (auto& step : dfr.after) MARIE_TRY(step());
  return MARIE_OK;
}

extern "C" {

int marie_scat_solver(marie_plan* p, const double* Einc, const double* Hinc, double dx, double freq,
                      const double* eps_r, const double* sigma_e, const double* rho, double tol, int form,
                      char solver, char precond, int max_it, int inner_it, int outer_it, int ritz, double* Jout,
                      double* Sout, double* Eout, double* Bout, double* Gsar, double* Pabs) {
  if (!p || !Einc || !eps_r || !sigma_e || !rho || !Jout) return set_error(MARIE_EINVAL, "NULL argument");
  if (!(dx > 0) || !(freq > 0)) return set_error(MARIE_EINVAL, "dx and freq must be positive");
  MARIE_TRACE("Scat_Solver");
  cudaStream_t st = p->stream;
  const long long V = p->d.V;
  const double Gram = dx * dx * dx;
  // Scat_Solver.m:155-160: the operators when the plan has none
  if (!p->has_op) MARIE_TRY(marie_plan_assemble(p, dx, freq, 'D', nullptr));
  if ((Bout || Hinc) && !p->has_opK) MARIE_TRY(marie_plan_assemble_k(p, dx, freq));
  DBuf tE, tH, teps, tsig, trho, tJ, tS, tEo, tB, er, part;
  const void *E_d, *H_d = nullptr, *eps_d, *sig_d, *rho_d;
  void *J_d, *S_d = nullptr, *Eo_d = nullptr, *B_d = nullptr;
  MARIE_TRY(stage_in(Einc, 3 * V * sizeof(double2), st, tE, &E_d));
  if (Hinc) MARIE_TRY(stage_in(Hinc, 3 * V * sizeof(double2), st, tH, &H_d));
  MARIE_TRY(stage_in(eps_r, V * sizeof(double), st, teps, &eps_d));
  MARIE_TRY(stage_in(sigma_e, V * sizeof(double), st, tsig, &sig_d));
  MARIE_TRY(stage_in(rho, V * sizeof(double), st, trho, &rho_d));
  MARIE_TRY(stage_out(Jout, 3 * V * sizeof(double2), st, tJ, &J_d));
  // SAR and the powers need E even when the caller does not ask for it
  MARIE_TRY(stage_out(Eout ? Eout : nullptr, 3 * V * sizeof(double2), st, tEo, &Eo_d));
  if (Sout) MARIE_TRY(stage_out(Sout, V * sizeof(double), st, tS, &S_d));
  if (Bout) MARIE_TRY(stage_out(Bout, 3 * V * sizeof(double2), st, tB, &B_d));
  HostPrefault pfJ, pfE, pfS, pfB;
  pfJ.start(Jout, 3 * V * sizeof(double2));
  if (Eout) pfE.start(Eout, 3 * V * sizeof(double2));
  if (Sout) pfS.start(Sout, V * sizeof(double));
  if (Bout) pfB.start(Bout, 3 * V * sizeof(double2));
  DBuf S_tmp;
  if (!S_d) {
    MARIE_TRY(S_tmp.alloc(V * sizeof(double), st));
    S_d = S_tmp.p;
  }
  MARIE_TRY(er.alloc(V * sizeof(double2), st));
  const double omega = 2.0 * M_PI * freq;
  k_complex_permittivity<<<grid_n(V), 256, 0, st>>>((const double*)eps_d, (const double*)sig_d, eps0() * omega, V,
                                                    er.as<double2>());
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  // the current (Scat_Solver.m:164)
  double iter[2], relres;
  int flag;
  MARIE_TRY(marie_jvie_solve(p, (const double*)E_d, (const double*)er.p, dx, freq, tol, form, solver, precond,
                             max_it, inner_it, outer_it, ritz, (double*)J_d, &flag, &relres, iter, nullptr, 0,
                             nullptr, nullptr));
  // total E (:181) and B = mu0 H (:186-187)
  const int prec = p->fN64 ? MARIE_FP64 : MARIE_FP32;
  MARIE_TRY(marie_e_field_nop(p, (const double*)J_d, Gram, freq, (const double*)E_d, (double*)Eo_d, prec));
  if (Bout) {
    const int precK = p->fK64 ? MARIE_FP64 : MARIE_FP32;
    MARIE_TRY(marie_h_field_kop(p, (const double*)J_d, Gram, (const double*)H_d, (double*)B_d, precK));
    k_scale_field<<<grid_n(3 * V), 256, 0, st>>>((double2*)B_d, 4.0 * M_PI * 1e-7, 3 * V);
    count_launch();
  }
  // SAR (:170-178), Pabs and Gsar (:190-194)
  const int G = 152 * 2;
  MARIE_TRY(part.alloc(2 * G * sizeof(double), st));
  k_sar_power<<<G, 256, 0, st>>>((const double2*)J_d, (const double2*)Eo_d, (const double*)sig_d,
                                 (const double*)rho_d, V, (double*)S_d, part.as<double>());
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  std::vector<double> hp(2 * G);
  MARIE_CUDA_TRY(cudaMemcpyAsync(hp.data(), part.p, 2 * G * sizeof(double), cudaMemcpyDeviceToHost, st));
  pfJ.join();
  pfE.join();
  pfS.join();
  pfB.join();
  MARIE_TRY(finish_out(Jout, J_d, 3 * V * sizeof(double2), st));
  if (Eout) MARIE_TRY(finish_out(Eout, Eo_d, 3 * V * sizeof(double2), st));
  if (Sout) MARIE_TRY(finish_out(Sout, S_d, V * sizeof(double), st));
  if (Bout) MARIE_TRY(finish_out(Bout, B_d, 3 * V * sizeof(double2), st));
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  double ssum = 0, psum = 0;
  for (int b = 0; b < G; ++b) {
    ssum += hp[b];
    psum += hp[G + b];
  }
  if (Gsar) *Gsar = ssum * Gram;
  if (Pabs) *Pabs = 0.5 * psum * Gram;
  return check_kernel_status(p);
}


int marie_jvie_solve(marie_plan* p, const double* Einc, const double* e_r, double dx, double freq, double tol,
                     int form, char solver, char precond, int max_it, int inner_it, int outer_it, int ritz,
                     double* Je, int* flag, double* relres, double* iter, double* resvec, int64_t resvec_cap,
                     int64_t* resvec_len, double* solvert) {
  if (!p || !Einc || !e_r || !Je) return set_error(MARIE_EINVAL, "NULL argument");
  if (!p->has_op) return set_error(MARIE_ENOOP, "plan has no operator");
  if (!(dx > 0) || !(freq > 0)) return set_error(MARIE_EINVAL, "dx and freq must be positive");
  MARIE_TRY(clamp_args(tol, form, precond, inner_it, outer_it));
  MARIE_TRACE("JVIE_Solver");
  SolverArgs sa;
  sa.solver = solver;
  sa.max_it = max_it;
  sa.ritz = ritz;
  clamp_solver(sa, inner_it);
  const auto t0 = std::chrono::steady_clock::now();
  cudaStream_t st = p->stream;
  const long long V = p->d.V;
  DBuf tE, tER, tJe;
  const void *E_d, *er_d;
  void* Je_d;
  MARIE_TRY(stage_in(Einc, 3 * V * sizeof(double2), st, tE, &E_d));
  MARIE_TRY(stage_in(e_r, V * sizeof(double2), st, tER, &er_d));
  MARIE_TRY(stage_out(Je, 3 * V * sizeof(double2), st, tJe, &Je_d));
  HostPrefault pf;
  pf.start(Je, 3 * V * sizeof(double2));
  SolveOut so;
  MARIE_TRY(jvie_solve_core(p, (const double2*)E_d, 3 * V, 1, (const double2*)er_d, dx, freq, form, precond, tol,
                            inner_it, outer_it, (double2*)Je_d, 3 * V, so, sa));
  pf.join();
  MARIE_TRY(finish_out(Je, Je_d, 3 * V * sizeof(double2), st));
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  const auto t1 = std::chrono::steady_clock::now();
  const bool bi = sa.solver == 'B';
  const GmresResult& R = so.r[0];
  const std::vector<double>& rv = bi ? so.b.resvec : R.resvec;
  if (flag) *flag = bi ? so.b.flag : R.flag;
  if (relres) *relres = bi ? so.b.relres : R.relres;
  if (iter) {
    iter[0] = bi ? so.b.iter : R.iter[0];
    iter[1] = bi ? 0.0 : R.iter[1];
  }
  if (resvec_len) *resvec_len = (int64_t)rv.size();
  if (resvec)
    for (int64_t i = 0; i < (int64_t)rv.size() && i < resvec_cap; ++i) resvec[i] = rv[i];
  if (solvert) *solvert = std::chrono::duration<double>(t1 - t0).count();
  return check_kernel_status(p);
}

int marie_jvie2solver(marie_plan* p, const int64_t* idx, int64_t n_idx, const double* Mr, const double* Mc,
                      double Gram, const double* Vrhs, double tol, int max_it, const double* Vini, double* Vsol,
                      int* flag, double* relres, double* iter, double* solvert) {
  if (!p || !idx || !Mr || !Mc || !Vrhs || !Vsol || n_idx < 1) return set_error(MARIE_EINVAL, "NULL argument");
  if (!p->has_op) return set_error(MARIE_ENOOP, "plan has no operator");
  if (!(tol > 0)) return set_error(MARIE_EINVAL, "tol must be positive");
  if (max_it < 1) return set_error(MARIE_EINVAL, "max_it must be >= 1");
  MARIE_TRACE("jvie2solver");
  const auto t0 = std::chrono::steady_clock::now();
  cudaStream_t st = p->stream;
  const long long V = p->d.V, n = n_idx;
  DBuf tidx, tMr, tMc, tb, tx0, tx;
  const void *idx_d, *Mr_d, *Mc_d, *b_d, *x0_d = nullptr;
  void* x_d;
  MARIE_TRY(stage_in(idx, n * sizeof(int64_t), st, tidx, &idx_d));
  MARIE_TRY(stage_in(Mr, V * sizeof(double2), st, tMr, &Mr_d));
  MARIE_TRY(stage_in(Mc, V * sizeof(double2), st, tMc, &Mc_d));
  MARIE_TRY(stage_in(Vrhs, n * sizeof(double2), st, tb, &b_d));
  if (Vini) MARIE_TRY(stage_in(Vini, n * sizeof(double2), st, tx0, &x0_d));
  MARIE_TRY(stage_out(Vsol, n * sizeof(double2), st, tx, &x_d));
  HostPrefault pf;
  pf.start(Vsol, n * sizeof(double2));
  if (flag) *flag = 0;
  if (relres) *relres = 0;
  if (iter) *iter = 0;
  // jvie2solver.m:35-38: an all-zero right-hand side is returned as the solution
  bool nz = true;
  MARIE_TRY(any_nonzero(p, (const double2*)b_d, n, &nz));
  if (!nz) {
    MARIE_CUDA_TRY(cudaMemcpyAsync(x_d, b_d, n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
  } else {
    // the mv_AN('notransp') operator on the DOFs idx (jvie2solver's fVIE): a = Gram Mr(idx), b = Mc(idx)
    JvieState S;
    S.n = n;
    MARIE_TRY(S.idx3.alloc(n * sizeof(int64_t), st));
    MARIE_CUDA_TRY(cudaMemcpyAsync(S.idx3.p, idx_d, n * sizeof(int64_t), cudaMemcpyDeviceToDevice, st));
    MARIE_TRY(S.a.alloc(n * sizeof(double2), st));
    MARIE_TRY(S.b.alloc(n * sizeof(double2), st));
    MARIE_TRY(S.pa.alloc(n * sizeof(double2), st));  // no preconditioner: pa, pb unused (pb = 0)
    MARIE_TRY(S.pb.alloc(n * sizeof(double2), st));
    MARIE_CUDA_TRY(cudaMemsetAsync(S.pa.p, 0, n * sizeof(double2), st));
    MARIE_CUDA_TRY(cudaMemsetAsync(S.pb.p, 0, n * sizeof(double2), st));
    MARIE_TRY(S.inv.alloc(3 * V * sizeof(int), st));
    MARIE_TRY(build_inverse_index(p, S.idx3.as<int64_t>(), n, S.inv.as<int>()));
    MARIE_TRY(build_coefficients(p, S.idx3.as<int64_t>(), n, (const double2*)Mr_d, (const double2*)Mc_d, Gram, 0,
                                 S.a.as<double2>(), S.b.as<double2>()));
    // bicgstab(fVIE, Vrhs, tol, max_it, [], [], Vini) (jvie2solver.m:54-77)
    SolverArgs sa;
    sa.solver = 'B';
    sa.max_it = max_it;
    SolveOut so;
    so.r.assign(1, GmresResult());
    MARIE_TRY(solve_single(p, S, (const double2*)b_d, (double2*)x_d, 0, tol, 50, 200, sa, so,
                           (const double2*)x0_d));
    if (flag) *flag = so.b.flag;
    if (relres) *relres = so.b.relres;
    if (iter) *iter = so.b.iter;
  }
  pf.join();
  MARIE_TRY(finish_out(Vsol, x_d, n * sizeof(double2), st));
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  if (solvert) *solvert = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return check_kernel_status(p);
}

int marie_jvie_solve_batch(marie_plan* p, const double* Einc, int64_t nexc, const double* e_r, double dx, double freq,
                           int form, char precond, double tol, int inner_it, int outer_it, double* Je, int* flag,
                           double* relres, int* iter, double* solvert) {
  if (!p || !Einc || !e_r || !Je || nexc < 1) return set_error(MARIE_EINVAL, "NULL argument or nexc < 1");
  if (!p->has_op) return set_error(MARIE_ENOOP, "plan has no operator");
  if (!(dx > 0) || !(freq > 0)) return set_error(MARIE_EINVAL, "dx and freq must be positive");
  MARIE_TRY(clamp_args(tol, form, precond, inner_it, outer_it));
  const auto t0 = std::chrono::steady_clock::now();
  cudaStream_t st = p->stream;
  const long long V = p->d.V;
  DBuf tE, tER, tJe;
  const void *E_d, *er_d;
  void* Je_d;
  MARIE_TRY(stage_in(Einc, (size_t)nexc * 3 * V * sizeof(double2), st, tE, &E_d));
  MARIE_TRY(stage_in(e_r, V * sizeof(double2), st, tER, &er_d));
  MARIE_TRY(stage_out(Je, (size_t)nexc * 3 * V * sizeof(double2), st, tJe, &Je_d));
  HostPrefault pf;
  pf.start(Je, (size_t)nexc * 3 * V * sizeof(double2));
  SolveOut so;
  MARIE_TRY(jvie_solve_core(p, (const double2*)E_d, 3 * V, (int)nexc, (const double2*)er_d, dx, freq, form, precond,
                            tol, inner_it, outer_it, (double2*)Je_d, 3 * V, so));
  pf.join();
  MARIE_TRY(finish_out(Je, Je_d, (size_t)nexc * 3 * V * sizeof(double2), st));
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  const auto t1 = std::chrono::steady_clock::now();
  for (int64_t e = 0; e < nexc; ++e) {
    if (flag) flag[e] = so.r[e].flag;
    if (relres) relres[e] = so.r[e].relres;
    if (iter) {
      iter[2 * e] = so.r[e].iter[0];
      iter[2 * e + 1] = so.r[e].iter[1];
    }
  }
  if (solvert) *solvert = std::chrono::duration<double>(t1 - t0).count();
  return check_kernel_status(p);
}

int marie_jvie_solve_bodies(int nbody, marie_plan* const* plans, const double* const* Einc, const int64_t* nexc,
                            const double* const* e_r, const double* dx, double freq, int form, char precond,
                            double tol, int inner_it, int outer_it, double* const* Je, int* flag, double* relres,
                            int* iter, double* solvert) {
  if (nbody < 1 || !plans || !Einc || !nexc || !e_r || !dx || !Je) return set_error(MARIE_EINVAL, "NULL argument");
  for (int b = 0; b < nbody; ++b)
    if (!plans[b]) return set_error(MARIE_EINVAL, "NULL plan (body %d)", b);
  const auto t0 = std::chrono::steady_clock::now();
  // bodies on one device whose plans refine in graphs: all refinements in one
  // graph launch
  bool one_launch = nbody >= 2;
  for (int b = 0; b < nbody && one_launch; ++b)
    one_launch = plans[b]->device == plans[0]->device && plans[b]->graph_refine &&
                 plans[b]->precision == MARIE_MIXED;
  if (one_launch) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaSetDevice(plans[0]->device);
    const int s = solve_bodies_one_launch(nbody, plans, Einc, nexc, e_r, dx, freq, form, precond, tol, inner_it,
                                          outer_it, Je, flag, relres, iter);
    cudaSetDevice(dev);
    if (s != MARIE_OK) return s;
    const auto t1 = std::chrono::steady_clock::now();
    if (solvert) *solvert = std::chrono::duration<double>(t1 - t0).count();
    return MARIE_OK;
  }
  std::vector<int> status(nbody, MARIE_OK);
  std::vector<std::string> msg(nbody);
  std::vector<long long> off(nbody + 1, 0);
  for (int b = 0; b < nbody; ++b) off[b + 1] = off[b] + nexc[b];
  // one host thread per body; each body's plan stream runs its own batch, so
  // the bodies execute concurrently on the device
  std::vector<std::thread> th;
  for (int b = 0; b < nbody; ++b) {
    th.emplace_back([&, b]() {
      int dev = 0;
      cudaGetDevice(&dev);
      cudaSetDevice(plans[b]->device);
      const int s = marie_jvie_solve_batch(plans[b], Einc[b], nexc[b], e_r[b], dx[b], freq, form, precond, tol,
                                           inner_it, outer_it, Je[b], flag ? flag + off[b] : nullptr,
                                           relres ? relres + off[b] : nullptr, iter ? iter + 2 * off[b] : nullptr,
                                           nullptr);
      status[b] = s;
      if (s != MARIE_OK) msg[b] = marie_last_error();
    });
  }
  for (auto& t : th) t.join();
  for (int b = 0; b < nbody; ++b)
    if (status[b] != MARIE_OK) return set_error(status[b], "body %d: %s", b, msg[b].c_str());
  const auto t1 = std::chrono::steady_clock::now();
  if (solvert) *solvert = std::chrono::duration<double>(t1 - t0).count();
  return MARIE_OK;
}

}  // extern "C"
