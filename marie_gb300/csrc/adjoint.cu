// Adjoint gradient of a field objective with respect to the per-voxel relative
// permittivity eps_r and conductivity sigma of the body (no counterpart in the
// reference, which has no derivatives; built on its J-VIE operator).
//
// In body voxels the total field is E = J / (j omega eps0 chi) with
// chi = eps_c - 1 and eps_c = eps_r - j sigma / (eps0 omega) (E_field_Nop.m:84
// with JVIE_Solver.m:151-156).  Dividing the J-VIE system A J = b by
// j omega eps0 chi gives K E = Gram Einc with K = Gram (1 + chi) - N chi,
// and K^T = Gram (1 + chi) - chi N is the reference's own form-1 operator A
// (N is symmetric).  For a real objective F(E):
//   dF = 2 Re(w^T dE),  w = dF/dE (Wirtinger),  dE = -K^{-1} (Gram - N) P_i E dchi_i
//   => solve A lambda = w (the same J-VIE solver), q = (Gram - N) lambda,
//      s_i = sum_c q_ic E_ic,
//      dF/d eps_r_i = -2 Re(s_i),  dF/d sigma_i = -2 Im(s_i) / (eps0 omega)
//      (+ the explicit 0.5 |E_i|^2 of the absorbed-power objective).
// Objectives: 0  F = sum_i 0.5 sigma_i |E_i|^2          (absorbed power)
//             1  F = sum_i |E_i - E_target,i|^2         (field misfit)
// over the body voxels.  Both solves use the plan's arithmetic (FP64, or the
// FP32-matvec GMRES-IR of a MARIE_MIXED plan).
#include <cmath>
#include <vector>

#include "plan.h"

namespace marie {

// E_k = J_k / (j omega eps0 chi_v) on body DOFs; w_k = dF/dE_k; per-block F partials
__global__ void k_adj_fields(const double2* __restrict__ J, const int64_t* __restrict__ idx3, long long n,
                             long long V, const double2* __restrict__ er, double omega_eps0, int objective,
                             const double2* __restrict__ Et, double2* __restrict__ E, double2* __restrict__ w,
                             double* __restrict__ Fpart) {
  double f = 0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const long long g = idx3[k] - 1;
    const double2 e = er[g % V];
    const double2 chi = mk<double2>(e.x - 1.0, e.y);
    const double2 den = mk<double2>(-omega_eps0 * chi.y, omega_eps0 * chi.x);  // j omega eps0 chi
    const double d2 = den.x * den.x + den.y * den.y;
    const double2 jv = J[k];
    const double2 Ek = mk<double2>((jv.x * den.x + jv.y * den.y) / d2, (jv.y * den.x - jv.x * den.y) / d2);
    E[k] = Ek;
    double2 wk;
    if (objective == 0) {
      const double sigma = -e.y * omega_eps0;  // eps_c = eps_r - j sigma/(eps0 omega)
      f += 0.5 * sigma * (Ek.x * Ek.x + Ek.y * Ek.y);
      wk = mk<double2>(0.5 * sigma * Ek.x, -0.5 * sigma * Ek.y);  // 0.5 sigma conj(E)
    } else {
      const double2 d = csub(Ek, Et[g]);
      f += d.x * d.x + d.y * d.y;
      wk = mk<double2>(d.x, -d.y);  // conj(E - Et)
    }
    // form-2 system rows are divided by eps_c: rhs w / eps_c
    const double ed = e.x * e.x + e.y * e.y;
    w[k] = mk<double2>((wk.x * e.x + wk.y * e.y) / ed, (wk.y * e.x - wk.x * e.y) / ed);
  }
  for (int o = 16; o > 0; o >>= 1) f += __shfl_xor_sync(0xffffffffu, f, o);
  __shared__ double sh[32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = f;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += sh[i];
    Fpart[blockIdx.x] = t;
  }
}

// fused gradient: s_v = sum_c q_{v,c} E_{v,c} over the three DOFs of voxel v
// (DOF k = c*nS + s), scattered to the grid.
__global__ void k_adj_grad(const double2* __restrict__ q, const double2* __restrict__ E, const int* __restrict__ idxS,
                           long long nS, const double2* __restrict__ er, double omega_eps0, int objective,
                           double* __restrict__ g_eps, double* __restrict__ g_sig) {
  for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < nS; s += (long long)gridDim.x * blockDim.x) {
    double2 acc = mk<double2>(0, 0);
    double e2 = 0;
    for (int c = 0; c < 3; ++c) {
      const double2 qq = q[c * nS + s], ee = E[c * nS + s];
      acc = cadd(acc, cmul(qq, ee));
      e2 += ee.x * ee.x + ee.y * ee.y;
    }
    const long long v = idxS[s];
    g_eps[v] = -2.0 * acc.x;
    double gs = -2.0 * acc.y / omega_eps0;
    if (objective == 0) gs += 0.5 * e2;
    g_sig[v] = gs;
  }
}

// forward + adjoint solves and the gradient assembly (jvie.cu, which owns the
// solver state)
int jvie_adjoint_core(marie_plan* p, const double2* Einc, const double2* er, double dx, double freq, int objective,
                      const double2* Et, double tol, int inner_it, int outer_it, double* F, double* g_eps,
                      double* g_sig, int* flags, int* iters);
}

using namespace marie;

extern "C" int marie_jvie_adjoint_grad(marie_plan* p, const double* Einc, const double* e_r, double dx, double freq,
                                       int objective, const double* E_target, double tol, int inner_it, int outer_it,
                                       double* F, double* dF_deps, double* dF_dsigma, int* flags, int* iters) {
  if (!p || !Einc || !e_r || !F || !dF_deps || !dF_dsigma) return set_error(MARIE_EINVAL, "NULL argument");
  if (objective != 0 && objective != 1) return set_error(MARIE_EINVAL, "objective must be 0 (power) or 1 (misfit)");
  if (objective == 1 && !E_target) return set_error(MARIE_EINVAL, "the misfit objective needs E_target");
  if (!p->has_op) return set_error(MARIE_ENOOP, "plan has no operator");
  if (tol < 1e-15 || tol >= 1) tol = 1e-3;
  if (inner_it < 1) inner_it = 50;
  if (outer_it < 1) outer_it = 200;
  cudaStream_t st = p->stream;
  const long long V = p->d.V;
  DBuf tE, tER, tEt, tge, tgs;
  const void *E_d, *er_d, *Et_d = nullptr;
  void *ge_d, *gs_d;
  MARIE_TRY(stage_in(Einc, 3 * V * sizeof(double2), st, tE, &E_d));
  MARIE_TRY(stage_in(e_r, V * sizeof(double2), st, tER, &er_d));
  if (E_target) MARIE_TRY(stage_in(E_target, 3 * V * sizeof(double2), st, tEt, &Et_d));
  MARIE_TRY(stage_out(dF_deps, V * sizeof(double), st, tge, &ge_d));
  MARIE_TRY(stage_out(dF_dsigma, V * sizeof(double), st, tgs, &gs_d));
  MARIE_TRY(jvie_adjoint_core(p, (const double2*)E_d, (const double2*)er_d, dx, freq, objective,
                              (const double2*)Et_d, tol, inner_it, outer_it, F, (double*)ge_d, (double*)gs_d, flags,
                              iters));
  MARIE_TRY(finish_out(dF_deps, ge_d, V * sizeof(double), st));
  MARIE_TRY(finish_out(dF_dsigma, gs_d, V * sizeof(double), st));
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  return check_kernel_status(p);
}
