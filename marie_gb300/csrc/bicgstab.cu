// BiCGSTAB on device vectors with the interface and outputs of MATLAB's
// bicgstab, which the reference's JVIE_Solver uses for its default solver 'B'
// (src_vie/src_solver/JVIE_Solver.m:451-499): [x, flag, relres, iter, resvec]
// with iter counted in half steps and resvec the absolute residual norm after
// every half step.  bicgstab is a MATLAB built-in, not part of the reference
// sources; this follows the published iteration (van der Vorst, SIAM J. Sci.
// Stat. Comput. 13, 1992) and MATLAB's documented conventions:
//   * preconditioner applied as ph = M2(M1(p)) (function handles), so the
//     recurrence residuals are those of the unpreconditioned system;
//   * flag 0 converged, 1 maxit reached, 2 preconditioner output not finite,
//     3 stagnation, 4 a breakdown scalar (rho, beta, r~'v, t't zero or not
//     finite);
//   * a small recurrence residual is confirmed with a true residual b - A x,
//     which then replaces it; up to min(n/50, 5, n - maxit) confirmations may
//     fail before flag 3;
//   * without convergence the iterate of smallest residual norm is returned.
//
// Device side: every vector update is fused with the reductions the next
// scalar needs (one pass per half step), the reductions are two-stage in a
// fixed order (bitwise reproducible), and the host reads the few scalars of
// each half step from pinned memory.
#include <algorithm>
#include <cmath>
#include <complex>
#include <limits>
#include <vector>

#include "plan.h"

namespace marie {

using cd = std::complex<double>;

static constexpr int BI_BLOCKS = 304;  // 2 x 152 SMs
static constexpr int BI_THREADS = 256;
static constexpr int BI_NQ = 5;  // reduced quantities per pass, at most

struct BiVec {
  const double2* b;
  const double2* rt;
  double2 *x, *xh, *r, *s, *p, *v, *ph, *sh, *t, *y;
  double2 alpha, omega, beta;
  long long n;
};

enum BiOp { BI_DOTV, BI_HALF, BI_TPASS, BI_FULL, BI_PUPD, BI_RES_S, BI_RES_R, BI_INIT };

template <int OP> struct BiNQ { static constexpr int value = 0; };
template <> struct BiNQ<BI_DOTV> { static constexpr int value = 4; };   // r~'v (2), |ph|^2, |x|^2
template <> struct BiNQ<BI_HALF> { static constexpr int value = 1; };   // |s|^2
template <> struct BiNQ<BI_TPASS> { static constexpr int value = 5; };  // t't, t's (2), |sh|^2, |xh|^2
template <> struct BiNQ<BI_FULL> { static constexpr int value = 3; };   // |r|^2, r~'r (2)
template <> struct BiNQ<BI_RES_S> { static constexpr int value = 1; };  // |s|^2
template <> struct BiNQ<BI_RES_R> { static constexpr int value = 3; };  // |r|^2, r~'r (2)
template <> struct BiNQ<BI_INIT> { static constexpr int value = 2; };   // |r|^2, |b|^2

__device__ __forceinline__ double bi_wsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// conj(a) * b accumulated into (re, im)
__device__ __forceinline__ void dotc(double2 a, double2 b, double& re, double& im) {
  re = fma(a.x, b.x, fma(a.y, b.y, re));
  im = fma(a.x, b.y, fma(-a.y, b.x, im));
}
__device__ __forceinline__ double2 axpy(double2 y, double2 a, double2 x) {  // y + a x
  return mk<double2>(fma(a.x, x.x, fma(-a.y, x.y, y.x)), fma(a.x, x.y, fma(a.y, x.x, y.y)));
}

// One fused vector pass; part[q * gridDim.x + block] = block partial of q.
template <int OP>
__global__ void __launch_bounds__(BI_THREADS) k_bi(BiVec a, double* __restrict__ part) {
  constexpr int NQ = BiNQ<OP>::value;
  double acc[NQ > 0 ? NQ : 1] = {};
  const long long chunk = (a.n + gridDim.x - 1) / gridDim.x;
  const long long i0 = blockIdx.x * chunk;
  const long long i1 = i0 + chunk < a.n ? i0 + chunk : a.n;
  for (long long i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    if constexpr (OP == BI_DOTV) {
      const double2 v = a.v[i], ph = a.ph[i], x = a.x[i];
      dotc(a.rt[i], v, acc[0], acc[1]);
      acc[2] = fma(ph.x, ph.x, fma(ph.y, ph.y, acc[2]));
      acc[3] = fma(x.x, x.x, fma(x.y, x.y, acc[3]));
    } else if constexpr (OP == BI_HALF) {
      a.xh[i] = axpy(a.x[i], a.alpha, a.ph[i]);
      const double2 s = axpy(a.r[i], mk<double2>(-a.alpha.x, -a.alpha.y), a.v[i]);
      a.s[i] = s;
      acc[0] = fma(s.x, s.x, fma(s.y, s.y, acc[0]));
    } else if constexpr (OP == BI_TPASS) {
      const double2 t = a.t[i], s = a.s[i], sh = a.sh[i], xh = a.xh[i];
      acc[0] = fma(t.x, t.x, fma(t.y, t.y, acc[0]));
      dotc(t, s, acc[1], acc[2]);
      acc[3] = fma(sh.x, sh.x, fma(sh.y, sh.y, acc[3]));
      acc[4] = fma(xh.x, xh.x, fma(xh.y, xh.y, acc[4]));
    } else if constexpr (OP == BI_FULL) {
      a.x[i] = axpy(a.xh[i], a.omega, a.sh[i]);
      const double2 r = axpy(a.s[i], mk<double2>(-a.omega.x, -a.omega.y), a.t[i]);
      a.r[i] = r;
      acc[0] = fma(r.x, r.x, fma(r.y, r.y, acc[0]));
      dotc(a.rt[i], r, acc[1], acc[2]);
    } else if constexpr (OP == BI_PUPD) {
      // p = r + beta (p - omega v)
      const double2 q = axpy(a.p[i], mk<double2>(-a.omega.x, -a.omega.y), a.v[i]);
      a.p[i] = axpy(a.r[i], a.beta, q);
    } else if constexpr (OP == BI_RES_S) {
      const double2 s = csub(a.b[i], a.y[i]);
      a.s[i] = s;
      acc[0] = fma(s.x, s.x, fma(s.y, s.y, acc[0]));
    } else if constexpr (OP == BI_RES_R) {
      const double2 r = csub(a.b[i], a.y[i]);
      a.r[i] = r;
      acc[0] = fma(r.x, r.x, fma(r.y, r.y, acc[0]));
      dotc(a.rt[i], r, acc[1], acc[2]);
    } else if constexpr (OP == BI_INIT) {
      // r = b - y (y = A x0, or null for x0 = 0); r~ = r
      const double2 b = a.b[i];
      const double2 r = a.y ? csub(b, a.y[i]) : b;
      a.r[i] = r;
      a.p[i] = r;  // r~ storage (rt is const in the struct)
      acc[0] = fma(r.x, r.x, fma(r.y, r.y, acc[0]));
      acc[1] = fma(b.x, b.x, fma(b.y, b.y, acc[1]));
    }
  }
  if constexpr (NQ > 0) {
    __shared__ double ws[NQ][BI_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NQ; ++q) {
      const double v = bi_wsum(acc[q]);
      if (lane == 0) ws[q][wid] = v;
    }
    __syncthreads();
    if (threadIdx.x < NQ) {
      double s = 0;
      for (int w = 0; w < BI_THREADS / 32; ++w) s += ws[threadIdx.x][w];
      part[(long long)threadIdx.x * gridDim.x + blockIdx.x] = s;
    }
  }
}

// out[q] = sum over blocks of part[q], fixed order; one block per quantity
__global__ void k_bi_fin(const double* __restrict__ part, int G, double* __restrict__ out) {
  __shared__ double ws[BI_THREADS / 32];
  double s = 0;
  for (int b = threadIdx.x; b < G; b += blockDim.x) s += part[(long long)blockIdx.x * G + b];
  s = bi_wsum(s);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) ws[wid] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += ws[w];
    out[blockIdx.x] = t;
  }
}

namespace {

struct BiWork {
  marie_plan* p = nullptr;
  long long n = 0;
  DBuf r, rt, pv, v, ph, s, sh, t, xh, y, xbest, part, red;
  BiVec a{};
  int init(marie_plan* pl, long long nn, bool precond) {
    p = pl;
    n = nn;
    cudaStream_t st = p->stream;
    const size_t vb = (size_t)n * sizeof(double2);
    for (DBuf* b : {&r, &rt, &pv, &v, &s, &t, &xh, &y, &xbest}) MARIE_TRY(b->alloc(vb, st));
    if (precond) {
      MARIE_TRY(ph.alloc(vb, st));
      MARIE_TRY(sh.alloc(vb, st));
    }
    MARIE_TRY(part.alloc((size_t)BI_BLOCKS * BI_NQ * sizeof(double), st));
    MARIE_TRY(red.alloc(BI_NQ * sizeof(double), st));
    MARIE_TRY(ensure_pinned(p, BI_NQ));
    a.rt = rt.as<double2>();
    a.r = r.as<double2>();
    a.p = pv.as<double2>();
    a.v = v.as<double2>();
    a.s = s.as<double2>();
    a.t = t.as<double2>();
    a.xh = xh.as<double2>();
    a.y = y.as<double2>();
    // without a preconditioner ph = p and sh = s (no copies)
    a.ph = precond ? ph.as<double2>() : a.p;
    a.sh = precond ? sh.as<double2>() : a.s;
    a.n = n;
    return MARIE_OK;
  }
  // run pass OP and, when it reduces, bring its NQ sums to q (host)
  template <int OP> int pass(double* q) {
    cudaStream_t st = p->stream;
    k_bi<OP><<<BI_BLOCKS, BI_THREADS, 0, st>>>(a, part.as<double>());
    count_launch();
    constexpr int NQ = BiNQ<OP>::value;
    if constexpr (NQ > 0) {
      k_bi_fin<<<NQ, BI_THREADS, 0, st>>>(part.as<double>(), BI_BLOCKS, red.as<double>());
      count_launch();
      MARIE_CUDA_TRY(cudaGetLastError());
      MARIE_CUDA_TRY(cudaMemcpyAsync(p->pinned, red.p, NQ * sizeof(double), cudaMemcpyDeviceToHost, st));
      MARIE_CUDA_TRY(cudaStreamSynchronize(st));
      for (int i = 0; i < NQ; ++i) q[i] = p->pinned[i];
    } else {
      MARIE_CUDA_TRY(cudaGetLastError());
    }
    return MARIE_OK;
  }
};

bool finite(cd v) { return std::isfinite(v.real()) && std::isfinite(v.imag()); }

}  // namespace

int bicgstab(marie_plan* p, const DevOp& A, const DevOp* M1, const DevOp* M2, const double2* b, long long n,
             double tol, int maxit, const double2* x0, double2* x, BicgResult& out) {
  if (maxit < 0) return set_error(MARIE_EINVAL, "maxit must be >= 0");
  MARIE_TRACE("bicgstab");
  cudaStream_t st = p->stream;
  const bool precond = M1 || M2;
  BiWork W;
  MARIE_TRY(W.init(p, n, precond));
  BiVec& a = W.a;
  a.b = b;
  a.x = x;
  out = BicgResult();
  const size_t vb = (size_t)n * sizeof(double2);
  auto prec = [&](const double2* in, double2* o) -> int {
    if (M1 && M2) {
      MARIE_TRY((*M1)(in, W.y.as<double2>()));
      return (*M2)(W.y.as<double2>(), o);
    }
    return M1 ? (*M1)(in, o) : (*M2)(in, o);
  };
  double q[BI_NQ];
  // x = x0; r = b - A x0 (or b when x0 is zero); r~ = r
  double x0n = 0;
  if (x0) MARIE_TRY(dev_norm2(p, x0, n, &x0n));
  BiVec ai = a;
  ai.p = W.rt.as<double2>();  // BI_INIT writes r~ through p
  if (x0 && x0n > 0) {
    MARIE_CUDA_TRY(cudaMemcpyAsync(x, x0, vb, cudaMemcpyDeviceToDevice, st));
    MARIE_TRY(A(x, W.y.as<double2>()));
  } else {
    MARIE_CUDA_TRY(cudaMemsetAsync(x, 0, vb, st));
    ai.y = nullptr;
  }
  std::swap(W.a, ai);
  MARIE_TRY(W.pass<BI_INIT>(q));
  std::swap(W.a, ai);
  const double nb = std::sqrt(q[1]);
  double nr = std::sqrt(q[0]);
  if (nb == 0) {
    MARIE_CUDA_TRY(cudaMemsetAsync(x, 0, vb, st));
    out.flag = 0;
    out.relres = 0;
    out.iter = 0;
    out.resvec = {0.0};
    return MARIE_OK;
  }
  const double tolb = tol * nb;
  out.resvec.push_back(nr);
  if (nr <= tolb) {
    out.flag = 0;
    out.relres = nr / nb;
    out.iter = 0;
    return MARIE_OK;
  }
  const double eps = std::numeric_limits<double>::epsilon();
  double best_nr = nr, best_it = 0;
  MARIE_CUDA_TRY(cudaMemcpyAsync(W.xbest.p, x, vb, cudaMemcpyDeviceToDevice, st));
  cd rho_old(1, 0), alpha(1, 0), omega(1, 0), rho(q[0], 0);  // r~ = r: rho_1 = |r|^2
  int flag = 1, stag = 0, extra = 0;
  double it = maxit;
  const long long max_extra = std::min<long long>(std::min<long long>(n / 50, 5), n - maxit);
  double nr_act = nr, nx = x0n;

  // true-residual confirmation behind a small recurrence residual (see header)
  enum { GO, OK, STOP };
  auto confirm = [&](double2* xc, bool half, double& nrc, int& outc) -> int {
    outc = GO;
    if (!(nrc <= tolb || stag >= 3 || extra)) return MARIE_OK;
    MARIE_TRY(A(xc, W.y.as<double2>()));
    if (half) {
      MARIE_TRY(W.pass<BI_RES_S>(q));
      nrc = std::sqrt(q[0]);
    } else {
      MARIE_TRY(W.pass<BI_RES_R>(q));
      nrc = std::sqrt(q[0]);
      rho = cd(q[1], q[2]);
    }
    if (nrc <= tolb) {
      outc = OK;
      return MARIE_OK;
    }
    if (stag >= 3 && extra == 0) stag = 0;
    ++extra;
    outc = extra >= max_extra ? STOP : GO;
    return MARIE_OK;
  };

  int i = 1;
  for (; i <= maxit; ++i) {
    if (rho == cd(0, 0) || !finite(rho)) {
      flag = 4;
      break;
    }
    if (i == 1) {
      MARIE_CUDA_TRY(cudaMemcpyAsync(a.p, a.r, vb, cudaMemcpyDeviceToDevice, st));
    } else {
      const cd beta = (rho / rho_old) * (alpha / omega);
      if (beta == cd(0, 0) || !finite(beta)) {
        flag = 4;
        break;
      }
      a.beta = mk<double2>(beta.real(), beta.imag());
      a.omega = mk<double2>(omega.real(), omega.imag());
      MARIE_TRY(W.pass<BI_PUPD>(q));
    }
    if (precond) MARIE_TRY(prec(a.p, a.ph));
    MARIE_TRY(A(a.ph, a.v));
    MARIE_TRY(W.pass<BI_DOTV>(q));
    const cd rtv(q[0], q[1]);
    const double nph = std::sqrt(q[2]);
    nx = std::sqrt(q[3]);
    if (!std::isfinite(q[2])) {
      flag = 2;
      break;
    }
    if (rtv == cd(0, 0) || !finite(rtv)) {
      flag = 4;
      break;
    }
    alpha = rho / rtv;
    stag = std::abs(alpha) * nph < eps * nx ? stag + 1 : 0;
    a.alpha = mk<double2>(alpha.real(), alpha.imag());
    MARIE_TRY(W.pass<BI_HALF>(q));
    nr_act = std::sqrt(q[0]);
    int oc;
    MARIE_TRY(confirm(a.xh, true, nr_act, oc));
    out.resvec.push_back(nr_act);
    if (oc != GO) {
      MARIE_CUDA_TRY(cudaMemcpyAsync(x, a.xh, vb, cudaMemcpyDeviceToDevice, st));
      flag = oc == OK ? 0 : 3;
      it = i - 0.5;
      break;
    }
    if (nr_act < best_nr) {
      best_nr = nr_act;
      best_it = i - 0.5;
      MARIE_CUDA_TRY(cudaMemcpyAsync(W.xbest.p, a.xh, vb, cudaMemcpyDeviceToDevice, st));
    }
    if (precond) MARIE_TRY(prec(a.s, a.sh));
    MARIE_TRY(A(a.sh, a.t));
    MARIE_TRY(W.pass<BI_TPASS>(q));
    const double tt = q[0];
    const cd ts(q[1], q[2]);
    const double nsh = std::sqrt(q[3]), nxh = std::sqrt(q[4]);
    if (!std::isfinite(q[3])) {
      flag = 2;
      break;
    }
    if (tt == 0 || !std::isfinite(tt)) {
      flag = 4;
      break;
    }
    omega = ts / tt;
    stag = std::abs(omega) * nsh < eps * nxh ? stag + 1 : 0;
    a.omega = mk<double2>(omega.real(), omega.imag());
    MARIE_TRY(W.pass<BI_FULL>(q));
    nr_act = std::sqrt(q[0]);
    const cd rho_next(q[1], q[2]);
    rho_old = rho;
    rho = rho_next;
    MARIE_TRY(confirm(x, false, nr_act, oc));
    out.resvec.push_back(nr_act);
    if (oc != GO) {
      flag = oc == OK ? 0 : 3;
      it = i;
      break;
    }
    if (nr_act < best_nr) {
      best_nr = nr_act;
      best_it = i;
      MARIE_CUDA_TRY(cudaMemcpyAsync(W.xbest.p, x, vb, cudaMemcpyDeviceToDevice, st));
    }
    if (omega == cd(0, 0)) {
      flag = 4;
      break;
    }
  }
  if (flag == 0) {
    out.relres = nr_act / nb;
  } else {
    if (flag == 2 || flag == 4) it = (double)out.resvec.size() / 2.0 - 0.5;
    // the best iterate's true residual against the last one
    MARIE_TRY(A(W.xbest.as<double2>(), W.y.as<double2>()));
    MARIE_TRY(W.pass<BI_RES_S>(q));  // s = b - A xbest (s is free now)
    const double nbest = std::sqrt(q[0]);
    if (nbest <= nr_act) {
      MARIE_CUDA_TRY(cudaMemcpyAsync(x, W.xbest.p, vb, cudaMemcpyDeviceToDevice, st));
      it = best_it;
      out.relres = nbest / nb;
    } else {
      out.relres = nr_act / nb;
    }
  }
  out.flag = flag;
  out.iter = it;
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  return MARIE_OK;
}

}  // namespace marie

using namespace marie;

extern "C" int marie_bicgstab(marie_plan* p, marie_op_fn A, void* A_ctx, const double* b, int64_t n, double tol,
                              int maxit, marie_op_fn M1, void* M1_ctx, marie_op_fn M2, void* M2_ctx, const double* x0,
                              double* x, int* flag, double* relres, double* iter, double* resvec, int64_t resvec_cap,
                              int64_t* resvec_len) {
  if (!p || !b || !x || n < 1) return set_error(MARIE_EINVAL, "NULL argument or n < 1");
  // user operators run outside the plan's stream: finish the plan's work first
  auto wrap = [p](marie_op_fn f, void* ctx, long long nn) -> DevOp {
    return [p, f, ctx, nn](const double2* xi, double2* yo) -> int {
      MARIE_CUDA_TRY(cudaStreamSynchronize(p->stream));
      const int s = f(ctx, reinterpret_cast<const double*>(xi), reinterpret_cast<double*>(yo), nn);
      if (s != MARIE_OK) return set_error(s, "user operator returned status %d", s);
      return MARIE_OK;
    };
  };
  DevOp opA, oM1, oM2;
  if (A)
    opA = wrap(A, A_ctx, n);
  else
    MARIE_TRY(bound_operator(p, n, &opA));  // NULL A: the plan's bound mv_AN
  if (M1) oM1 = wrap(M1, M1_ctx, n);
  if (M2) oM2 = wrap(M2, M2_ctx, n);
  const size_t bytes = (size_t)n * sizeof(double2);
  DBuf tb, tx0, txo;
  const void *b_d, *x0_d = nullptr;
  void* x_d;
  MARIE_TRY(stage_in(b, bytes, p->stream, tb, &b_d));
  if (x0) MARIE_TRY(stage_in(x0, bytes, p->stream, tx0, &x0_d));
  MARIE_TRY(stage_out(x, bytes, p->stream, txo, &x_d));
  BicgResult res;
  MARIE_TRY(bicgstab(p, opA, M1 ? &oM1 : nullptr, M2 ? &oM2 : nullptr, (const double2*)b_d, n, tol, maxit,
                     (const double2*)x0_d, (double2*)x_d, res));
  MARIE_TRY(finish_out(x, x_d, bytes, p->stream));
  MARIE_CUDA_TRY(cudaStreamSynchronize(p->stream));
  if (flag) *flag = res.flag;
  if (relres) *relres = res.relres;
  if (iter) *iter = res.iter;
  const int64_t nr = (int64_t)res.resvec.size();
  if (resvec_len) *resvec_len = nr;
  if (resvec)
    for (int64_t i = 0; i < nr && i < resvec_cap; ++i) resvec[i] = res.resvec[i];
  return check_kernel_status(p);
}
