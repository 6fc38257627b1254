// GMRES with deflated restarting on device vectors, with the semantics of the
// reference's pgmresDR (src_numeric/src_iterative/pgmresDR.m:84-282,
// pgmresDR_iter.m:36-142, getHarmVecs1.m, getHarmVecs2.m):
//   * the first cycle is GMRES(m) with classical Gram-Schmidt; every later
//     cycle keeps its Krylov vectors orthogonal to C (B = C' w, w -= C B);
//   * after a cycle, x += [U V] y and r -= [C V] (H2 y) with y the least-squares
//     solution of H2 y = [C V]' r (H2 = [D B; 0 H], D the column norms of U);
//   * the ritz harmonic Ritz vectors of smallest |theta| (getHarmVecs1 after
//     the first cycle, the generalized problem of getHarmVecs2 afterwards)
//     become the new U, and C = [C V] Q, U = U / R from qr(H2 P, 0);
//   * right preconditioners are applied once to the accumulated x at the end,
//     then x = x0 + x and the true residual gives relres and flag.
// Device side: the Krylov basis [C | V] (n x (ritz + m + 1), FP64 complex,
// columns contiguous), U, and the fused dot / update / combine kernels of the
// GMRES path (fixed-order reductions).  Host side: the projected problems
// (least squares, QR, eigenpairs) in FP64 on matrices of size ~m.
#include <cmath>
#include <vector>

#include "dense.h"
#include "plan.h"

namespace marie {

// vector kernels of krylov.cu
__global__ void k_dot_partials(const double2* Vb, long long ld, int ncols, const double2* w, long long n,
                               double2* partial);
__global__ void k_reduce_cols(const double2* partial, int G, double2* out);
__global__ void k_update_norm(const double2* Vb, long long ld, int ncols, const double2* h, double2* w, long long n,
                              double* partial);
__global__ void k_reduce_real(const double* partial, int G, double* out);
__global__ void k_scale(const double2* x, double s, double2* y, long long n);
__global__ void k_sub_from(const double2* x, double2* y, long long n);
__global__ void k_add_to(const double2* x, double2* y, long long n);
__global__ void k_combine(const double2* Vb, long long ld, int ncols, const double2* c, double2* y, long long n);

namespace {

using dense::cd;
using dense::Mat;

constexpr int DR_BLOCKS = 304;  // the reduction grid of krylov.cu
constexpr int DR_THREADS = 256;
constexpr int DR_MAXCOLS = 128;  // k_combine / k_update_norm stage this many coefficients

inline int grid_n(long long n) { return grid_stride_blocks(n, 8); }

struct DrWork {
  marie_plan* p = nullptr;
  long long n = 0;
  int m = 0, kmax = 0;
  DBuf CV, U, Unew, tmp, tmp2, w2, dpart, npart, dev_c, nrm;
  // [C | V]: C in columns [kmax - kc, kmax), V in [kmax, kmax + m + 1)
  double2* col(int j) { return CV.as<double2>() + (long long)j * n; }
  double2* V(int j) { return col(kmax + j); }
  double2* Ucol(int j) { return U.as<double2>() + (long long)j * n; }
  double2* Unewcol(int j) { return Unew.as<double2>() + (long long)j * n; }
  int init(marie_plan* pl, long long nn, int mm, int kk) {
    p = pl;
    n = nn;
    m = mm;
    kmax = kk;
    cudaStream_t st = p->stream;
    const size_t vb = (size_t)n * sizeof(double2);
    MARIE_TRY(CV.alloc(vb * (kmax + m + 1), st));
    MARIE_TRY(U.alloc(vb * (kmax > 0 ? kmax : 1), st));
    MARIE_TRY(Unew.alloc(vb * (kmax > 0 ? kmax : 1), st));
    MARIE_TRY(tmp.alloc(vb, st));
    MARIE_TRY(tmp2.alloc(vb, st));
    MARIE_TRY(w2.alloc(vb, st));
    MARIE_TRY(dpart.alloc((size_t)DR_BLOCKS * (kmax + m + 1) * sizeof(double2), st));
    MARIE_TRY(npart.alloc((size_t)DR_BLOCKS * sizeof(double), st));
    MARIE_TRY(dev_c.alloc((size_t)(kmax + m + 2) * sizeof(double2), st));
    MARIE_TRY(nrm.alloc(sizeof(double), st));
    MARIE_TRY(ensure_pinned(p, 2 * (size_t)(kmax + m + 2) + 2));
    return MARIE_OK;
  }
  // out[j] = Vb(:, j)^H w for j < ncols (host)
  int dots(const double2* Vb, int ncols, const double2* w, std::vector<cd>& out) {
    cudaStream_t st = p->stream;
    out.assign(ncols, cd(0, 0));
    if (ncols == 0) return MARIE_OK;
    k_dot_partials<<<DR_BLOCKS, DR_THREADS, 0, st>>>(Vb, n, ncols, w, n, dpart.as<double2>());
    count_launch();
    k_reduce_cols<<<ncols, DR_THREADS, 0, st>>>(dpart.as<double2>(), DR_BLOCKS, dev_c.as<double2>());
    count_launch();
    MARIE_CUDA_TRY(cudaGetLastError());
    MARIE_CUDA_TRY(cudaMemcpyAsync(p->pinned, dev_c.p, ncols * sizeof(double2), cudaMemcpyDeviceToHost, st));
    MARIE_CUDA_TRY(cudaStreamSynchronize(st));
    for (int j = 0; j < ncols; ++j) out[j] = cd(p->pinned[2 * j], p->pinned[2 * j + 1]);
    return MARIE_OK;
  }
  // w -= Vb(:, :ncols) h; returns ||w|| (host)
  int update(const double2* Vb, int ncols, const std::vector<cd>& h, double2* w, double* norm) {
    cudaStream_t st = p->stream;
    MARIE_TRY(upload(h));
    k_update_norm<<<DR_BLOCKS, DR_THREADS, 0, st>>>(Vb, n, ncols, dev_c.as<double2>(), w, n, npart.as<double>());
    count_launch();
    k_reduce_real<<<1, DR_THREADS, 0, st>>>(npart.as<double>(), DR_BLOCKS, nrm.as<double>());
    count_launch();
    MARIE_CUDA_TRY(cudaGetLastError());
    MARIE_CUDA_TRY(cudaMemcpyAsync(p->pinned, nrm.p, sizeof(double), cudaMemcpyDeviceToHost, st));
    MARIE_CUDA_TRY(cudaStreamSynchronize(st));
    *norm = std::sqrt(p->pinned[0]);
    return MARIE_OK;
  }
  int upload(const std::vector<cd>& c) {
    cudaStream_t st = p->stream;
    // the previous kernels that read dev_c are ordered before this copy on st;
    // the host buffer must not change while the copy is pending
    MARIE_CUDA_TRY(cudaStreamSynchronize(st));
    for (size_t j = 0; j < c.size(); ++j) {
      p->pinned[2 * j] = c[j].real();
      p->pinned[2 * j + 1] = c[j].imag();
    }
    MARIE_CUDA_TRY(cudaMemcpyAsync(dev_c.p, p->pinned, c.size() * sizeof(double2), cudaMemcpyHostToDevice, st));
    return MARIE_OK;
  }
  // y = Vb(:, :ncols) c (ncols >= 1)
  int combine(const double2* Vb, int ncols, const std::vector<cd>& c, double2* y) {
    MARIE_TRY(upload(c));
    k_combine<<<grid_n(n), 256, 0, p->stream>>>(Vb, n, ncols, dev_c.as<double2>(), y, n);
    count_launch();
    MARIE_CUDA_TRY(cudaGetLastError());
    return MARIE_OK;
  }
  int add(const double2* x, double2* y) {
    k_add_to<<<grid_n(n), 256, 0, p->stream>>>(x, y, n);
    count_launch();
    MARIE_CUDA_TRY(cudaGetLastError());
    return MARIE_OK;
  }
  int sub(const double2* x, double2* y) {  // y = x - y
    k_sub_from<<<grid_n(n), 256, 0, p->stream>>>(x, y, n);
    count_launch();
    MARIE_CUDA_TRY(cudaGetLastError());
    return MARIE_OK;
  }
};

// One cycle of pgmresDR_iter.m on the residual r: V, H (k+1 x k), B (kc x k),
// k steps and the absolute LSQ residual norms.  C = the kc columns before V.
int dr_cycle(DrWork& W, const DevOp& A, const DevOp* L1, const DevOp* L2, const DevOp* R1, const DevOp* R2,
             const double2* r, int kc, double tol, Mat& H, Mat& B, int& k_out, std::vector<double>& resvec) {
  marie_plan* p = W.p;
  cudaStream_t st = p->stream;
  const long long n = W.n;
  const int m = W.m;
  double rn = 0;
  MARIE_TRY(dev_norm2(p, r, n, &rn));
  k_scale<<<grid_n(n), 256, 0, st>>>(r, 1.0 / rn, W.V(0), n);
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  H = Mat(m + 1, m);
  B = Mat(kc, m);
  resvec.clear();
  // Givens data for the LSQ residual norm ||rhs - H y|| (= |g(k+1)|)
  Mat R(m + 1, m);
  std::vector<double> gc(m);
  std::vector<cd> gs(m), g(m + 1, cd(0, 0));
  g[0] = rn;
  int k = 0;
  for (k = 1; k <= m; ++k) {
    // w = L2 L1 A R1 R2 v_k
    const double2* src = W.V(k - 1);
    double2* a = W.tmp.as<double2>();
    double2* b = W.tmp2.as<double2>();
    if (R2) {
      MARIE_TRY((*R2)(src, a));
      src = a;
      std::swap(a, b);
    }
    if (R1) {
      MARIE_TRY((*R1)(src, a));
      src = a;
      std::swap(a, b);
    }
    double2* wk = W.V(k);
    if (!L1 && !L2) {
      MARIE_TRY(A(src, wk));
    } else {
      MARIE_TRY(A(src, a));
      src = a;
      std::swap(a, b);
      if (L1 && L2) {
        MARIE_TRY((*L1)(src, a));
        MARIE_TRY((*L2)(a, wk));
      } else {
        MARIE_TRY((L1 ? *L1 : *L2)(src, wk));
      }
    }
    double hn = 0;
    if (kc > 0) {
      std::vector<cd> bc;
      MARIE_TRY(W.dots(W.col(W.kmax - kc), kc, wk, bc));
      for (int i = 0; i < kc; ++i) B(i, k - 1) = bc[i];
      MARIE_TRY(W.update(W.col(W.kmax - kc), kc, bc, wk, &hn));
    }
    std::vector<cd> h;
    MARIE_TRY(W.dots(W.V(0), k, wk, h));
    MARIE_TRY(W.update(W.V(0), k, h, wk, &hn));
    for (int i = 0; i < k; ++i) H(i, k - 1) = h[i];
    H(k, k - 1) = hn;
    k_scale<<<grid_n(n), 256, 0, st>>>(wk, 1.0 / hn, wk, n);  // 0/0 as the reference on breakdown
    count_launch();
    MARIE_CUDA_TRY(cudaGetLastError());
    // rotate the new column and extend g
    const int kk = k - 1;
    for (int i = 0; i <= k; ++i) R(i, kk) = H(i, kk);
    for (int i = 0; i < kk; ++i) {
      const cd x = R(i, kk), y = R(i + 1, kk);
      R(i, kk) = gc[i] * x + gs[i] * y;
      R(i + 1, kk) = -std::conj(gs[i]) * x + gc[i] * y;
    }
    {
      const cd x = R(kk, kk);
      const double ax = std::abs(x), ay = std::abs(R(k, kk));
      if (ax == 0.0) {
        gc[kk] = 0;
        gs[kk] = 1.0;
      } else {
        const double rho = std::hypot(ax, ay);
        gc[kk] = ax / rho;
        gs[kk] = (x / ax) * ay / rho;
      }
      const cd gk = g[kk];
      g[kk] = gc[kk] * gk;
      g[k] = -std::conj(gs[kk]) * gk;
    }
    resvec.push_back(std::abs(g[k]));
    if (resvec.back() < tol) break;
  }
  if (k > m) k = m;
  k_out = k;
  // truncate to the k steps taken
  Mat Ht(k + 1, k), Bt(kc, k);
  for (int j = 0; j < k; ++j) {
    for (int i = 0; i <= k; ++i) Ht(i, j) = H(i, j);
    for (int i = 0; i < kc; ++i) Bt(i, j) = B(i, j);
  }
  H = Ht;
  B = Bt;
  return MARIE_OK;
}

// eigenvectors of M ordered by ascending |eigenvalue| (the sortrows of
// getHarmVecs1.m / getHarmVecs2.m), columns [first, first + count)
Mat sorted_vecs(const Mat& M, int first, int count) {
  std::vector<cd> vals;
  Mat vecs;
  dense::eig(M, vals, vecs);
  const int n = M.r;
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return std::abs(vals[a]) < std::abs(vals[b]); });
  Mat P(n, count);
  for (int j = 0; j < count; ++j)
    for (int i = 0; i < n; ++i) P(i, j) = vecs(i, order[first + j]);
  return P;
}

// getHarmVecs1.m: H is (m+1) x m
Mat harm_vecs1(const Mat& H, int m, int k) {
  Mat Hm(m, m);
  for (int j = 0; j < m; ++j)
    for (int i = 0; i < m; ++i) Hm(i, j) = H(i, j);
  Mat em(m, 1);
  em(m - 1, 0) = 1.0;
  const Mat f = dense::solve(dense::adj(Hm), em);  // last column of H_m^{-H}
  const cd h2 = H(m, m - 1) * H(m, m - 1);
  Mat Mh = Hm;
  for (int i = 0; i < m; ++i) Mh(i, m - 1) += h2 * f(i, 0);
  return sorted_vecs(Mh, 0, k);
}

// getHarmVecs2.m with CU = C'U (k x k) and VU = V'U ((m-k+1) x k)
Mat harm_vecs2(const Mat& H2, int m, int k, const Mat& CU, const Mat& VU) {
  const Mat Bm = dense::mul(dense::adj(H2), H2);
  Mat Wm(m + 1, m);
  for (int j = 0; j < k; ++j) {
    for (int i = 0; i < k; ++i) Wm(i, j) = CU(i, j);
    for (int i = 0; i < m + 1 - k; ++i) Wm(k + i, j) = VU(i, j);
  }
  for (int i = k; i < m; ++i) Wm(i, i) = 1.0;
  const Mat Am = dense::mul(dense::adj(H2), Wm);
  // eig(A, B) with B = H2' H2 Hermitian positive definite: eig(B \ A)
  return sorted_vecs(dense::solve(Bm, Am), m - k, k);
}

std::vector<cd> column(const Mat& M, int j) {
  std::vector<cd> c(M.r);
  for (int i = 0; i < M.r; ++i) c[i] = M(i, j);
  return c;
}

}  // namespace

int gmres_dr(marie_plan* p, const DevOp& A, const DevOp* L1, const DevOp* L2, const DevOp* R1, const DevOp* R2,
             const double2* b, long long n, int restart, double tol, int maxit, int ritz, const double2* x0,
             double2* x, GmresResult& out) {
  if (restart < 2) return set_error(MARIE_EINVAL, "pgmresDR needs restart >= 2");
  if (maxit < 0) return set_error(MARIE_EINVAL, "maxit must be >= 0");
  MARIE_TRACE("pgmresDR");
  // pgmresDR.m:55-60
  if (ritz < 1)
    ritz = std::min(10, (int)std::floor(restart / 2.0 + 0.5));
  else
    ritz = std::min(ritz, restart - 1);
  if (restart + ritz + 1 > DR_MAXCOLS)
    return set_error(MARIE_EINVAL, "pgmresDR: restart + ritz + 1 above %d is not built", DR_MAXCOLS);
  cudaStream_t st = p->stream;
  const size_t vb = (size_t)n * sizeof(double2);
  DrWork W;
  MARIE_TRY(W.init(p, n, restart, ritz));
  DBuf rbuf, bpb, xa;
  MARIE_TRY(rbuf.alloc(vb, st));
  MARIE_TRY(bpb.alloc(vb, st));
  MARIE_TRY(xa.alloc(vb, st));
  double2* r = rbuf.as<double2>();
  double2* xacc = xa.as<double2>();
  // r = b - A x0 (A x0 = 0 for a zero x0)
  double x0n = 0;
  if (x0) MARIE_TRY(dev_norm2(p, x0, n, &x0n));
  if (x0 && x0n > 0) {
    MARIE_TRY(A(x0, r));
    MARIE_TRY(W.sub(b, r));
  } else {
    MARIE_CUDA_TRY(cudaMemcpyAsync(r, b, vb, cudaMemcpyDeviceToDevice, st));
  }
  MARIE_CUDA_TRY(cudaMemcpyAsync(bpb.p, b, vb, cudaMemcpyDeviceToDevice, st));
  for (const DevOp* L : {L1, L2}) {
    if (!L) continue;
    MARIE_TRY((*L)(r, W.tmp.as<double2>()));
    MARIE_CUDA_TRY(cudaMemcpyAsync(r, W.tmp.p, vb, cudaMemcpyDeviceToDevice, st));
    MARIE_TRY((*L)(bpb.as<double2>(), W.tmp.as<double2>()));
    MARIE_CUDA_TRY(cudaMemcpyAsync(bpb.p, W.tmp.p, vb, cudaMemcpyDeviceToDevice, st));
  }
  double bnorm = 0, rn0 = 0;
  MARIE_TRY(dev_norm2(p, bpb.as<double2>(), n, &bnorm));
  MARIE_TRY(dev_norm2(p, r, n, &rn0));
  out = GmresResult();
  if (bnorm == 0) {
    // zero right-hand side: x = x0 (zero) at once instead of the reference's 0/0
    if (x0 && x0n > 0)
      MARIE_CUDA_TRY(cudaMemcpyAsync(x, x0, vb, cudaMemcpyDeviceToDevice, st));
    else
      MARIE_CUDA_TRY(cudaMemsetAsync(x, 0, vb, st));
    MARIE_CUDA_TRY(cudaStreamSynchronize(st));
    out.flag = 0;
    out.relres = 0;
    out.resvec.push_back(0.0);
    return MARIE_OK;
  }
  out.resvec.push_back(rn0 / bnorm);
  int outit = 0, pk = 0;
  std::vector<double> rin;
  Mat H, Bm;
  // first cycle: plain GMRES(m)
  MARIE_TRY(dr_cycle(W, A, L1, L2, R1, R2, r, 0, tol * bnorm, H, Bm, pk, rin));
  for (double v : rin) out.resvec.push_back(v / bnorm);
  {
    std::vector<cd> vr;
    MARIE_TRY(W.dots(W.V(0), pk + 1, r, vr));
    const std::vector<cd> y = dense::lstsq(H, vr);
    MARIE_TRY(W.combine(W.V(0), pk, y, xacc));
    MARIE_TRY(W.combine(W.V(0), pk + 1, dense::mulv(H, y), W.tmp.as<double2>()));
    MARIE_TRY(W.sub(r, W.tmp.as<double2>()));  // tmp = r - V H y
    MARIE_CUDA_TRY(cudaMemcpyAsync(r, W.tmp.p, vb, cudaMemcpyDeviceToDevice, st));
  }
  int kc = 0;
  auto rebase = [&](const Mat& P, const Mat& Hx, const double2* Ubase, int nU, const double2* Vbase, int nV,
                    const double2* CVbase, int nCV) -> int {
    // U = [Ubase(:, :nU) Vbase(:, :nV)] P ; [Q, R] = qr(Hx P, 0) ; C = CVbase Q ; U = U / R
    const int kn = P.c;
    for (int j = 0; j < kn; ++j) {
      std::vector<cd> pu(P.r);
      for (int i = 0; i < P.r; ++i) pu[i] = P(i, j);
      std::vector<cd> pa(pu.begin(), pu.begin() + nU), pb(pu.begin() + nU, pu.end());
      if (nU > 0) {
        MARIE_TRY(W.combine(Ubase, nU, pa, W.Unewcol(j)));
        MARIE_TRY(W.combine(Vbase, nV, pb, W.tmp.as<double2>()));
        MARIE_TRY(W.add(W.tmp.as<double2>(), W.Unewcol(j)));
      } else {
        MARIE_TRY(W.combine(Vbase, nV, pb, W.Unewcol(j)));
      }
    }
    Mat Q, R;
    dense::qr_thin(dense::mul(Hx, P), Q, R);
    // C = CVbase Q into Ucol scratch first (C and V are read), then into place
    for (int j = 0; j < kn; ++j) MARIE_TRY(W.combine(CVbase, nCV, column(Q, j), W.Ucol(j)));
    for (int j = 0; j < kn; ++j)
      MARIE_CUDA_TRY(cudaMemcpyAsync(W.col(W.kmax - kn + j), W.Ucol(j), vb, cudaMemcpyDeviceToDevice, st));
    // U = Unew R^{-1}
    Mat Ri = dense::rdiv_upper(Mat::eye(kn), R);
    for (int j = 0; j < kn; ++j) MARIE_TRY(W.combine(W.Unewcol(0), kn, column(Ri, j), W.Ucol(j)));
    kc = kn;
    return MARIE_OK;
  };
  if (out.resvec.back() > tol) {
    const Mat P = harm_vecs1(H, pk, std::min(ritz, pk - 1));
    MARIE_TRY(rebase(P, H, nullptr, 0, W.V(0), pk, W.V(0), pk + 1));
  }
  while (out.resvec.back() > tol && outit < maxit) {
    ++outit;
    MARIE_TRY(dr_cycle(W, A, L1, L2, R1, R2, r, kc, tol * bnorm, H, Bm, pk, rin));
    for (double v : rin) out.resvec.push_back(v / bnorm);
    // D = diag(1 / ||U(:, i)||), U = U D
    Mat D(kc, kc);
    for (int i = 0; i < kc; ++i) {
      double d = 0;
      MARIE_TRY(dev_norm2(p, W.Ucol(i), n, &d));
      D(i, i) = 1.0 / d;
      k_scale<<<grid_n(n), 256, 0, st>>>(W.Ucol(i), 1.0 / d, W.Ucol(i), n);
      count_launch();
    }
    MARIE_CUDA_TRY(cudaGetLastError());
    // H2 = [D, B; 0, H]
    Mat H2(kc + pk + 1, kc + pk);
    for (int i = 0; i < kc; ++i) {
      H2(i, i) = D(i, i);
      for (int j = 0; j < pk; ++j) H2(i, kc + j) = Bm(i, j);
    }
    for (int j = 0; j < pk; ++j)
      for (int i = 0; i <= pk; ++i) H2(kc + i, kc + j) = H(i, j);
    const double2* CVb = W.col(W.kmax - kc);
    std::vector<cd> cr;
    MARIE_TRY(W.dots(CVb, kc + pk + 1, r, cr));
    const std::vector<cd> y = dense::lstsq(H2, cr);
    // x += [U V(:, :pk)] y
    std::vector<cd> yu(y.begin(), y.begin() + kc), yv(y.begin() + kc, y.end());
    MARIE_TRY(W.combine(W.Ucol(0), kc, yu, W.tmp.as<double2>()));
    MARIE_TRY(W.add(W.tmp.as<double2>(), xacc));
    MARIE_TRY(W.combine(W.V(0), pk, yv, W.tmp.as<double2>()));
    MARIE_TRY(W.add(W.tmp.as<double2>(), xacc));
    // r -= [C V] H2 y
    MARIE_TRY(W.combine(CVb, kc + pk + 1, dense::mulv(H2, y), W.tmp.as<double2>()));
    MARIE_TRY(W.sub(r, W.tmp.as<double2>()));
    MARIE_CUDA_TRY(cudaMemcpyAsync(r, W.tmp.p, vb, cudaMemcpyDeviceToDevice, st));
    if (out.resvec.back() > tol) {
      // C'U and V'U for getHarmVecs2
      Mat CU(kc, kc), VU(pk + 1, kc);
      for (int j = 0; j < kc; ++j) {
        std::vector<cd> d;
        MARIE_TRY(W.dots(CVb, kc + pk + 1, W.Ucol(j), d));
        for (int i = 0; i < kc; ++i) CU(i, j) = d[i];
        for (int i = 0; i <= pk; ++i) VU(i, j) = d[kc + i];
      }
      const Mat P = harm_vecs2(H2, pk + kc, kc, CU, VU);
      MARIE_TRY(rebase(P, H2, W.Ucol(0), kc, W.V(0), pk, CVb, kc + pk + 1));
    }
  }
  // x = x0 + R1 R2 xacc
  const double2* src = xacc;
  double2* a = W.tmp.as<double2>();
  double2* bb = W.tmp2.as<double2>();
  if (R2) {
    MARIE_TRY((*R2)(src, a));
    src = a;
    std::swap(a, bb);
  }
  if (R1) {
    MARIE_TRY((*R1)(src, a));
    src = a;
  }
  MARIE_CUDA_TRY(cudaMemcpyAsync(x, src, vb, cudaMemcpyDeviceToDevice, st));
  if (x0 && x0n > 0) MARIE_TRY(W.add(x0, x));
  out.iter[0] = pk;
  out.iter[1] = outit;
  // true residual
  MARIE_TRY(A(x, W.tmp.as<double2>()));
  MARIE_TRY(W.sub(b, W.tmp.as<double2>()));
  double tr = 0, bn = 0;
  MARIE_TRY(dev_norm2(p, W.tmp.as<double2>(), n, &tr));
  MARIE_TRY(dev_norm2(p, b, n, &bn));
  out.relres = tr / bn;
  out.flag = out.relres <= tol ? 0 : 1;
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  return MARIE_OK;
}

}  // namespace marie

using namespace marie;

extern "C" int marie_pgmres_dr(marie_plan* p, marie_op_fn A, void* A_ctx, const double* b, int64_t n, int restart,
                               double tol, int maxit, int ritz, marie_op_fn L1, void* L1_ctx, marie_op_fn L2,
                               void* L2_ctx, marie_op_fn R1, void* R1_ctx, marie_op_fn R2, void* R2_ctx,
                               const double* x0, double* x, int* flag, double* relres, int* iter, double* resvec,
                               int64_t resvec_cap, int64_t* resvec_len) {
  if (!p || !b || !x || n < 1) return set_error(MARIE_EINVAL, "NULL argument or n < 1");
  auto wrap = [p](marie_op_fn f, void* ctx, long long nn) -> DevOp {
    return [p, f, ctx, nn](const double2* xi, double2* yo) -> int {
      MARIE_CUDA_TRY(cudaStreamSynchronize(p->stream));
      const int s = f(ctx, reinterpret_cast<const double*>(xi), reinterpret_cast<double*>(yo), nn);
      if (s != MARIE_OK) return set_error(s, "user operator returned status %d", s);
      return MARIE_OK;
    };
  };
  DevOp opA, oL1, oL2, oR1, oR2;
  if (A)
    opA = wrap(A, A_ctx, n);
  else
    MARIE_TRY(bound_operator(p, n, &opA));  // NULL A: the plan's bound mv_AN
  if (L1) oL1 = wrap(L1, L1_ctx, n);
  if (L2) oL2 = wrap(L2, L2_ctx, n);
  if (R1) oR1 = wrap(R1, R1_ctx, n);
  if (R2) oR2 = wrap(R2, R2_ctx, n);
  const size_t bytes = (size_t)n * sizeof(double2);
  DBuf tb, tx0, txo;
  const void *b_d, *x0_d = nullptr;
  void* x_d;
  MARIE_TRY(stage_in(b, bytes, p->stream, tb, &b_d));
  if (x0) MARIE_TRY(stage_in(x0, bytes, p->stream, tx0, &x0_d));
  MARIE_TRY(stage_out(x, bytes, p->stream, txo, &x_d));
  GmresResult res;
  MARIE_TRY(gmres_dr(p, opA, L1 ? &oL1 : nullptr, L2 ? &oL2 : nullptr, R1 ? &oR1 : nullptr, R2 ? &oR2 : nullptr,
                     (const double2*)b_d, n, restart, tol, maxit, ritz, (const double2*)x0_d, (double2*)x_d, res));
  MARIE_TRY(finish_out(x, x_d, bytes, p->stream));
  MARIE_CUDA_TRY(cudaStreamSynchronize(p->stream));
  if (flag) *flag = res.flag;
  if (relres) *relres = res.relres;
  if (iter) {
    iter[0] = res.iter[0];
    iter[1] = res.iter[1];
  }
  const int64_t nr = (int64_t)res.resvec.size();
  if (resvec_len) *resvec_len = nr;
  if (resvec)
    for (int64_t i = 0; i < nr && i < resvec_cap; ++i) resvec[i] = res.resvec[i];
  return check_kernel_status(p);
}
