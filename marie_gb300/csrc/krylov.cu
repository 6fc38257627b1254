// Restarted GMRES on device vectors with the semantics of the reference's
// pgmres / pgmres_iter (src_numeric/src_iterative/pgmres.m:70-181,
// pgmres_iter.m:22-150): classical Gram-Schmidt (one pass), preconditioners as
// operator products, x0 = 0 unless given, the restart residual kept as V*res,
// and a true residual recomputed once at the end.
//
// Device side: the Krylov basis V (n x (m+1), FP64 complex, columns
// contiguous), the fused V^H w dot products and the fused w -= V h update with
// its norm.  All reductions are two-stage in a fixed order, so results are
// bitwise reproducible run to run.  Host side: the Hessenberg column, the
// complex Givens rotations and the small least-squares solve (FP64).
#include <cmath>
#include <complex>
#include <vector>

#include "plan.h"

namespace marie {

static constexpr int RED_BLOCKS = 304;  // 2 x 152 SMs
static constexpr int RED_THREADS = 256;

template <typename V> __device__ __forceinline__ V warp_sum(V v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
  }
  return v;
}
__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block-wide sum of a double2; result valid in thread 0
__device__ double2 block_sum(double2 v) {
  __shared__ double2 ws[32];
  v = warp_sum(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) ws[wid] = v;
  __syncthreads();
  double2 r = mk<double2>(0, 0);
  if (wid == 0) {
    const int nw = blockDim.x >> 5;
    r = lane < nw ? ws[lane] : mk<double2>(0, 0);
    r = warp_sum(r);
  }
  return r;
}

__device__ __forceinline__ void chunk_of(long long n, long long& i0, long long& i1) {
  const long long chunk = (n + gridDim.x - 1) / gridDim.x;
  i0 = blockIdx.x * chunk;
  i1 = i0 + chunk < n ? i0 + chunk : n;
}

// partial[j * G + b] = sum over block b's chunk of conj(V_j) * w, j < ncols
__global__ void __launch_bounds__(RED_THREADS)
k_dot_partials(const double2* __restrict__ Vb, long long ld, int ncols, const double2* __restrict__ w, long long n,
               double2* __restrict__ partial) {
  long long i0, i1;
  chunk_of(n, i0, i1);
  for (int c0 = 0; c0 < ncols; c0 += 4) {
    double2 acc[4] = {mk<double2>(0, 0), mk<double2>(0, 0), mk<double2>(0, 0), mk<double2>(0, 0)};
    const int nc = ncols - c0 < 4 ? ncols - c0 : 4;
    for (long long i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
      const double2 wv = w[i];
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (q < nc) {
          const double2 v = Vb[(c0 + q) * ld + i];
          acc[q].x += v.x * wv.x + v.y * wv.y;
          acc[q].y += v.x * wv.y - v.y * wv.x;
        }
    }
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const double2 s = block_sum(acc[q]);
      if (q < nc && threadIdx.x == 0) partial[(long long)(c0 + q) * gridDim.x + blockIdx.x] = s;
    }
  }
}

// out[j] = sum_b partial[j * G + b]; one block per column, fixed order
__global__ void k_reduce_cols(const double2* __restrict__ partial, int G, double2* __restrict__ out) {
  double2 acc = mk<double2>(0, 0);
  for (int b = threadIdx.x; b < G; b += blockDim.x) acc = cadd(acc, partial[(long long)blockIdx.x * G + b]);
  acc = block_sum(acc);
  if (threadIdx.x == 0) out[blockIdx.x] = acc;
}

// w -= V[:, :ncols] h ; partial[b] = sum |w|^2 over block chunk
__global__ void __launch_bounds__(RED_THREADS)
k_update_norm(const double2* __restrict__ Vb, long long ld, int ncols, const double2* __restrict__ h,
              double2* __restrict__ w, long long n, double* __restrict__ partial) {
  __shared__ double2 hs[128];
  for (int j = threadIdx.x; j < ncols; j += blockDim.x) hs[j] = h[j];
  __syncthreads();
  long long i0, i1;
  chunk_of(n, i0, i1);
  double acc = 0;
  for (long long i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    double2 v = w[i];
    for (int j = 0; j < ncols; ++j) v = csub(v, cmul(Vb[j * ld + i], hs[j]));
    w[i] = v;
    acc += v.x * v.x + v.y * v.y;
  }
  const double2 s = block_sum(mk<double2>(acc, 0));
  if (threadIdx.x == 0) partial[blockIdx.x] = s.x;
}

__global__ void k_norm_partials(const double2* __restrict__ x, long long n, double* __restrict__ partial) {
  long long i0, i1;
  chunk_of(n, i0, i1);
  double acc = 0;
  for (long long i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    const double2 v = x[i];
    acc += v.x * v.x + v.y * v.y;
  }
  const double2 s = block_sum(mk<double2>(acc, 0));
  if (threadIdx.x == 0) partial[blockIdx.x] = s.x;
}

__global__ void k_reduce_real(const double* __restrict__ partial, int G, double* __restrict__ out) {
  double2 acc = mk<double2>(0, 0);
  for (int b = threadIdx.x; b < G; b += blockDim.x) acc.x += partial[b];
  acc = block_sum(acc);
  if (threadIdx.x == 0) *out = acc.x;
}

// y = s * x (real s)
__global__ void k_scale(const double2* __restrict__ x, double s, double2* __restrict__ y, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = mk<double2>(x[i].x * s, x[i].y * s);
}
// y = x - y
__global__ void k_sub_from(const double2* __restrict__ x, double2* __restrict__ y, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = csub(x[i], y[i]);
}
// y += x
__global__ void k_add_to(const double2* __restrict__ x, double2* __restrict__ y, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = cadd(y[i], x[i]);
}
// y = V[:, :ncols] c   (c on device)
__global__ void k_combine(const double2* __restrict__ Vb, long long ld, int ncols, const double2* __restrict__ c,
                          double2* __restrict__ y, long long n) {
  __shared__ double2 cs[128];
  for (int j = threadIdx.x; j < ncols; j += blockDim.x) cs[j] = c[j];
  __syncthreads();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double2 v = mk<double2>(0, 0);
    for (int j = 0; j < ncols; ++j) v = cadd(v, cmul(Vb[j * ld + i], cs[j]));
    y[i] = v;
  }
}

static inline int grid_n(long long n) { return grid_stride_blocks(n, 8); }

int dev_norm2(marie_plan* p, const double2* x, long long n, double* out_host) {
  DBuf part, res;
  MARIE_TRY(part.alloc(RED_BLOCKS * sizeof(double), p->stream));
  MARIE_TRY(res.alloc(sizeof(double), p->stream));
  k_norm_partials<<<RED_BLOCKS, RED_THREADS, 0, p->stream>>>(x, n, part.as<double>());
  count_launch();
  k_reduce_real<<<1, RED_THREADS, 0, p->stream>>>(part.as<double>(), RED_BLOCKS, res.as<double>());
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  double h = 0;
  MARIE_CUDA_TRY(cudaMemcpyAsync(&h, res.p, sizeof(double), cudaMemcpyDeviceToHost, p->stream));
  MARIE_CUDA_TRY(cudaStreamSynchronize(p->stream));
  *out_host = std::sqrt(h);
  return MARIE_OK;
}

using cd = std::complex<double>;

namespace {
struct Work {
  marie_plan* p;
  long long n;
  int m;
  DBuf Vb, w, tmp, tmp2, dpart, npart, hdev, nrm, cdev;
  int init(marie_plan* pl, long long nn, int mm) {
    p = pl;
    n = nn;
    m = mm;
    cudaStream_t s = p->stream;
    MARIE_TRY(Vb.alloc((size_t)n * (m + 1) * sizeof(double2), s));
    MARIE_TRY(w.alloc((size_t)n * sizeof(double2), s));
    MARIE_TRY(tmp.alloc((size_t)n * sizeof(double2), s));
    MARIE_TRY(tmp2.alloc((size_t)n * sizeof(double2), s));
    MARIE_TRY(dpart.alloc((size_t)RED_BLOCKS * (m + 1) * sizeof(double2), s));
    MARIE_TRY(npart.alloc((size_t)RED_BLOCKS * sizeof(double), s));
    MARIE_TRY(hdev.alloc((size_t)(m + 2) * sizeof(double2), s));
    MARIE_TRY(nrm.alloc(sizeof(double), s));
    MARIE_TRY(cdev.alloc((size_t)(m + 2) * sizeof(double2), s));
    MARIE_TRY(ensure_pinned(p, 2 * (m + 2) + 2));
    return MARIE_OK;
  }
  double2* col(int j) { return Vb.as<double2>() + (long long)j * n; }
};

// apply op chain: y = op(x); an op may not work in place
int apply(const DevOp& op, const double2* x, double2* y) { return op(x, y); }

}  // namespace

// One restart cycle (pgmres_iter.m).  x is updated in place; r holds the
// (left-preconditioned) residual on entry and V*res on exit.
static int gmres_cycle(Work& W, const DevOp& A, const DevOp* L1, const DevOp* L2, const DevOp* R1, const DevOp* R2,
                       double2* x, double2* r, double tolabs, int& k_out, std::vector<double>& resvec_inner) {
  marie_plan* p = W.p;
  cudaStream_t st = p->stream;
  const long long n = W.n;
  const int m = W.m;
  double rnorm = 0;
  MARIE_TRY(dev_norm2(p, r, n, &rnorm));
  // V(:,1) = r / norm(r)   (division by zero gives Inf/NaN exactly as the reference)
  k_scale<<<grid_n(n), 256, 0, st>>>(r, 1.0 / rnorm, W.col(0), n);
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());

  std::vector<cd> H((size_t)(m + 1) * m, cd(0, 0));  // column-major (m+1) x m, unrotated
  std::vector<cd> R((size_t)(m + 1) * m, cd(0, 0));  // rotated copy
  std::vector<double> cs(m);
  std::vector<cd> sn(m);
  std::vector<cd> g(m + 1, cd(0, 0));
  g[0] = cd(rnorm, 0);
  std::vector<cd> y, res;
  resvec_inner.clear();
  int k = 0;
  for (k = 1; k <= m; ++k) {
    const double2* v = W.col(k - 1);
    const double2* src = v;
    double2* a_in = W.tmp.as<double2>();
    double2* a_out = W.tmp2.as<double2>();
    if (R1) {
      MARIE_TRY(apply(*R1, src, a_in));
      src = a_in;
    }
    if (R2) {
      double2* o = (src == a_in) ? a_out : a_in;
      MARIE_TRY(apply(*R2, src, o));
      src = o;
    }
    double2* wk = W.col(k);
    if (!L1 && !L2) {
      MARIE_TRY(apply(A, src, wk));
    } else {
      double2* o = (src == a_in) ? a_out : a_in;
      MARIE_TRY(apply(A, src, o));
      src = o;
      if (L1 && L2) {
        double2* o2 = (src == a_in) ? a_out : a_in;
        MARIE_TRY(apply(*L1, src, o2));
        MARIE_TRY(apply(*L2, o2, wk));
      } else {
        MARIE_TRY(apply(L1 ? *L1 : *L2, src, wk));
      }
    }
    // CGS: h = V(:,1:k)' w ; w -= V(:,1:k) h ; ||w||
    k_dot_partials<<<RED_BLOCKS, RED_THREADS, 0, st>>>(W.col(0), n, k, wk, n, W.dpart.as<double2>());
    count_launch();
    k_reduce_cols<<<k, RED_THREADS, 0, st>>>(W.dpart.as<double2>(), RED_BLOCKS, W.hdev.as<double2>());
    count_launch();
    k_update_norm<<<RED_BLOCKS, RED_THREADS, 0, st>>>(W.col(0), n, k, W.hdev.as<double2>(), wk, n,
                                                     W.npart.as<double>());
    count_launch();
    k_reduce_real<<<1, RED_THREADS, 0, st>>>(W.npart.as<double>(), RED_BLOCKS, W.nrm.as<double>());
    count_launch();
    MARIE_CUDA_TRY(cudaGetLastError());
    MARIE_CUDA_TRY(cudaMemcpyAsync(p->pinned, W.hdev.p, k * sizeof(double2), cudaMemcpyDeviceToHost, st));
    MARIE_CUDA_TRY(cudaMemcpyAsync(p->pinned + 2 * k, W.nrm.p, sizeof(double), cudaMemcpyDeviceToHost, st));
    MARIE_CUDA_TRY(cudaStreamSynchronize(st));
    const int kk = k - 1;
    for (int i = 0; i < k; ++i) H[(size_t)kk * (m + 1) + i] = cd(p->pinned[2 * i], p->pinned[2 * i + 1]);
    const double hn = std::sqrt(p->pinned[2 * k]);
    H[(size_t)kk * (m + 1) + k] = cd(hn, 0);
    // V(:,k+1) = w / H(k+1,k).  A zero norm (happy breakdown) leaves the column
    // at zero instead of 0/0; it only ever multiplies a zero residual entry.
    k_scale<<<grid_n(n), 256, 0, st>>>(wk, hn > 0 ? 1.0 / hn : 0.0, wk, n);
    count_launch();
    MARIE_CUDA_TRY(cudaGetLastError());
    // Givens update of the rotated column
    for (int i = 0; i <= k; ++i) R[(size_t)kk * (m + 1) + i] = H[(size_t)kk * (m + 1) + i];
    for (int i = 0; i < kk; ++i) {
      cd& a = R[(size_t)kk * (m + 1) + i];
      cd& b = R[(size_t)kk * (m + 1) + i + 1];
      const cd t = cs[i] * a + sn[i] * b;
      b = -std::conj(sn[i]) * a + cs[i] * b;
      a = t;
    }
    {
      cd& a = R[(size_t)kk * (m + 1) + kk];
      cd& b = R[(size_t)kk * (m + 1) + kk + 1];
      const double aa = std::abs(a), bb = std::abs(b);
      if (aa == 0.0) {
        cs[kk] = 0.0;
        sn[kk] = 1.0;
        a = b;
      } else {
        const double rho = std::hypot(aa, bb);
        const cd ph = a / aa;
        cs[kk] = aa / rho;
        sn[kk] = ph * std::conj(b) / rho;
        a = ph * rho;
      }
      b = 0.0;
      const cd gk = g[kk];
      g[kk] = cs[kk] * gk;
      g[kk + 1] = -std::conj(sn[kk]) * gk;
    }
    // y = R \ g(1:k), res = rhs - Hc*y with the unrotated Hc
    y.assign(k, cd(0, 0));
    for (int i = k - 1; i >= 0; --i) {
      cd s = g[i];
      for (int j = i + 1; j < k; ++j) s -= R[(size_t)j * (m + 1) + i] * y[j];
      y[i] = s / R[(size_t)i * (m + 1) + i];
    }
    res.assign(k + 1, cd(0, 0));
    res[0] = cd(rnorm, 0);
    for (int j = 0; j < k; ++j)
      for (int i = 0; i <= j + 1 && i <= k; ++i) res[i] -= H[(size_t)j * (m + 1) + i] * y[j];
    double rr = 0;
    for (auto& e : res) rr += std::norm(e);
    resvec_inner.push_back(std::sqrt(rr));
    if (resvec_inner.back() < tolabs) break;
  }
  if (k > m) k = m;
  k_out = k;
  // xupd = V(:,1:k) y ; right preconditioners ; x += xupd ; r = V(:,1:k+1) res
  double2* hp = reinterpret_cast<double2*>(p->pinned);
  for (int j = 0; j < k; ++j) hp[j] = mk<double2>(y[j].real(), y[j].imag());
  MARIE_CUDA_TRY(cudaMemcpyAsync(W.cdev.p, hp, k * sizeof(double2), cudaMemcpyHostToDevice, st));
  k_combine<<<grid_n(n), 256, 0, st>>>(W.col(0), n, k, W.cdev.as<double2>(), W.tmp.as<double2>(), n);
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  double2* upd = W.tmp.as<double2>();
  if (R1) {
    MARIE_TRY(apply(*R1, upd, W.tmp2.as<double2>()));
    upd = W.tmp2.as<double2>();
  }
  if (R2) {
    double2* o = upd == W.tmp.as<double2>() ? W.tmp2.as<double2>() : W.tmp.as<double2>();
    MARIE_TRY(apply(*R2, upd, o));
    upd = o;
  }
  k_add_to<<<grid_n(n), 256, 0, st>>>(upd, x, n);
  count_launch();
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  for (int j = 0; j <= k; ++j) hp[j] = mk<double2>(res[j].real(), res[j].imag());
  MARIE_CUDA_TRY(cudaMemcpyAsync(W.cdev.p, hp, (k + 1) * sizeof(double2), cudaMemcpyHostToDevice, st));
  k_combine<<<grid_n(n), 256, 0, st>>>(W.col(0), n, k + 1, W.cdev.as<double2>(), r, n);
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  return MARIE_OK;
}

int gmres(marie_plan* p, const DevOp& A, const DevOp* L1, const DevOp* L2, const DevOp* R1, const DevOp* R2,
          const double2* b, long long n, int restart, double tol, int maxit, const double2* x0, double2* x,
          GmresResult& out) {
  if (restart < 1) return set_error(MARIE_EINVAL, "restart must be >= 1");
  if (restart > 127) return set_error(MARIE_EINVAL, "restart must be <= 127");
  if (maxit < 0) return set_error(MARIE_EINVAL, "maxit must be >= 0");
  cudaStream_t st = p->stream;
  Work W;
  MARIE_TRY(W.init(p, n, restart));
  DBuf rbuf, bp, ax;
  MARIE_TRY(rbuf.alloc(n * sizeof(double2), st));
  MARIE_TRY(bp.alloc(n * sizeof(double2), st));
  MARIE_TRY(ax.alloc(n * sizeof(double2), st));
  double2* r = rbuf.as<double2>();
  // x = x0 ; r = b - A x0 when x0 has non-zeros, else r = b
  double x0n = 0;
  if (x0) MARIE_TRY(dev_norm2(p, x0, n, &x0n));
  if (x0 && x0n > 0) {
    MARIE_CUDA_TRY(cudaMemcpyAsync(x, x0, n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    MARIE_TRY(A(x, r));
    k_sub_from<<<grid_n(n), 256, 0, st>>>(b, r, n);
    count_launch();
  } else {
    MARIE_CUDA_TRY(cudaMemsetAsync(x, 0, n * sizeof(double2), st));
    MARIE_CUDA_TRY(cudaMemcpyAsync(r, b, n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
  }
  MARIE_CUDA_TRY(cudaMemcpyAsync(bp.p, b, n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
  if (L1) {
    MARIE_TRY((*L1)(r, W.tmp.as<double2>()));
    MARIE_CUDA_TRY(cudaMemcpyAsync(r, W.tmp.p, n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    MARIE_TRY((*L1)(bp.as<double2>(), W.tmp.as<double2>()));
    MARIE_CUDA_TRY(cudaMemcpyAsync(bp.p, W.tmp.p, n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
  }
  if (L2) {
    MARIE_TRY((*L2)(r, W.tmp.as<double2>()));
    MARIE_CUDA_TRY(cudaMemcpyAsync(r, W.tmp.p, n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    MARIE_TRY((*L2)(bp.as<double2>(), W.tmp.as<double2>()));
    MARIE_CUDA_TRY(cudaMemcpyAsync(bp.p, W.tmp.p, n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
  }
  double bnorm = 0, rn = 0;
  MARIE_TRY(dev_norm2(p, bp.as<double2>(), n, &bnorm));
  MARIE_TRY(dev_norm2(p, r, n, &rn));
  out.resvec.clear();
  out.resvec.push_back(rn / bnorm);
  int outit = 0, pk = 0;
  std::vector<double> inner;
  while (out.resvec.back() > tol && outit < maxit) {
    ++outit;
    MARIE_TRY(gmres_cycle(W, A, L1, L2, R1, R2, x, r, tol * bnorm, pk, inner));
    for (double v : inner) out.resvec.push_back(v / bnorm);
  }
  out.iter[0] = pk;
  out.iter[1] = outit;
  // true residual
  MARIE_TRY(A(x, ax.as<double2>()));
  k_sub_from<<<grid_n(n), 256, 0, st>>>(b, ax.as<double2>(), n);
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  double tr = 0, bn = 0;
  MARIE_TRY(dev_norm2(p, ax.as<double2>(), n, &tr));
  MARIE_TRY(dev_norm2(p, b, n, &bn));
  out.relres = tr / bn;
  out.flag = (out.relres <= tol) ? 0 : 1;
  return MARIE_OK;
}

}  // namespace marie

using namespace marie;

extern "C" int marie_pgmres(marie_plan* p, marie_op_fn A, void* A_ctx, const double* b, int64_t n, int restart,
                            double tol, int maxit, marie_op_fn L1, void* L1_ctx, marie_op_fn L2, void* L2_ctx,
                            marie_op_fn R1, void* R1_ctx, marie_op_fn R2, void* R2_ctx, const double* x0, double* x,
                            int* flag, double* relres, int* iter, double* resvec, int64_t resvec_cap,
                            int64_t* resvec_len) {
  if (!p || !b || !x || n < 1) return set_error(MARIE_EINVAL, "NULL argument or n < 1");
  MARIE_TRACE("pgmres");
  // User operators run outside the plan's stream: finish the plan's work
  // before handing them x; they return with y complete.
  auto wrap = [p](marie_op_fn f, void* ctx, long long nn) -> DevOp {
    return [p, f, ctx, nn](const double2* xi, double2* yo) -> int {
      MARIE_CUDA_TRY(cudaStreamSynchronize(p->stream));
      const int s = f(ctx, reinterpret_cast<const double*>(xi), reinterpret_cast<double*>(yo), nn);
      if (s != MARIE_OK) return set_error(s, "user operator returned status %d", s);
      return MARIE_OK;
    };
  };
  DevOp opA;
  if (A)
    opA = wrap(A, A_ctx, n);
  else
    MARIE_TRY(bound_operator(p, n, &opA));  // NULL A: the plan's bound mv_AN
  DevOp oL1, oL2, oR1, oR2;
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
  MARIE_TRY(gmres(p, opA, L1 ? &oL1 : nullptr, L2 ? &oL2 : nullptr, R1 ? &oR1 : nullptr, R2 ? &oR2 : nullptr,
                  (const double2*)b_d, n, restart, tol, maxit, (const double2*)x0_d, (double2*)x_d, res));
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
