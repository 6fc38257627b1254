// Batched, device-driven restarted GMRES for S systems that share one
// operator (many right-hand sides of one body), with the semantics of the
// reference's pgmres / pgmres_iter (src_numeric/src_iterative/pgmres.m:70-181,
// pgmres_iter.m:22-150):
//   * classical Gram-Schmidt, one pass (pgmres_iter.m:106-107);
//   * the least-squares problem Hc \ rhs solved at every step (here by complex
//     Givens rotations, then y by back-substitution) and the residual norm
//     taken as ||rhs - Hc y|| (pgmres_iter.m:116-120);
//   * a cycle stops at the first step whose residual is below tol*||b||;
//   * x += R(V y), r = V(:,1:k+1) res at the end of a cycle (:133-150);
//   * the true residual ||b - A x|| / ||b|| once at the end (pgmres.m:175).
// All systems advance in lockstep; a system that has stopped inside a cycle
// is skipped by every kernel (stop[s] < step), including the matvec passes.
// The Hessenberg update, the rotations and the small solve run on the device
// in FP64 (one warp per system), so a whole restart cycle has no host
// synchronisation and is replayed as one CUDA graph launch.
//
// The Krylov basis is stored and combined in FP64 (VB = double2, the
// reference's arithmetic) or, for the inner solves of mixed-precision
// refinement, in FP32 (VB = float2): the matvec then reads and writes FP32
// basis columns (BatchOp::apply32), and the dots, the Gram-Schmidt update and
// the basis combinations run as FP32 FMAs with FP64 reductions across
// threads, reading half the bytes.  Hessenberg entries, rotations, residual
// norms, the iterate and the restart residual stay FP64.
#include <cmath>
#include <type_traits>
#include <algorithm>
#include <vector>

#include "plan.h"

namespace marie {

// Row blocks per system of the reductions: a fixed count (2 per SM of a GB300),
// so that the two-stage sums, and with them the results, do not depend on the
// device the solve runs on.
static constexpr int BG = 152 * 2;
// row blocks of the dots and the update with an FP32 basis: these stream the
// basis at HBM speed rather than at the FP64 rate, so they want more loads in
// flight (four blocks per SM)
static constexpr int BG32 = 152 * 4;
static constexpr int BT = 256;

__device__ __forceinline__ double2 wsum2(double2 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
  }
  return v;
}
__device__ __forceinline__ double wsum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
// block sum, valid in thread 0
__device__ double2 bsum2(double2 v) {
  __shared__ double2 ws[32];
  v = wsum2(v);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) ws[wid] = v;
  __syncthreads();
  double2 r = mk<double2>(0, 0);
  if (wid == 0) {
    r = lane < (int)(blockDim.x >> 5) ? ws[lane] : mk<double2>(0, 0);
    r = wsum2(r);
  }
  return r;
}
__device__ __forceinline__ void rows_of(long long n, long long& i0, long long& i1) {
  const long long chunk = (n + gridDim.x - 1) / gridDim.x;
  i0 = blockIdx.x * chunk;
  i1 = i0 + chunk < n ? i0 + chunk : n;
}
__device__ __forceinline__ bool skip(const int* stop, int s, int step) { return stop[s] < step; }
__device__ __forceinline__ float fmaT(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fmaT(double a, double b, double c) { return __fma_rn(a, b, c); }

// ||X_s||^2 partials: X_s = X + s*xs
__global__ void __launch_bounds__(BT) kb_norm_part(const double2* __restrict__ X, long long xs, long long n,
                                                   const int* __restrict__ stop, int step, double* __restrict__ part) {
  const int s = blockIdx.y;
  if (stop && skip(stop, s, step)) return;
  const double2* x = X + s * xs;
  long long i0, i1;
  rows_of(n, i0, i1);
  double a = 0;
  for (long long i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    const double2 v = x[i];
    a = fma(v.x, v.x, fma(v.y, v.y, a));
  }
  const double2 r = bsum2(mk<double2>(a, 0));
  if (threadIdx.x == 0) part[(long long)s * gridDim.x + blockIdx.x] = r.x;
}

// norm[s] = sqrt(sum of partials), fixed order
__global__ void kb_norm_fin(const double* __restrict__ part, int G, const int* __restrict__ stop, int step,
                            double* __restrict__ out) {
  const int s = blockIdx.x;
  if (stop && skip(stop, s, step)) return;
  double a = 0;
  for (int b = threadIdx.x; b < G; b += 32) a += part[(long long)s * G + b];
  a = wsum(a);
  if (threadIdx.x == 0) out[s] = sqrt(a);
}

// Load unit of the streaming basis kernels: one complex for the FP64 basis,
// two for the FP32 basis (16-byte loads; its column stride ld is even and the
// padding rows [n, ld) hold zeros).  Accumulators are the basis precision.
template <typename VB> struct BUnit;
template <> struct BUnit<double2> {
  using U = double2;
  static constexpr int W = 1;
  __device__ __forceinline__ static U zero() { return mk<double2>(0, 0); }
  // acc += conj(v) w
  __device__ __forceinline__ static void dot(double2& acc, U v, U w) {
    acc.x = fmaT(v.x, w.x, fmaT(v.y, w.y, acc.x));
    acc.y = fmaT(v.x, w.y, fmaT(-v.y, w.x, acc.y));
  }
  // w -= v c
  __device__ __forceinline__ static void axpy(U& w, U v, double2 c) {
    w.x = fmaT(-v.x, c.x, fmaT(v.y, c.y, w.x));
    w.y = fmaT(-v.x, c.y, fmaT(-v.y, c.x, w.y));
  }
  __device__ __forceinline__ static double norm2(U w, double a) { return fmaT(w.x, w.x, fmaT(w.y, w.y, a)); }
  __device__ __forceinline__ static U scale(U w, double f) { return mk<double2>(w.x * f, w.y * f); }
};
template <> struct BUnit<float2> {
  using U = float4;  // (re, im) of rows 2i and 2i+1
  static constexpr int W = 2;
  __device__ __forceinline__ static U zero() { return make_float4(0.f, 0.f, 0.f, 0.f); }
  __device__ __forceinline__ static void dot(float2& acc, U v, U w) {
    acc.x = fmaT(v.x, w.x, fmaT(v.y, w.y, fmaT(v.z, w.z, fmaT(v.w, w.w, acc.x))));
    acc.y = fmaT(v.x, w.y, fmaT(-v.y, w.x, fmaT(v.z, w.w, fmaT(-v.w, w.z, acc.y))));
  }
  __device__ __forceinline__ static void axpy(U& w, U v, float2 c) {
    w.x = fmaT(-v.x, c.x, fmaT(v.y, c.y, w.x));
    w.y = fmaT(-v.x, c.y, fmaT(-v.y, c.x, w.y));
    w.z = fmaT(-v.z, c.x, fmaT(v.w, c.y, w.z));
    w.w = fmaT(-v.z, c.y, fmaT(-v.w, c.x, w.w));
  }
  __device__ __forceinline__ static float norm2(U w, float a) {
    return fmaT(w.x, w.x, fmaT(w.y, w.y, fmaT(w.z, w.z, fmaT(w.w, w.w, a))));
  }
  __device__ __forceinline__ static U scale(U w, float f) { return make_float4(w.x * f, w.y * f, w.z * f, w.w * f); }
};

__device__ __forceinline__ float2 wsum2f(float2 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
  }
  return v;
}
// warp sum of per-lane partial dots: FP64 lanes in FP64; FP32 lanes in FP32
// (a few more roundings on a 32-term sum), then FP64 across warps and blocks
__device__ __forceinline__ double2 warp_dot_sum(double2 v) { return wsum2(v); }
__device__ __forceinline__ double2 warp_dot_sum(float2 v) { return cvt<double2>(wsum2f(v)); }

// cycle start: V_s(:,0) = r_s / beta_s (zeros in the padding rows n..ld)
template <typename VB>
__global__ void kb_cycle_init(const double2* __restrict__ r, long long rs, VB* __restrict__ Vb, long long vs,
                              long long n, long long ld, const double* __restrict__ beta,
                              const int* __restrict__ stop) {
  const int s = blockIdx.y;
  if (stop[s] < 1) return;
  const double inv = 1.0 / beta[s];  // 0 -> Inf/NaN exactly as the reference's r / norm(r)
  const double2* x = r + s * rs;
  VB* v = Vb + s * vs;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < ld; i += (long long)gridDim.x * blockDim.x)
    v[i] = i < n ? cvt<VB>(mk<double2>(x[i].x * inv, x[i].y * inv)) : mk<VB>(0, 0);
}

// The block that finishes last (counted in cnt[s], reset by that block) runs
// the reduction over the blocks' partials: the usual fence-then-count
// pattern, no waiting.  The final sums have a fixed order whichever block
// runs them.
__device__ __forceinline__ bool last_block(unsigned* cnt) {
  __shared__ bool is_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) is_last = atomicAdd(cnt, 1u) == gridDim.x - 1;
  __syncthreads();
  if (is_last) {
    __threadfence();
    if (threadIdx.x == 0) *cnt = 0;
  }
  return is_last;
}

// One sweep over NC basis columns c0..c0+NC-1 (units of U, column stride nu):
// the block's partial sums of conj(V(:,j)) w, reduced in the block (warp sums,
// then warp partials in warp order by one thread per column: a fixed order).
// NC is a template argument so that a short last sweep issues no idle work.
template <int NC, typename VB>
__device__ __forceinline__ void kb_dot_sweep(const typename BUnit<VB>::U* __restrict__ V,
                                             const typename BUnit<VB>::U* __restrict__ w, long long nu,
                                             long long i0, long long i1, int c0, double2* __restrict__ part_s,
                                             double2 (*red)[8]) {
  using BU = BUnit<VB>;
  VB acc[NC];
#pragma unroll
  for (int q = 0; q < NC; ++q) acc[q] = mk<VB>(0, 0);
#pragma unroll 4
  for (long long i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    const typename BU::U wv = w[i];
#pragma unroll
    for (int q = 0; q < NC; ++q) BU::dot(acc[q], V[(long long)(c0 + q) * nu + i], wv);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NC; ++q) {
    const double2 r = warp_dot_sum(acc[q]);
    if (lane == 0) red[wid][q] = r;
  }
  __syncthreads();
  if (threadIdx.x < NC) {
    double2 r = red[0][threadIdx.x];
    for (int w2 = 1; w2 < BT / 32; ++w2) r = cadd(r, red[w2][threadIdx.x]);
    part_s[(long long)(c0 + threadIdx.x) * gridDim.x + blockIdx.x] = r;
  }
  __syncthreads();  // red is reused by the next sweep
}

// partial[s][j][b] = sum over block rows of conj(V_s(:,j)) w_s, j < k, w_s = V_s(:,k);
// h[s][j] = sum_b partial[s][j][b].  ld: column stride in complex elements.
template <typename VB>
__global__ void __launch_bounds__(BT) kb_dots(const VB* __restrict__ Vb, long long vs, long long ld, int k,
                                              const int* __restrict__ stop, double2* __restrict__ part,
                                              unsigned* __restrict__ cnt, double2* __restrict__ h, int hld) {
  using U = typename BUnit<VB>::U;
  const int s = blockIdx.y;
  if (skip(stop, s, k)) return;
  const long long nu = ld / BUnit<VB>::W;
  const U* V = reinterpret_cast<const U*>(Vb + s * vs);
  const U* w = V + (long long)k * nu;
  double2* part_s = part + (long long)s * 128 * gridDim.x;
  __shared__ double2 red[BT / 32][8];
  long long i0, i1;
  rows_of(nu, i0, i1);
  int c0 = 0;
  for (; c0 + 8 <= k; c0 += 8) kb_dot_sweep<8, VB>(V, w, nu, i0, i1, c0, part_s, red);
  switch (k - c0) {
    case 1: kb_dot_sweep<1, VB>(V, w, nu, i0, i1, c0, part_s, red); break;
    case 2: kb_dot_sweep<2, VB>(V, w, nu, i0, i1, c0, part_s, red); break;
    case 3: kb_dot_sweep<3, VB>(V, w, nu, i0, i1, c0, part_s, red); break;
    case 4: kb_dot_sweep<4, VB>(V, w, nu, i0, i1, c0, part_s, red); break;
    case 5: kb_dot_sweep<5, VB>(V, w, nu, i0, i1, c0, part_s, red); break;
    case 6: kb_dot_sweep<6, VB>(V, w, nu, i0, i1, c0, part_s, red); break;
    case 7: kb_dot_sweep<7, VB>(V, w, nu, i0, i1, c0, part_s, red); break;
    default: break;
  }
  // h[s][j] = sum_b part[s][j][b] by the last block, one warp per column
  if (!last_block(cnt + s)) return;
  const int G = gridDim.x, lane = threadIdx.x & 31;
  for (int j = threadIdx.x >> 5; j < k; j += BT / 32) {
    double2 a = mk<double2>(0, 0);
    for (int b = lane; b < G; b += 32) a = cadd(a, __ldcg(part_s + (long long)j * G + b));
    a = wsum2(a);
    if (lane == 0) h[(long long)s * hld + j] = a;
  }
}

struct GState {
  double2* H;    // [S][(m+1)*m] unrotated, column-major
  double2* R;    // [S][(m+1)*m] rotated
  double2* g;    // [S][m+1]
  double* cs;    // [S][m]
  double2* sn;   // [S][m]
  double2* y;    // [S][m]
  double2* res;  // [S][m+1]
  double* resv;  // [S][m]
  double* beta;  // [S]
  double* tolabs;  // [S]
  double* hn;    // [S]
  int* stop;     // [S]: last step of the current cycle (0 = not iterating)
};

__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  const double d = b.x * b.x + b.y * b.y;
  return mk<double2>((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

// One warp per system: store H column k, apply the previous rotations to it,
// form the new rotation and update g (pgmres_iter.m:106-125).  The LSQ
// residual norm ||rhs - Hc y|| equals |g(k+1)| after the rotations, so the
// per-step stop test needs no solve; y = R \ g and the explicit residual
// res = rhs - Hc y (which restarts the next cycle as V*res) are formed once,
// at the step that ends the cycle.
// Run by one full warp (lane = 0..31) for system s.
__device__ void givens_warp(const GState& G, int m, int k, const double2* __restrict__ h, int hld,
                            const double* __restrict__ npart, int NB, int s, int lane) {
  if (G.stop[s] < k) return;
  const int ld = m + 1;
  double2* H = G.H + (long long)s * ld * m;
  double2* R = G.R + (long long)s * ld * m;
  double2* g = G.g + (long long)s * ld;
  double* cs = G.cs + (long long)s * m;
  double2* sn = G.sn + (long long)s * m;
  double2* y = G.y + (long long)s * m;
  double2* res = G.res + (long long)s * ld;
  __shared__ double2 col_s[128], sn_s[128];
  __shared__ double cs_s[128];
  const int kk = k - 1;
  double nn = 0;
  for (int b = lane; b < NB; b += 32) nn += __ldcg(npart + (long long)s * NB + b);
  nn = wsum(nn);
  const double hnv = sqrt(nn);
  for (int i = lane; i < k; i += 32) {
    const double2 v = h[(long long)s * hld + i];
    H[kk * ld + i] = v;
    col_s[i] = v;
  }
  for (int i = lane; i < kk; i += 32) {
    cs_s[i] = cs[i];
    sn_s[i] = sn[i];
  }
  if (lane == 0) {
    H[kk * ld + k] = mk<double2>(hnv, 0);
    if (k == 1) g[0] = mk<double2>(G.beta[s], 0);
  }
  __syncwarp();
  double rn = 0;
  if (lane == 0) {
    double2* col = R + kk * ld;
    // the rotated entry i+1 is carried in a register along the chain
    double2 a = col_s[0];
    for (int i = 0; i < kk; ++i) {
      const double2 b = col_s[i + 1];
      const double c = cs_s[i];
      const double2 sv = sn_s[i];
      col[i] = cadd(cscale(a, c), cmul(sv, b));
      a = csub(cscale(b, c), cmulc(a, sv));  // -conj(s) a + c b
    }
    const double aa = hypot(a.x, a.y), bb = hnv;
    double c;
    double2 sv;
    if (aa == 0.0) {
      c = 0.0;
      sv = mk<double2>(1.0, 0.0);
      col[kk] = mk<double2>(bb, 0);
    } else {
      const double rho = hypot(aa, bb);
      const double2 ph = mk<double2>(a.x / aa, a.y / aa);
      c = aa / rho;
      sv = cscale(ph, bb / rho);  // ph * conj(b) / rho, b real
      col[kk] = cscale(ph, rho);
    }
    col[k] = mk<double2>(0, 0);
    cs[kk] = c;
    sn[kk] = sv;
    const double2 gk = g[kk];
    g[kk] = cscale(gk, c);
    const double2 gn = mk<double2>(-(sv.x * gk.x + sv.y * gk.y), -(sv.x * gk.y - sv.y * gk.x));  // -conj(s) g
    g[k] = gn;
    rn = hypot(gn.x, gn.y);
    G.resv[(long long)s * m + kk] = rn;
    G.hn[s] = hnv;
  }
  rn = __shfl_sync(0xffffffffu, rn, 0);
  if (!(rn < G.tolabs[s] || k == m)) return;
  __syncwarp();
  // back-substitution y = R(0:k,0:k) \ g(0:k)
  for (int i = k - 1; i >= 0; --i) {
    double2 p = mk<double2>(0, 0);
    for (int j = i + 1 + lane; j < k; j += 32) p = cadd(p, cmul(R[j * ld + i], y[j]));
    p = wsum2(p);
    if (lane == 0) y[i] = cdiv(csub(g[i], p), R[i * ld + i]);
    __syncwarp();
  }
  // res = rhs - Hc y with rhs = [beta; 0], Hc = H(0:k+1, 0:k)
  for (int i = lane; i <= k; i += 32) {
    double2 v = i == 0 ? mk<double2>(G.beta[s], 0) : mk<double2>(0, 0);
    for (int j = (i > 0 ? i - 1 : 0); j < k; ++j) v = csub(v, cmul(H[j * ld + i], y[j]));
    res[i] = v;
  }
  if (lane == 0) G.stop[s] = k;
}
// w_s -= V_s(:,0:k) h_s with w_s = V_s(:,k) ; partial norms of the new w_s,
// then the Givens step of the system (givens_warp) by the last block
template <typename VB>
__global__ void __launch_bounds__(BT) kb_update(VB* __restrict__ Vb, long long vs, long long ld, int k,
                                                const double2* __restrict__ h, int hld,
                                                const int* __restrict__ stop, double* __restrict__ part,
                                                unsigned* __restrict__ cnt, GState G, int m) {
  using BU = BUnit<VB>;
  using U = typename BU::U;
  using R = decltype(VB::x);
  const int s = blockIdx.y;
  if (skip(stop, s, k)) return;
  __shared__ VB hs[128];
  for (int j = threadIdx.x; j < k; j += blockDim.x) hs[j] = cvt<VB>(h[(long long)s * hld + j]);
  __syncthreads();
  const long long nu = ld / BU::W;
  U* V = reinterpret_cast<U*>(Vb + s * vs);
  U* w = V + (long long)k * nu;
  long long i0, i1;
  rows_of(nu, i0, i1);
  R a = 0;
  for (long long i = i0 + threadIdx.x; i < i1; i += blockDim.x) {
    U v = w[i];
#pragma unroll 8
    for (int j = 0; j < k; ++j) BU::axpy(v, V[(long long)j * nu + i], hs[j]);
    w[i] = v;
    a = BU::norm2(v, a);
  }
  const double2 r = bsum2(mk<double2>((double)a, 0));
  if (threadIdx.x == 0) part[(long long)s * gridDim.x + blockIdx.x] = r.x;
  if (!last_block(cnt + s)) return;
  if (threadIdx.x < 32) givens_warp(G, m, k, h, hld, part, gridDim.x, s, threadIdx.x);
}

// V_s(:,k) /= H(k+1,k)  (zero norm leaves a zero column instead of 0/0)
template <typename VB>
__global__ void kb_scale(VB* __restrict__ Vb, long long vs, long long ld, int k, const double* __restrict__ hn,
                         const int* __restrict__ stop) {
  using BU = BUnit<VB>;
  using U = typename BU::U;
  using R = decltype(VB::x);
  const int s = blockIdx.y;
  if (skip(stop, s, k)) return;
  const double h = hn[s];
  const R inv = (R)(h > 0 ? 1.0 / h : 0.0);
  const long long nu = ld / BU::W;
  U* w = reinterpret_cast<U*>(Vb + s * vs) + (long long)k * nu;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nu; i += (long long)gridDim.x * blockDim.x)
    w[i] = BU::scale(w[i], inv);
}

// out_s = V_s(:, 0:c_s) coef_s with c_s = stop[s] + extra (skipped when
// stop[s] < 1), summed in the basis precision; accumulate adds out_s (FP64)
template <typename VB>
__global__ void kb_combine(const VB* __restrict__ Vb, long long vs, long long n, long long ld,
                           const double2* __restrict__ coef, int cld, const int* __restrict__ stop, int extra,
                           double2* __restrict__ out, long long os, int accumulate) {
  const int s = blockIdx.y;
  const int k = stop[s];
  if (k < 1) return;
  const int nc = k + extra;
  __shared__ VB cf[129];
  for (int j = threadIdx.x; j < nc; j += blockDim.x) cf[j] = cvt<VB>(coef[(long long)s * cld + j]);
  __syncthreads();
  const VB* V = Vb + s * vs;
  double2* o = out + s * os;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    VB v = mk<VB>(0, 0);
    for (int j = 0; j < nc; ++j) {
      const VB b = V[(long long)j * ld + i];
      v.x = fmaT(b.x, cf[j].x, fmaT(-b.y, cf[j].y, v.x));
      v.y = fmaT(b.x, cf[j].y, fmaT(b.y, cf[j].x, v.y));
    }
    const double2 r = cvt<double2>(v);
    o[i] = accumulate ? cadd(o[i], r) : r;
  }
}

// y_s += x_s for systems in this cycle
__global__ void kb_add(const double2* __restrict__ x, long long xs, double2* __restrict__ y, long long ys, long long n,
                       const int* __restrict__ stop) {
  const int s = blockIdx.y;
  if (stop[s] < 1) return;
  const double2* a = x + s * xs;
  double2* b = y + s * ys;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = cadd(b[i], a[i]);
}

// y_s = b_s - y_s (all systems)
__global__ void kb_sub_from(const double2* __restrict__ b, long long bs, double2* __restrict__ y, long long ys,
                            long long n) {
  const int s = blockIdx.y;
  const double2* a = b + s * bs;
  double2* c = y + s * ys;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    c[i] = csub(a[i], c[i]);
}

static inline int gx(long long n) { return grid_stride_blocks(n, 4); }

// Closes one restart cycle on the device, as the host loop of gmres_batch does
// between cycles: per active system the outer count, the last step, the
// residual estimates appended to its history, its next activity (above its
// tolerance and below maxit) and its stop mark for the next cycle; a
// non-finite residual ends the loop with err = system + 1.  Sets the loop
// condition of the conditional graph node: another cycle while any system is
// active, never more than maxit cycles.
__global__ void kb_cycle_close(int S, int m, int maxit, const double* __restrict__ resv,
                               const double* __restrict__ bnorm, const double* __restrict__ tolr, int* __restrict__ stop,
                               int* __restrict__ act, int* __restrict__ outit, int* __restrict__ pk,
                               double* __restrict__ hist, int* __restrict__ hlen, long long cap, int* __restrict__ err,
                               int* __restrict__ ncycles, cudaGraphConditionalHandle cond) {
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  for (int s = threadIdx.x; s < S; s += blockDim.x) {
    if (!act[s]) continue;
    outit[s] += 1;
    const int k = stop[s];
    pk[s] = k;
    double last = 0;
    int len = hlen[s];
    for (int j = 0; j < k; ++j) {
      last = resv[(long long)s * m + j] / bnorm[s];
      if (len < cap) hist[(long long)s * cap + len++] = last;
    }
    hlen[s] = len;
    bool a;
    if (!isfinite(last)) {
      atomicCAS(err, 0, s + 1);
      a = false;
    } else {
      a = last > tolr[s] && outit[s] < maxit;
    }
    act[s] = a ? 1 : 0;
    stop[s] = a ? m : 0;
    if (a) atomicOr(&any, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const int c = ++*ncycles;
    cudaGraphSetConditional(cond, (any && *err == 0 && c < maxit) ? 1u : 0u);
  }
}

struct BatchWork {
  int S = 0, m = 0;
  long long n = 0, ld = 0;  // rows; column stride of the basis
  bool f32 = false;  // FP32 basis (t1f, t2f: FP32 work vectors of the preconditioner chains)
  int bg = BG;       // row blocks of kb_dots / kb_update
  DBuf V, t1, t2, t1f, t2f, r, part_d, part_n, h, H, R, g, cs, sn, y, res, resv, beta, tol, hn, stop, norms;
  DBuf cnt;  // [2][S] last-block counters of kb_dots and kb_update (zero between launches)
  GState gs{};
  cudaGraphExec_t exec = nullptr;
  long long graph_nodes = 0;
  // Two groups (Sa > 0): systems [0, Sa) step on the plan's stream, [Sa, S)
  // on st2; ev_a / ev_b order the groups' matvecs, ev_fork / ev_join bracket
  // the steps of a cycle.
  int Sa = 0;
  cudaStream_t st2 = nullptr;
  cudaEvent_t ev_a = nullptr, ev_b = nullptr, ev_fork = nullptr, ev_join = nullptr;
  ~BatchWork() {
    if (exec) cudaGraphExecDestroy(exec);
    for (cudaEvent_t e : {ev_a, ev_b, ev_fork, ev_join})
      if (e) cudaEventDestroy(e);
    if (st2) cudaStreamDestroy(st2);
  }
  int init_groups() {
    Sa = (S + 1) / 2;
    MARIE_CUDA_TRY(cudaStreamCreateWithFlags(&st2, cudaStreamNonBlocking));
    for (cudaEvent_t* e : {&ev_a, &ev_b, &ev_fork, &ev_join})
      MARIE_CUDA_TRY(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    return MARIE_OK;
  }
  int init(cudaStream_t st, int S_, int m_, long long n_, bool f32_) {
    S = S_;
    m = m_;
    n = n_;
    f32 = f32_;
    // FP32 basis columns padded to a multiple of 64 rows (16-byte loads of
    // row pairs); the padding stays zero: the matvec writes rows < n only and
    // the updates of zero rows give zeros
    ld = f32 ? (n + 63) / 64 * 64 : n;
    MARIE_TRY(V.alloc((size_t)S * (m + 1) * ld * (f32 ? sizeof(float2) : sizeof(double2)), st));
    if (f32) {
      MARIE_CUDA_TRY(cudaMemsetAsync(V.p, 0, (size_t)S * (m + 1) * ld * sizeof(float2), st));
      MARIE_TRY(t1f.alloc((size_t)S * n * sizeof(float2), st));
      MARIE_TRY(t2f.alloc((size_t)S * n * sizeof(float2), st));
    }
    MARIE_TRY(t1.alloc((size_t)S * n * sizeof(double2), st));
    MARIE_TRY(t2.alloc((size_t)S * n * sizeof(double2), st));
    bg = f32 ? BG32 : BG;
    MARIE_TRY(part_d.alloc((size_t)S * 128 * bg * sizeof(double2), st));
    MARIE_TRY(part_n.alloc((size_t)S * (bg > BG ? bg : BG) * sizeof(double), st));
    MARIE_TRY(h.alloc((size_t)S * (m + 1) * sizeof(double2), st));
    MARIE_TRY(H.alloc((size_t)S * (m + 1) * m * sizeof(double2), st));
    MARIE_TRY(R.alloc((size_t)S * (m + 1) * m * sizeof(double2), st));
    MARIE_TRY(g.alloc((size_t)S * (m + 1) * sizeof(double2), st));
    MARIE_TRY(cs.alloc((size_t)S * m * sizeof(double), st));
    MARIE_TRY(sn.alloc((size_t)S * m * sizeof(double2), st));
    MARIE_TRY(y.alloc((size_t)S * m * sizeof(double2), st));
    MARIE_TRY(res.alloc((size_t)S * (m + 1) * sizeof(double2), st));
    MARIE_TRY(resv.alloc((size_t)S * m * sizeof(double), st));
    MARIE_TRY(beta.alloc((size_t)S * sizeof(double), st));
    MARIE_TRY(tol.alloc((size_t)S * sizeof(double), st));
    MARIE_TRY(hn.alloc((size_t)S * sizeof(double), st));
    MARIE_TRY(stop.alloc((size_t)S * sizeof(int), st));
    MARIE_TRY(norms.alloc((size_t)S * sizeof(double), st));
    MARIE_TRY(cnt.alloc((size_t)2 * S * sizeof(unsigned), st));
    MARIE_CUDA_TRY(cudaMemsetAsync(cnt.p, 0, (size_t)2 * S * sizeof(unsigned), st));
    gs = GState{H.as<double2>(), R.as<double2>(), g.as<double2>(), cs.as<double>(), sn.as<double2>(),
                y.as<double2>(), res.as<double2>(), resv.as<double>(), beta.as<double>(), tol.as<double>(),
                hn.as<double>(), stop.as<int>()};
    return MARIE_OK;
  }
  long long vs() const { return (long long)(m + 1) * ld; }
};

// batched norms of X_s (stride xs) into host array
static int bnorms(marie_plan* p, BatchWork& W, const double2* X, long long xs, std::vector<double>& out) {
  cudaStream_t st = p->stream;
  kb_norm_part<<<dim3(BG, W.S), BT, 0, st>>>(X, xs, W.n, nullptr, 0, W.part_n.as<double>());
  kb_norm_fin<<<W.S, 32, 0, st>>>(W.part_n.as<double>(), BG, nullptr, 0, W.norms.as<double>());
  count_launch(2);
  MARIE_CUDA_TRY(cudaGetLastError());
  out.resize(W.S);
  MARIE_CUDA_TRY(cudaMemcpyAsync(out.data(), W.norms.p, W.S * sizeof(double), cudaMemcpyDeviceToHost, st));
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  return MARIE_OK;
}

// dst = L1 A R1 src for the basis columns (stride vs) of systems g0 ..
// g0 + Sg - 1 (src, dst point at system g0), FP64 or FP32 vectors
static int basis_matvec(BatchWork& W, const BatchOp& A, const BatchOp* L1, const BatchOp* R1, const double2* src,
                        double2* dst, int k, int g0, int Sg) {
  const long long n = W.n, vs = W.vs();
  const int* stop = W.stop.as<int>() + g0;
  double2* t1 = W.t1.as<double2>() + g0 * n;
  double2* t2 = W.t2.as<double2>() + g0 * n;
  long long ss = vs;
  if (R1) {
    MARIE_TRY(R1->apply(src, ss, t1, n, Sg, stop, k));
    src = t1;
    ss = n;
  }
  if (L1) {
    MARIE_TRY(A.apply(src, ss, t2, n, Sg, stop, k));
    return L1->apply(t2, n, dst, vs, Sg, stop, k);
  }
  return A.apply(src, ss, dst, vs, Sg, stop, k);
}
static int basis_matvec(BatchWork& W, const BatchOp& A, const BatchOp* L1, const BatchOp* R1, const float2* src,
                        float2* dst, int k, int g0, int Sg) {
  const long long n = W.n, vs = W.vs();
  const int* stop = W.stop.as<int>() + g0;
  float2* t1 = W.t1f.as<float2>() + g0 * n;
  float2* t2 = W.t2f.as<float2>() + g0 * n;
  long long ss = vs;
  if (R1) {
    MARIE_TRY(R1->apply32(src, ss, t1, n, Sg, stop, k));
    src = t1;
    ss = n;
  }
  if (L1) {
    MARIE_TRY(A.apply32(src, ss, t2, n, Sg, stop, k));
    return L1->apply32(t2, n, dst, vs, Sg, stop, k);
  }
  return A.apply32(src, ss, dst, vs, Sg, stop, k);
}

// Gram-Schmidt step k of systems g0 .. g0 + Sg - 1 on stream sm: dots,
// update (its last block runs the Givens step) and scale
template <typename VB>
static void group_gs(BatchWork& W, int g0, int Sg, int k, cudaStream_t sm) {
  const int S = W.S, m = W.m;
  const long long vs = W.vs(), ld = W.ld;
  VB* V = W.V.as<VB>() + g0 * vs;
  const int* stop = W.stop.as<int>() + g0;
  unsigned* cnt = W.cnt.as<unsigned>();
  double2* h = W.h.as<double2>() + (long long)g0 * (m + 1);
  GState gs = W.gs;
  gs.H += (long long)g0 * (m + 1) * m;
  gs.R += (long long)g0 * (m + 1) * m;
  gs.g += (long long)g0 * (m + 1);
  gs.cs += (long long)g0 * m;
  gs.sn += (long long)g0 * m;
  gs.y += (long long)g0 * m;
  gs.res += (long long)g0 * (m + 1);
  gs.resv += (long long)g0 * m;
  gs.beta += g0;
  gs.tolabs += g0;
  gs.hn += g0;
  gs.stop += g0;
  kb_dots<VB><<<dim3(W.bg, Sg), BT, 0, sm>>>(V, vs, ld, k, stop, W.part_d.as<double2>() + (long long)g0 * 128 * W.bg,
                                             cnt + g0, h, m + 1);
  kb_update<VB><<<dim3(W.bg, Sg), BT, 0, sm>>>(V, vs, ld, k, h, m + 1, stop,
                                               W.part_n.as<double>() + (long long)g0 * W.bg, cnt + S + g0, gs, m);
  kb_scale<VB><<<dim3(gx(ld / BUnit<VB>::W), Sg), 256, 0, sm>>>(V, vs, ld, k, W.hn.as<double>() + g0, stop);
  count_launch(3);
}

// The m steps of a cycle in two groups: group a's matvec, then group b's
// matvec on the second stream while group a's Gram-Schmidt runs, then group
// a's next matvec while group b's Gram-Schmidt runs, and so on.  The matvecs
// alternate (they share the plan's workspace); each group's Gram-Schmidt
// overlaps the other group's matvec.
template <typename VB>
static int steps_in_two_groups(marie_plan* p, BatchWork& W, const BatchOp& A, const BatchOp* L1, const BatchOp* R1) {
  const int Sa = W.Sa, Sb = W.S - W.Sa, m = W.m;
  const long long ld = W.ld, vs = W.vs();
  VB* Va = W.V.as<VB>();
  VB* Vb = Va + Sa * vs;
  cudaStream_t sa = p->stream, sb = W.st2;
  MARIE_CUDA_TRY(cudaEventRecord(W.ev_fork, sa));
  MARIE_CUDA_TRY(cudaStreamWaitEvent(sb, W.ev_fork, 0));
  int rc = MARIE_OK;
  cudaError_t ce = cudaSuccess;
  for (int k = 1; k <= m; ++k) {
    if (k > 1 && (ce = cudaStreamWaitEvent(sa, W.ev_b, 0)) != cudaSuccess) break;
    if ((rc = basis_matvec(W, A, L1, R1, Va + (k - 1) * ld, Va + k * ld, k, 0, Sa)) != MARIE_OK) break;
    if ((ce = cudaEventRecord(W.ev_a, sa)) != cudaSuccess) break;
    group_gs<VB>(W, 0, Sa, k, sa);
    if ((ce = cudaStreamWaitEvent(sb, W.ev_a, 0)) != cudaSuccess) break;
    p->stream = sb;  // the operators launch on the plan's stream
    rc = basis_matvec(W, A, L1, R1, Vb + (k - 1) * ld, Vb + k * ld, k, Sa, Sb);
    p->stream = sa;
    if (rc != MARIE_OK) break;
    if ((ce = cudaEventRecord(W.ev_b, sb)) != cudaSuccess) break;
    group_gs<VB>(W, Sa, Sb, k, sb);
  }
  p->stream = sa;
  // join the second stream back, also after an error (a capture in progress
  // cannot end with a stream left out)
  const cudaError_t e1 = cudaEventRecord(W.ev_join, sb);
  const cudaError_t e2 = cudaStreamWaitEvent(sa, W.ev_join, 0);
  if (rc != MARIE_OK) return rc;
  if (ce == cudaSuccess) ce = (e1 != cudaSuccess) ? e1 : e2;
  if (ce != cudaSuccess) return set_error(MARIE_ECUDA, "two-group GMRES steps: %s", cudaGetErrorString(ce));
  return MARIE_OK;
}

// one restart cycle for all systems with stop[s] = m (others stop[s] = 0)
template <typename VB>
static int cycle(marie_plan* p, BatchWork& W, const BatchOp& A, const BatchOp* L1, const BatchOp* R1, double2* X,
                 long long xs, double2* Rv, long long rs) {
  cudaStream_t st = p->stream;
  const int S = W.S, m = W.m;
  const long long n = W.n, ld = W.ld, vs = W.vs();
  VB* V = W.V.as<VB>();
  int* stop = W.stop.as<int>();
  kb_norm_part<<<dim3(BG, S), BT, 0, st>>>(Rv, rs, n, stop, 1, W.part_n.as<double>());
  kb_norm_fin<<<S, 32, 0, st>>>(W.part_n.as<double>(), BG, stop, 1, W.beta.as<double>());
  kb_cycle_init<VB><<<dim3(gx(ld), S), 256, 0, st>>>(Rv, rs, V, vs, n, ld, W.beta.as<double>(), stop);
  count_launch(3);
  if (W.Sa > 0) {
    MARIE_TRY(steps_in_two_groups<VB>(p, W, A, L1, R1));
  } else {
    for (int k = 1; k <= m; ++k) {
      // V(:,k) = L1 A R1 V(:,k-1), in the basis precision
      MARIE_TRY(basis_matvec(W, A, L1, R1, V + (long long)(k - 1) * ld, V + (long long)k * ld, k, 0, S));
      group_gs<VB>(W, 0, S, k, st);
    }
  }
  // x += R1(V y) ; r = V(:,1:k+1) res
  kb_combine<VB><<<dim3(gx(n), S), 256, 0, st>>>(V, vs, n, ld, W.y.as<double2>(), m, stop, 0, W.t1.as<double2>(), n,
                                                 0);
  count_launch();
  const double2* upd = W.t1.as<double2>();
  if (R1) {
    MARIE_TRY(R1->apply(upd, n, W.t2.as<double2>(), n, S, stop, 1));
    upd = W.t2.as<double2>();
  }
  kb_add<<<dim3(gx(n), S), 256, 0, st>>>(upd, n, X, xs, n, stop);
  kb_combine<VB><<<dim3(gx(n), S), 256, 0, st>>>(V, vs, n, ld, W.res.as<double2>(), m + 1, stop, 1, Rv, rs, 0);
  count_launch(2);
  MARIE_CUDA_TRY(cudaGetLastError());
  return MARIE_OK;
}

// Runs the remaining restart cycles of gmres_batch in one launch of a graph
// whose conditional WHILE node repeats {one cycle, kb_cycle_close}; the
// state the host loop keeps between cycles (activity, outer counts, last
// steps, residual histories) lives on the device and is copied back once.
// *ran = false (and nothing run) when the graph cannot be built here, e.g.
// a driver without conditional nodes, or a history longer than 4 M entries.
template <typename CycleFn, typename TolOf>
static int cycles_in_one_launch(marie_plan* p, BatchWork& W, CycleFn& one_cycle, int S, int m, int maxit,
                                std::vector<int>& active, std::vector<int>& outit, std::vector<int>& pk,
                                const std::vector<double>& bnorm, TolOf& tol_of, std::vector<GmresResult>& out,
                                bool* ran) {
  *ran = false;
  const long long cap = (long long)m * maxit;
  if (cap <= 0 || cap * S > (4LL << 20)) return MARIE_OK;
  cudaStream_t st = p->stream;
  DBuf d_act, d_outit, d_pk, d_hist, d_hlen, d_bn, d_tol, d_err, d_nc;
  MARIE_TRY(d_act.alloc(S * sizeof(int), st));
  MARIE_TRY(d_outit.alloc(S * sizeof(int), st));
  MARIE_TRY(d_pk.alloc(S * sizeof(int), st));
  MARIE_TRY(d_hist.alloc((size_t)S * cap * sizeof(double), st));
  MARIE_TRY(d_hlen.alloc(S * sizeof(int), st));
  MARIE_TRY(d_bn.alloc(S * sizeof(double), st));
  MARIE_TRY(d_tol.alloc(S * sizeof(double), st));
  MARIE_TRY(d_err.alloc(2 * sizeof(int), st));
  std::vector<double> tolr(S);
  for (int s = 0; s < S; ++s) tolr[s] = tol_of(s);
  MARIE_CUDA_TRY(cudaMemcpyAsync(d_act.p, active.data(), S * sizeof(int), cudaMemcpyHostToDevice, st));
  MARIE_CUDA_TRY(cudaMemcpyAsync(d_outit.p, outit.data(), S * sizeof(int), cudaMemcpyHostToDevice, st));
  MARIE_CUDA_TRY(cudaMemcpyAsync(d_pk.p, pk.data(), S * sizeof(int), cudaMemcpyHostToDevice, st));
  MARIE_CUDA_TRY(cudaMemsetAsync(d_hlen.p, 0, S * sizeof(int), st));
  MARIE_CUDA_TRY(cudaMemcpyAsync(d_bn.p, bnorm.data(), S * sizeof(double), cudaMemcpyHostToDevice, st));
  MARIE_CUDA_TRY(cudaMemcpyAsync(d_tol.p, tolr.data(), S * sizeof(double), cudaMemcpyHostToDevice, st));
  MARIE_CUDA_TRY(cudaMemsetAsync(d_err.p, 0, 2 * sizeof(int), st));
  int* err = d_err.as<int>();
  int* ncyc = err + 1;
  // build: graph -> WHILE node (condition 1 at every launch) -> body captured
  cudaGraph_t g = nullptr;
  cudaGraphExec_t exec = nullptr;
  size_t body_nodes = 0;
  auto fail = [&]() {
    cudaGetLastError();
    if (exec) cudaGraphExecDestroy(exec);
    if (g) cudaGraphDestroy(g);
    return MARIE_OK;  // *ran stays false: the caller runs the per-cycle graphs
  };
  if (cudaGraphCreate(&g, 0) != cudaSuccess) return fail();
  cudaGraphConditionalHandle cond;
  if (cudaGraphConditionalHandleCreate(&cond, g, 1, cudaGraphCondAssignDefault) != cudaSuccess) return fail();
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = cond;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t node;
  if (cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp) != cudaSuccess) return fail();
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  if (cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return fail();
  const int s1 = one_cycle();
  kb_cycle_close<<<1, 128, 0, st>>>(S, m, maxit, W.resv.as<double>(), d_bn.as<double>(), d_tol.as<double>(),
                                    W.stop.as<int>(), d_act.as<int>(), d_outit.as<int>(), d_pk.as<int>(),
                                    d_hist.as<double>(), d_hlen.as<int>(), cap, err, ncyc, cond);
  cudaGraph_t captured = nullptr;
  const cudaError_t ec = cudaStreamEndCapture(st, &captured);
  if (s1 != MARIE_OK || ec != cudaSuccess) return fail();
  cudaGraphGetNodes(body, nullptr, &body_nodes);
  if (cudaGraphInstantiate(&exec, g, 0) != cudaSuccess) return fail();
  if (cudaGraphLaunch(exec, st) != cudaSuccess) return fail();
  *ran = true;
  count_graph_loop();
  int hc[2];
  std::vector<int> hlen(S), act2(S), outit2(S), pk2(S);
  std::vector<double> hist((size_t)S * cap);
  MARIE_CUDA_TRY(cudaMemcpyAsync(hc, err, 2 * sizeof(int), cudaMemcpyDeviceToHost, st));
  MARIE_CUDA_TRY(cudaMemcpyAsync(hlen.data(), d_hlen.p, S * sizeof(int), cudaMemcpyDeviceToHost, st));
  MARIE_CUDA_TRY(cudaMemcpyAsync(act2.data(), d_act.p, S * sizeof(int), cudaMemcpyDeviceToHost, st));
  MARIE_CUDA_TRY(cudaMemcpyAsync(outit2.data(), d_outit.p, S * sizeof(int), cudaMemcpyDeviceToHost, st));
  MARIE_CUDA_TRY(cudaMemcpyAsync(pk2.data(), d_pk.p, S * sizeof(int), cudaMemcpyDeviceToHost, st));
  MARIE_CUDA_TRY(cudaMemcpyAsync(hist.data(), d_hist.p, hist.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  const cudaError_t es = cudaStreamSynchronize(st);
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(g);
  MARIE_CUDA_TRY(es);
  count_launch((long long)hc[1] * (long long)body_nodes);
  for (int s = 0; s < S; ++s) {
    for (int j = 0; j < hlen[s]; ++j) out[s].resvec.push_back(hist[(size_t)s * cap + j]);
    active[s] = act2[s];
    outit[s] = outit2[s];
    pk[s] = pk2[s];
  }
  if (hc[0]) return set_error(MARIE_EBREAKDOWN, "non-finite GMRES residual (system %d, cycle %d)", hc[0] - 1,
                              outit[hc[0] - 1]);
  return MARIE_OK;
}

int gmres_batch(marie_plan* p, const BatchOp& A, const BatchOp* L1, const BatchOp* R1, const double2* B,
                long long bs, long long n, int S, int restart, double tol, int maxit, double2* X, long long xs,
                std::vector<GmresResult>& out, bool use_graph, const std::vector<int>* active_in,
                bool true_residual, bool fp32_basis, const std::vector<double>* tol_s) {
  if (restart < 1 || restart > 127) return set_error(MARIE_EINVAL, "restart must be in [1, 127]");
  if (tol_s && (int)tol_s->size() < S) return set_error(MARIE_EINVAL, "one tolerance per system");
  // the relative tolerance of system s
  auto tol_of = [&](int s) { return tol_s ? (*tol_s)[s] : tol; };
  if (S < 1) return set_error(MARIE_EINVAL, "need at least one system");
  cudaStream_t st = p->stream;
  BatchWork W;
  if (fp32_basis && (!A.apply32 || (L1 && !L1->apply32) || (R1 && !R1->apply32)))
    return set_error(MARIE_EINVAL, "an FP32 Krylov basis needs operators on FP32 vectors");
  MARIE_TRY(W.init(st, S, restart, n, fp32_basis));
  if (p->batch_groups == 2 && S >= 2) MARIE_TRY(W.init_groups());
  auto run_cycle = [&](double2* Xc, double2* Rc) {
    return W.f32 ? cycle<float2>(p, W, A, L1, R1, Xc, xs, Rc, n) : cycle<double2>(p, W, A, L1, R1, Xc, xs, Rc, n);
  };
  DBuf rb, bpb;
  MARIE_TRY(rb.alloc((size_t)S * n * sizeof(double2), st));
  double2* Rv = rb.as<double2>();
  const long long rs = n;
  // x0 = 0 ; r = b ; left preconditioning of r and b (pgmres.m:118-150)
  for (int s = 0; s < S; ++s) MARIE_CUDA_TRY(cudaMemsetAsync(X + s * xs, 0, n * sizeof(double2), st));
  for (int s = 0; s < S; ++s)
    MARIE_CUDA_TRY(cudaMemcpyAsync(Rv + s * rs, B + s * bs, n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
  std::vector<double> bnorm(S), rn(S);
  std::vector<int> all(S, 1);
  DBuf allstop;
  MARIE_TRY(allstop.alloc(S * sizeof(int), st));
  {
    std::vector<int> big(S, 1 << 30);
    MARIE_CUDA_TRY(cudaMemcpyAsync(allstop.p, big.data(), S * sizeof(int), cudaMemcpyHostToDevice, st));
  }
  if (L1) {
    MARIE_TRY(bpb.alloc((size_t)S * n * sizeof(double2), st));
    MARIE_TRY(L1->apply(Rv, rs, W.t1.as<double2>(), n, S, allstop.as<int>(), 1));
    MARIE_CUDA_TRY(cudaMemcpyAsync(Rv, W.t1.p, (size_t)S * n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    MARIE_CUDA_TRY(cudaMemcpyAsync(bpb.p, Rv, (size_t)S * n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
    MARIE_TRY(bnorms(p, W, bpb.as<double2>(), n, bnorm));
  } else {
    MARIE_TRY(bnorms(p, W, B, bs, bnorm));
  }
  MARIE_TRY(bnorms(p, W, Rv, rs, rn));
  out.assign(S, GmresResult());
  std::vector<int> outit(S, 0), pk(S, 0), active(S, 0);
  for (int s = 0; s < S; ++s) {
    const bool wanted = !active_in || (*active_in)[s];
    if (wanted && !std::isfinite(bnorm[s]))
      return set_error(MARIE_EBREAKDOWN, "non-finite right-hand side (system %d)", s);
    // b = 0 has the exact solution x = 0 (the reference's pgmres errors out)
    out[s].resvec.push_back(bnorm[s] > 0 ? rn[s] / bnorm[s] : 0.0);
    active[s] = (out[s].resvec.back() > tol_of(s) && maxit > 0 && wanted) ? 1 : 0;
  }
  std::vector<double> tolabs(S);
  for (int s = 0; s < S; ++s) tolabs[s] = tol_of(s) * bnorm[s];
  MARIE_CUDA_TRY(cudaMemcpyAsync(W.tol.p, tolabs.data(), S * sizeof(double), cudaMemcpyHostToDevice, st));
  std::vector<int> stop(S);
  std::vector<double> resv((size_t)S * restart);
  int cycles = 0;
  bool loop_tried = false;
  while (true) {
    bool any = false;
    for (int s = 0; s < S; ++s) {
      stop[s] = active[s] ? restart : 0;
      any = any || active[s];
    }
    if (!any) break;
    MARIE_TRACE("pgmres restart cycle");
    MARIE_CUDA_TRY(cudaMemcpyAsync(W.stop.p, stop.data(), S * sizeof(int), cudaMemcpyHostToDevice, st));
    if (use_graph && cycles >= 1 && !loop_tried && p->graph_refine) {
      // every remaining cycle in one graph launch (a conditional WHILE node
      // whose body is one cycle and its device-side close); the per-cycle
      // graphs below when the device or the sizes do not allow it
      loop_tried = true;
      bool ran = false;
      auto one_cycle = [&]() { return run_cycle(X, Rv); };
      MARIE_TRY(cycles_in_one_launch(p, W, one_cycle, S, restart, maxit, active, outit, pk, bnorm, tol_of, out,
                                     &ran));
      if (ran) break;
    }
    if (use_graph && cycles >= 1) {
      if (!W.exec) {
        cudaGraph_t graph;
        MARIE_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        const int s1 = run_cycle(X, Rv);
        cudaError_t e = cudaStreamEndCapture(st, &graph);
        MARIE_TRY(s1);
        MARIE_CUDA_TRY(e);
        size_t nodes = 0;
        cudaGraphGetNodes(graph, nullptr, &nodes);
        W.graph_nodes = (long long)nodes;
        e = cudaGraphInstantiate(&W.exec, graph, 0);
        cudaGraphDestroy(graph);
        MARIE_CUDA_TRY(e);
      }
      MARIE_CUDA_TRY(cudaGraphLaunch(W.exec, st));
      count_launch(W.graph_nodes);
    } else {
      MARIE_TRY(run_cycle(X, Rv));
    }
    ++cycles;
    MARIE_CUDA_TRY(cudaMemcpyAsync(stop.data(), W.stop.p, S * sizeof(int), cudaMemcpyDeviceToHost, st));
    MARIE_CUDA_TRY(cudaMemcpyAsync(resv.data(), W.resv.p, resv.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    MARIE_CUDA_TRY(cudaStreamSynchronize(st));
    for (int s = 0; s < S; ++s) {
      if (!active[s]) continue;
      ++outit[s];
      pk[s] = stop[s];
      for (int j = 0; j < stop[s]; ++j) out[s].resvec.push_back(resv[(size_t)s * restart + j] / bnorm[s]);
      if (!std::isfinite(out[s].resvec.back()))
        return set_error(MARIE_EBREAKDOWN, "non-finite GMRES residual (system %d, cycle %d)", s, outit[s]);
      active[s] = (out[s].resvec.back() > tol_of(s) && outit[s] < maxit) ? 1 : 0;
    }
  }
  for (int s = 0; s < S; ++s) {
    out[s].iter[0] = pk[s];
    out[s].iter[1] = outit[s];
  }
  if (!true_residual) {
    for (int s = 0; s < S; ++s) {
      out[s].relres = out[s].resvec.back();
      out[s].flag = out[s].relres <= tol_of(s) ? 0 : 1;
    }
    return MARIE_OK;
  }
  // true residuals (pgmres.m:175-180)
  {
    std::vector<int> big(S, 1 << 30);
    MARIE_CUDA_TRY(cudaMemcpyAsync(allstop.p, big.data(), S * sizeof(int), cudaMemcpyHostToDevice, st));
  }
  MARIE_TRY(A.apply(X, xs, W.t1.as<double2>(), n, S, allstop.as<int>(), 1));
  kb_sub_from<<<dim3(gx(n), S), 256, 0, st>>>(B, bs, W.t1.as<double2>(), n, n);
  count_launch();
  std::vector<double> tr, bn;
  MARIE_TRY(bnorms(p, W, W.t1.as<double2>(), n, tr));
  MARIE_TRY(bnorms(p, W, B, bs, bn));
  for (int s = 0; s < S; ++s) {
    out[s].iter[0] = pk[s];
    out[s].iter[1] = outit[s];
    out[s].relres = bn[s] > 0 ? tr[s] / bn[s] : 0.0;
    out[s].flag = out[s].relres <= tol_of(s) ? 0 : 1;
  }
  return MARIE_OK;
}


// ---------------------------------------------------------------------------
// Mixed-precision refinement in one graph launch
// ---------------------------------------------------------------------------
size_t batch_norm_scratch(int S) { return (size_t)S * BG; }

int batch_norms_dev(marie_plan* p, const double2* X, long long xs, long long n, int S, const int* mask, double* part,
                    double* out) {
  kb_norm_part<<<dim3(BG, S), BT, 0, p->stream>>>(X, xs, n, mask, 1, part);
  kb_norm_fin<<<S, 32, 0, p->stream>>>(part, BG, mask, 1, out);
  count_launch(2);
  MARIE_CUDA_TRY(cudaGetLastError());
  return MARIE_OK;
}

// rn = bn, relres = rn / bn: the state before the first refinement step
__global__ void kr_start(int S, const double* __restrict__ bn, double* __restrict__ rn, double* __restrict__ relres) {
  for (int s = threadIdx.x; s < S; s += blockDim.x) {
    rn[s] = bn[s];
    relres[s] = rn[s] / bn[s];
  }
}

// Opens a refinement step: act = relres > tol and, for the active systems,
// the inner tolerance min(0.5, max(0.5 tol ||b|| / ||r||, 1e-5)) (the
// comparisons of std::min / std::max, so that NaN propagates alike)
__global__ void kr_open(int S, double tol, const double* __restrict__ relres, const double* __restrict__ bn,
                        const double* __restrict__ rn, int* __restrict__ act, double* __restrict__ itol) {
  for (int s = threadIdx.x; s < S; s += blockDim.x) {
    const bool a = relres[s] > tol;
    act[s] = a ? 1 : 0;
    if (a) {
      double v = 0.5 * tol * bn[s] / rn[s];
      v = (v < 1e-5) ? 1e-5 : v;
      itol[s] = (v < 0.5) ? v : 0.5;
    }
  }
}

// Opens the inner GMRES of a step (x0 = 0, r = the step's residual): its
// active systems, absolute tolerances, first-cycle stop marks and counters,
// and the condition of the restart-cycle loop.  err: a wanted system with a
// non-finite right-hand side.
__global__ void kr_inner_open(int S, int m, int maxit, const int* __restrict__ act, const double* __restrict__ itol,
                              const double* __restrict__ bnorm, const double* __restrict__ rn0,
                              double* __restrict__ tolabs, int* __restrict__ stop, int* __restrict__ act_in,
                              int* __restrict__ outit, int* __restrict__ pk, int* __restrict__ err,
                              int* __restrict__ ncycles, cudaGraphConditionalHandle cond) {
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  for (int s = threadIdx.x; s < S; s += blockDim.x) {
    const bool wanted = act[s] != 0;
    if (wanted && !isfinite(bnorm[s])) atomicCAS(err, 0, s + 1);
    const double r0 = bnorm[s] > 0 ? rn0[s] / bnorm[s] : 0.0;
    const bool a = r0 > itol[s] && maxit > 0 && wanted;
    act_in[s] = a ? 1 : 0;
    stop[s] = a ? m : 0;
    tolabs[s] = itol[s] * bnorm[s];
    outit[s] = 0;
    pk[s] = 0;
    if (a) atomicOr(&any, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    *ncycles = 0;
    cudaGraphSetConditional(cond, (any && *err == 0) ? 1u : 0u);
  }
}

// Closes a refinement step for the systems it moved: the step's inner
// counts, the residual norm before (the scale of the step's inner history)
// and after, relres, the end of the step's history; another step while any
// system is above tol, no error occurred and fewer than max_refine ran.
__global__ void kr_close(int S, int MR, double tol, int max_refine, const int* __restrict__ act,
                         const int* __restrict__ outit, const int* __restrict__ pk, const double* __restrict__ rn_new,
                         const double* __restrict__ bn, const int* __restrict__ hlen, double* __restrict__ rn,
                         double* __restrict__ relres, int* __restrict__ inner_total, int* __restrict__ last_p,
                         int* __restrict__ step_end, double* __restrict__ step_scale, double* __restrict__ step_relres,
                         int* __restrict__ step_act, int* __restrict__ nstep, const int* __restrict__ err,
                         const int* __restrict__ ncycles, int* __restrict__ cycles_total,
                         cudaGraphConditionalHandle cond) {
  __shared__ int any, j;
  if (threadIdx.x == 0) {
    any = 0;
    j = *nstep;
  }
  __syncthreads();
  for (int s = threadIdx.x; s < S; s += blockDim.x) {
    const long long o = (long long)s * MR + j;
    if (act[s]) {
      step_scale[o] = rn[s];
      inner_total[s] += outit[s];
      last_p[s] = pk[s];
      rn[s] = rn_new[s];
      relres[s] = rn[s] / bn[s];
      step_end[o] = hlen[s];
      step_relres[o] = relres[s];
      step_act[o] = 1;
    } else {
      step_act[o] = 0;
    }
    if (relres[s] > tol) atomicOr(&any, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    *nstep = j + 1;
    *cycles_total += *ncycles;
    cudaGraphSetConditional(cond, (any && *err == 0 && j + 1 < max_refine) ? 1u : 0u);
  }
}

// Leaf nodes (no dependents) of a graph.
static int graph_leaves(cudaGraph_t g, std::vector<cudaGraphNode_t>& out) {
  size_t n = 0;
  MARIE_CUDA_TRY(cudaGraphGetNodes(g, nullptr, &n));
  std::vector<cudaGraphNode_t> all(n);
  MARIE_CUDA_TRY(cudaGraphGetNodes(g, all.data(), &n));
  out.clear();
  for (cudaGraphNode_t nd : all) {
    size_t d = 0;
    MARIE_CUDA_TRY(cudaGraphNodeGetDependentNodes(nd, nullptr, nullptr, &d));
    if (d == 0) out.push_back(nd);
  }
  return MARIE_OK;
}

// Kernel nodes of a graph (not counting the nodes inside conditional bodies).
static long long kernel_nodes(cudaGraph_t g) {
  size_t n = 0;
  if (cudaGraphGetNodes(g, nullptr, &n) != cudaSuccess) return 0;
  std::vector<cudaGraphNode_t> all(n);
  if (cudaGraphGetNodes(g, all.data(), &n) != cudaSuccess) return 0;
  long long k = 0;
  for (cudaGraphNode_t nd : all) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++k;
  }
  return k;
}

struct RefineJob::Impl {
  marie_plan* p = nullptr;
  BatchOp A32;
  BatchOp L1v, R1v;
  bool hasL1 = false, hasR1 = false;
  RefineOps ops;
  const double2* Bv = nullptr;
  double2* X = nullptr;
  long long n = 0, cap = 0;
  int S = 0, m = 0, maxit_in = 0, MR = 0;
  double tol = 0;
  BatchWork W;
  DBuf rr, dd, rv, bp, dv, iv, hs, sv;
  // views of the buffers
  double2 *Rr = nullptr, *D = nullptr, *Rv = nullptr, *bpb = nullptr;
  double *dp = nullptr, *bn = nullptr, *rn = nullptr, *rn_new = nullptr, *relres = nullptr, *itol = nullptr,
         *bnorm_in = nullptr, *rn_in = nullptr, *npart = nullptr, *hist = nullptr, *step_scale = nullptr,
         *step_relres = nullptr;
  int *ip = nullptr, *act = nullptr, *act_in = nullptr, *outit = nullptr, *pk = nullptr, *inner_total = nullptr,
      *last_p = nullptr, *hlen = nullptr, *allstop = nullptr, *err = nullptr, *ncyc = nullptr, *nstep = nullptr,
      *tcyc = nullptr, *step_end = nullptr, *step_act = nullptr;
  size_t nd = 0;
  long long nodes_step = 0, nodes_cycle = 0;
  const BatchOp* L1() const { return hasL1 ? &L1v : nullptr; }
  const BatchOp* R1() const { return hasR1 ? &R1v : nullptr; }
  int run_cycle() {
    return W.f32 ? cycle<float2>(p, W, A32, L1(), R1(), D, n, Rv, n) : cycle<double2>(p, W, A32, L1(), R1(), D, n, Rv, n);
  }
};

RefineJob::RefineJob() : d(new Impl) {}
RefineJob::~RefineJob() = default;

int RefineJob::prepare(marie_plan* p, const BatchOp& A32, const BatchOp* L1, const BatchOp* R1, const RefineOps& ops,
                       const double2* Bv, long long n, int S, int m, double tol, int maxit_in, int max_refine,
                       bool fp32_basis, double2* X, bool* ok) {
  *ok = false;
  if (S < 1 || m < 1 || m > 127 || max_refine < 1) return MARIE_OK;
  const long long cap = (long long)m * (maxit_in > 0 ? maxit_in : 1) * max_refine;  // inner history per system
  if (cap * S > (16LL << 20)) return MARIE_OK;
  if (fp32_basis && (!A32.apply32 || (L1 && !L1->apply32) || (R1 && !R1->apply32))) return MARIE_OK;
  Impl& J = *d;
  J.p = p;
  J.A32 = A32;
  if (L1) J.L1v = *L1;
  if (R1) J.R1v = *R1;
  J.hasL1 = L1 != nullptr;
  J.hasR1 = R1 != nullptr;
  J.ops = ops;
  J.Bv = Bv;
  J.X = X;
  J.n = n;
  J.cap = cap;
  J.S = S;
  J.m = m;
  J.maxit_in = maxit_in;
  J.MR = max_refine;
  J.tol = tol;
  cudaStream_t st = p->stream;
  // matvec workspaces at their largest, so that nothing is allocated while capturing
  MARIE_TRY(ensure_workspace(p, MARIE_FP64, S < p->nrhs_max ? S : p->nrhs_max, true));
  MARIE_TRY(J.W.init(st, S, m, n, fp32_basis));
  if (p->batch_groups == 2 && S >= 2) MARIE_TRY(J.W.init_groups());
  MARIE_TRY(J.rr.alloc((size_t)S * n * sizeof(double2), st));
  MARIE_TRY(J.dd.alloc((size_t)S * n * sizeof(double2), st));
  MARIE_TRY(J.rv.alloc((size_t)S * n * sizeof(double2), st));
  if (L1) MARIE_TRY(J.bp.alloc((size_t)S * n * sizeof(double2), st));
  // FP64 per system: bn rn rn_new relres itol bnorm_in rn_in, then the norm scratch
  J.nd = 7 * (size_t)S + batch_norm_scratch(S);
  MARIE_TRY(J.dv.alloc(J.nd * sizeof(double), st));
  // int per system: act act_in outit pk inner_total last_p hlen allstop, then err ncycles nstep cycles
  MARIE_TRY(J.iv.alloc((8 * (size_t)S + 4) * sizeof(int), st));
  MARIE_TRY(J.hs.alloc((size_t)S * cap * sizeof(double), st));
  // per system and step: scale, relres (FP64), end, act (int)
  MARIE_TRY(J.sv.alloc((size_t)S * max_refine * (2 * sizeof(double) + 2 * sizeof(int)), st));
  J.Rr = J.rr.as<double2>();
  J.D = J.dd.as<double2>();
  J.Rv = J.rv.as<double2>();
  J.bpb = J.bp.as<double2>();
  J.dp = J.dv.as<double>();
  J.bn = J.dp;
  J.rn = J.dp + S;
  J.rn_new = J.dp + 2 * S;
  J.relres = J.dp + 3 * S;
  J.itol = J.dp + 4 * S;
  J.bnorm_in = J.dp + 5 * S;
  J.rn_in = J.dp + 6 * S;
  J.npart = J.dp + 7 * S;
  J.ip = J.iv.as<int>();
  J.act = J.ip;
  J.act_in = J.ip + S;
  J.outit = J.ip + 2 * S;
  J.pk = J.ip + 3 * S;
  J.inner_total = J.ip + 4 * S;
  J.last_p = J.ip + 5 * S;
  J.hlen = J.ip + 6 * S;
  J.allstop = J.ip + 7 * S;
  J.err = J.ip + 8 * S;
  J.ncyc = J.err + 1;
  J.nstep = J.err + 2;
  J.tcyc = J.err + 3;
  J.hist = J.hs.as<double>();
  J.step_scale = J.sv.as<double>();
  J.step_relres = J.step_scale + (size_t)S * max_refine;
  J.step_end = reinterpret_cast<int*>(J.step_relres + (size_t)S * max_refine);
  J.step_act = J.step_end + (size_t)S * max_refine;
  // eager start: x = 0, r = b, ||b||, relres = 1, counters 0
  MARIE_CUDA_TRY(cudaMemsetAsync(X, 0, (size_t)S * n * sizeof(double2), st));
  MARIE_CUDA_TRY(cudaMemcpyAsync(J.Rr, Bv, (size_t)S * n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
  MARIE_TRY(batch_norms_dev(p, Bv, n, n, S, nullptr, J.npart, J.bn));
  kr_start<<<1, 128, 0, st>>>(S, J.bn, J.rn, J.relres);
  count_launch();
  MARIE_CUDA_TRY(cudaMemsetAsync(J.ip, 0, (8 * (size_t)S + 4) * sizeof(int), st));
  std::vector<int> big(S, 1 << 30);
  MARIE_CUDA_TRY(cudaMemcpyAsync(J.allstop, big.data(), S * sizeof(int), cudaMemcpyHostToDevice, st));
  MARIE_CUDA_TRY(cudaGetLastError());
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));  // the start is done before any graph of it launches
  *ok = true;
  return MARIE_OK;
}

// Adds WHILE(refinement step) { open ; WHILE(restart cycle) { cycle ; close } ;
// update ; close } to g, as a root node independent of g's other nodes.
bool RefineJob::add_to(cudaGraph_t g) {
  Impl& J = *d;
  marie_plan* p = J.p;
  cudaStream_t st = p->stream;
  const int S = J.S, m = J.m;
  const long long n = J.n;
  bool capturing = false;
  auto stop_capture = [&]() {
    if (capturing) {
      cudaGraph_t junk = nullptr;
      cudaStreamEndCapture(st, &junk);
      capturing = false;
    }
    cudaGetLastError();
    return false;
  };
  auto begin = [&](cudaGraph_t body, const cudaGraphNode_t* deps, size_t ndeps) {
    if (cudaStreamBeginCaptureToGraph(st, body, deps, nullptr, ndeps, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
      return false;
    capturing = true;
    return true;
  };
  auto end = [&]() {
    cudaGraph_t tmp = nullptr;
    capturing = false;
    return cudaStreamEndCapture(st, &tmp) == cudaSuccess;
  };
  cudaGraphConditionalHandle h_step, h_cycle;
  if (cudaGraphConditionalHandleCreate(&h_step, g, 1, cudaGraphCondAssignDefault) != cudaSuccess) return stop_capture();
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h_step;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t n_step;
  if (cudaGraphAddNode(&n_step, g, nullptr, nullptr, 0, &cp) != cudaSuccess) return stop_capture();
  cudaGraph_t b_step = cp.conditional.phGraph_out[0];
  if (cudaGraphConditionalHandleCreate(&h_cycle, b_step, 0, 0) != cudaSuccess) return stop_capture();
  // step, part 1: open, inner start (x0 = 0, r = the step's residual, left preconditioning), inner open
  if (!begin(b_step, nullptr, 0)) return stop_capture();
  {
    kr_open<<<1, 128, 0, st>>>(S, J.tol, J.relres, J.bn, J.rn, J.act, J.itol);
    count_launch();
    bool ok = cudaMemsetAsync(J.D, 0, (size_t)S * n * sizeof(double2), st) == cudaSuccess &&
              cudaMemcpyAsync(J.Rv, J.Rr, (size_t)S * n * sizeof(double2), cudaMemcpyDeviceToDevice, st) ==
                  cudaSuccess;
    if (ok && J.hasL1) {
      ok = J.L1v.apply(J.Rv, n, J.W.t1.as<double2>(), n, S, J.allstop, 1) == MARIE_OK &&
           cudaMemcpyAsync(J.Rv, J.W.t1.p, (size_t)S * n * sizeof(double2), cudaMemcpyDeviceToDevice, st) ==
               cudaSuccess &&
           cudaMemcpyAsync(J.bpb, J.Rv, (size_t)S * n * sizeof(double2), cudaMemcpyDeviceToDevice, st) == cudaSuccess;
    }
    ok = ok && batch_norms_dev(p, J.hasL1 ? J.bpb : J.Rr, n, n, S, nullptr, J.npart, J.bnorm_in) == MARIE_OK;
    ok = ok && batch_norms_dev(p, J.Rv, n, n, S, nullptr, J.npart, J.rn_in) == MARIE_OK;
    kr_inner_open<<<1, 128, 0, st>>>(S, m, J.maxit_in, J.act, J.itol, J.bnorm_in, J.rn_in, J.W.tol.as<double>(),
                                     J.W.stop.as<int>(), J.act_in, J.outit, J.pk, J.err, J.ncyc, h_cycle);
    count_launch();
    if (!end() || !ok) return stop_capture();
  }
  std::vector<cudaGraphNode_t> lv;
  if (graph_leaves(b_step, lv) != MARIE_OK) return stop_capture();
  cudaGraphNodeParams ip2 = {};
  ip2.type = cudaGraphNodeTypeConditional;
  ip2.conditional.handle = h_cycle;
  ip2.conditional.type = cudaGraphCondTypeWhile;
  ip2.conditional.size = 1;
  cudaGraphNode_t n_cycle;
  if (cudaGraphAddNode(&n_cycle, b_step, lv.data(), nullptr, lv.size(), &ip2) != cudaSuccess) return stop_capture();
  cudaGraph_t b_cycle = ip2.conditional.phGraph_out[0];
  // the restart cycle and its device-side close
  if (!begin(b_cycle, nullptr, 0)) return stop_capture();
  {
    const int rc = J.run_cycle();
    kb_cycle_close<<<1, 128, 0, st>>>(S, m, J.maxit_in, J.W.resv.as<double>(), J.bnorm_in, J.itol,
                                      J.W.stop.as<int>(), J.act_in, J.outit, J.pk, J.hist, J.hlen, J.cap, J.err,
                                      J.ncyc, h_cycle);
    count_launch();
    if (!end() || rc != MARIE_OK) return stop_capture();
  }
  // step, part 2: x += d, the FP64 residual and its norm, close
  if (!begin(b_step, &n_cycle, 1)) return stop_capture();
  {
    int rc = J.ops.add(J.D, J.X, J.act);
    if (rc == MARIE_OK) rc = J.ops.residual(J.X, J.Rr, J.act);
    if (rc == MARIE_OK) rc = batch_norms_dev(p, J.Rr, n, n, S, J.act, J.npart, J.rn_new);
    kr_close<<<1, 128, 0, st>>>(S, J.MR, J.tol, J.MR, J.act, J.outit, J.pk, J.rn_new, J.bn, J.hlen, J.rn, J.relres,
                                J.inner_total, J.last_p, J.step_end, J.step_scale, J.step_relres, J.step_act, J.nstep,
                                J.err, J.ncyc, J.tcyc, h_step);
    count_launch();
    if (!end() || rc != MARIE_OK) return stop_capture();
  }
  J.nodes_step = kernel_nodes(b_step);
  J.nodes_cycle = kernel_nodes(b_cycle);
  return true;
}

int RefineJob::finish(std::vector<GmresResult>& out) {
  Impl& J = *d;
  cudaStream_t st = J.p->stream;
  const int S = J.S, MR = J.MR;
  const long long cap = J.cap;
  std::vector<double> hd(J.nd), hsv((size_t)S * MR * 2);
  std::vector<int> hi(8 * (size_t)S + 4), hsi((size_t)S * MR * 2);
  MARIE_CUDA_TRY(cudaMemcpyAsync(hd.data(), J.dp, J.nd * sizeof(double), cudaMemcpyDeviceToHost, st));
  MARIE_CUDA_TRY(cudaMemcpyAsync(hi.data(), J.ip, hi.size() * sizeof(int), cudaMemcpyDeviceToHost, st));
  MARIE_CUDA_TRY(cudaMemcpyAsync(hsv.data(), J.step_scale, hsv.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
  MARIE_CUDA_TRY(cudaMemcpyAsync(hsi.data(), J.step_end, hsi.size() * sizeof(int), cudaMemcpyDeviceToHost, st));
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  const int e_code = hi[8 * S], steps = hi[8 * S + 2], cycles = hi[8 * S + 3];
  count_launch((long long)steps * J.nodes_step + (long long)cycles * J.nodes_cycle);
  if (e_code != 0) return set_error(MARIE_EBREAKDOWN, "non-finite GMRES residual (system %d)", e_code - 1);
  std::vector<double> hh;
  if (*std::max_element(hi.begin() + 6 * S, hi.begin() + 7 * S) > 0) {
    hh.resize((size_t)S * cap);
    MARIE_CUDA_TRY(cudaMemcpyAsync(hh.data(), J.hist, hh.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  }
  const double* h_bn = hd.data();
  const double* h_relres = hd.data() + 3 * S;
  const double* h_scale = hsv.data();
  const double* h_srel = hsv.data() + (size_t)S * MR;
  const int* h_end = hsi.data();
  const int* h_sact = hsi.data() + (size_t)S * MR;
  out.assign(S, GmresResult());
  for (int s = 0; s < S; ++s) {
    GmresResult& r = out[s];
    r.resvec.push_back(h_bn[s] / h_bn[s]);  // rn / bn before any step (rn = bn)
    int from = 0;
    for (int j = 0; j < steps && j < MR; ++j) {
      const size_t o = (size_t)s * MR + j;
      if (!h_sact[o]) continue;
      for (int i = from; i < h_end[o] && i < cap; ++i) r.resvec.push_back(hh[(size_t)s * cap + i] * h_scale[o] / h_bn[s]);
      from = h_end[o];
      r.resvec.push_back(h_srel[o]);
    }
    r.relres = h_relres[s];
    r.flag = r.relres <= J.tol ? 0 : 1;
    r.iter[0] = hi[5 * S + s];
    r.iter[1] = hi[4 * S + s];
  }
  return MARIE_OK;
}

int launch_refine_jobs(const std::vector<RefineJob*>& jobs, cudaStream_t st, bool* ran) {
  *ran = false;
  const long long launches0 = marie_launch_count();
  cudaGraph_t g = nullptr;
  cudaGraphExec_t exec = nullptr;
  auto fail = [&]() {
    cudaGetLastError();
    if (exec) cudaGraphExecDestroy(exec);
    if (g) cudaGraphDestroy(g);
    count_launch(launches0 - marie_launch_count());  // nothing of the captures ran
    return MARIE_OK;  // *ran stays false: the callers refine from the host
  };
  if (cudaGraphCreate(&g, 0) != cudaSuccess) return fail();
  for (RefineJob* j : jobs)
    if (!j->add_to(g)) return fail();
  if (cudaGraphInstantiate(&exec, g, 0) != cudaSuccess) return fail();
  count_launch(launches0 - marie_launch_count());  // the captures ran nothing; counted by finish()
  if (cudaGraphLaunch(exec, st) != cudaSuccess) return fail();
  *ran = true;
  count_graph_loop();
  const cudaError_t es = cudaStreamSynchronize(st);
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(g);
  MARIE_CUDA_TRY(es);
  return MARIE_OK;
}

int refine_batch_graph(marie_plan* p, const BatchOp& A32, const BatchOp* L1, const BatchOp* R1, const RefineOps& ops,
                       const double2* Bv, long long n, int S, int m, double tol, int maxit_in, int max_refine,
                       bool fp32_basis, double2* X, std::vector<GmresResult>& out, bool* ran) {
  *ran = false;
  RefineJob job;
  bool ok = false;
  MARIE_TRY(job.prepare(p, A32, L1, R1, ops, Bv, n, S, m, tol, maxit_in, max_refine, fp32_basis, X, &ok));
  if (!ok) return MARIE_OK;
  std::vector<RefineJob*> one{&job};
  MARIE_TRY(launch_refine_jobs(one, p->stream, ran));
  if (!*ran) return MARIE_OK;
  return job.finish(out);
}

}  // namespace marie
