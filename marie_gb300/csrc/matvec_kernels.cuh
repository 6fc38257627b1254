// The circulant-embedded J-VIE matvec as five FFT passes over the 2L x 2M x 2N
// padded grid, with the gather of the local DOF vector fused into the first
// pass and the crop, diagonal (Gram*Mr, Mc) scaling and DOF scatter fused into
// the last one.  The zero half of the padded input is never loaded, and only the
// N retained z-planes / M retained y-rows are written back after the inverse
// transforms.
//
//   xfwd : rows (y<M, z<N, c)      gather J via inv map, FFT_x (L of 2L non-zero)
//   cols : columns (kx, z<N, c)    FFT_y forward (M of 2M non-zero)
//   zmul : columns (kx, ky)        FFT_z (N of 2N) x3, 3x3 symmetric fN multiply,
//                                  inverse FFT_z, keep z<N        (in place)
//   cols : columns (kx, z<N, c)    inverse FFT_y, keep y<M
//   xinv : rows (y<M, z<N, c)      inverse FFT_x, keep x<L, epilogue, scatter
//
// Spectra layout (column-major like the reference's arrays, kx fastest):
//   A[c][z][y][kx]  : 3 x N x M  x 2L   (after xfwd / before xinv)
//   B[c][z][ky][kx] : 3 x N x 2M x 2L   (after the y transform)
// fN layout: fN[q][kz][ky][kx], q in [xx,xy,xz,yy,yz,zz], pre-scaled by 1/(8LMN)
// so that the inverse transforms need no normalisation.
#pragma once
#include "fft.cuh"

namespace marie {

struct Dims {
  int L, M, N, Lp, Mp, Np;
  long long V;  // L*M*N
};

// Epilogue: out[k] = A_k * J[k] - (conjout ? conj(v) : B_k * v)
struct Epilogue {
  const double2* a;  // per-DOF, or null -> a_s
  const double2* b;  // per-DOF, or null -> b_s
  double2 a_s, b_s;
  int conjout;
};
// Prologue: x_in[k] = (pre ? pre[k] : 1) * (conjin ? conj(J[k]) : J[k])
struct Prologue {
  const double2* pre;
  int conjin;
};

template <int N> struct RowCfg {
  static constexpr int T = FFT<float2, N, false>::T;
  static constexpr int S = (256 / T) < 2 ? 2 : (256 / T);
  static constexpr int THREADS = S * T;
};

// Stage the twiddle table (N entries) into shared memory.
template <typename V>
__device__ __forceinline__ void stage_twiddles(V* tw_s, const V* __restrict__ tw, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) tw_s[i] = tw[i];
}

// ---------------------------------------------------------------------------
// xfwd: gather + forward x transform.  grid.x = ceil(rows / S), grid.y = rhs
// ---------------------------------------------------------------------------
template <typename T, int NL>
__global__ void __launch_bounds__(RowCfg<NL>::THREADS)
k_xfwd(const double2* __restrict__ J, long long j_stride, const int* __restrict__ inv, Prologue pro,
       cplx<T>* __restrict__ A, long long a_stride, Dims d, const cplx<T>* __restrict__ tw) {
  using V = cplx<T>;
  using F = FFT<V, NL, false>;
  constexpr int S = RowCfg<NL>::S;
  constexpr int ES = S + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* tw_s = reinterpret_cast<V*>(smem_raw);
  V* buf = tw_s + NL;
  const int rows = d.M * d.N * 3;
  const int row0 = blockIdx.x * S;
  const double2* Jr = J + blockIdx.y * j_stride;
  const double2* prer = pro.pre;  // prologue coefficients are shared by all rhs
  stage_twiddles(tw_s, tw, NL);
  // gather: x fastest across threads
  for (int i = threadIdx.x; i < S * d.L; i += blockDim.x) {
    const int s = i / d.L, x = i - s * d.L;
    const int row = row0 + s;
    V val = mk<V>(0, 0);
    if (row < rows) {
      const long long g3 = (long long)row * d.L + x;  // row = y + M*(z + N*c)
      const int k = inv[g3];
      if (k >= 0) {
        double2 jv = Jr[k];
        if (pro.conjin) jv.y = -jv.y;
        if (prer) jv = cmul(prer[k], jv);
        val = cvt<V>(jv);
      }
    }
    buf[x * ES + s] = val;
  }
  __syncthreads();
  const int s = threadIdx.x % S, t = threadIdx.x / S;
  V reg[F::E];
  F::load_half(reg, buf + s, ES, t, d.L);
  F::run(reg, buf + s, ES, t, tw_s);
  __syncthreads();
  F::store(reg, buf + s, ES, t);
  __syncthreads();
  V* Ar = A + blockIdx.y * a_stride;
  for (int i = threadIdx.x; i < S * NL; i += blockDim.x) {
    const int ss = i / NL, kx = i - ss * NL;
    const int row = row0 + ss;
    if (row < rows) Ar[(long long)row * NL + kx] = buf[kx * ES + ss];
  }
}

// ---------------------------------------------------------------------------
// xinv: inverse x transform + crop + epilogue + scatter to DOFs.
// ---------------------------------------------------------------------------
template <typename T, int NL>
__global__ void __launch_bounds__(RowCfg<NL>::THREADS)
k_xinv(const cplx<T>* __restrict__ A, long long a_stride, const double2* __restrict__ J, long long j_stride,
       const int* __restrict__ inv, Epilogue ep, double2* __restrict__ out, long long o_stride, Dims d,
       const cplx<T>* __restrict__ tw) {
  using V = cplx<T>;
  using F = FFT<V, NL, true>;
  constexpr int S = RowCfg<NL>::S;
  constexpr int ES = S + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* tw_s = reinterpret_cast<V*>(smem_raw);
  V* buf = tw_s + NL;
  const int rows = d.M * d.N * 3;
  const int row0 = blockIdx.x * S;
  const V* Ar = A + blockIdx.y * a_stride;
  stage_twiddles(tw_s, tw, NL);
  for (int i = threadIdx.x; i < S * NL; i += blockDim.x) {
    const int s = i / NL, kx = i - s * NL;
    const int row = row0 + s;
    buf[kx * ES + s] = (row < rows) ? Ar[(long long)row * NL + kx] : mk<V>(0, 0);
  }
  __syncthreads();
  const int s = threadIdx.x % S, t = threadIdx.x / S;
  V reg[F::E];
  F::load(reg, buf + s, ES, t, NL);
  F::run(reg, buf + s, ES, t, tw_s);
  __syncthreads();
  F::store(reg, buf + s, ES, t);
  __syncthreads();
  const double2* Jr = J + blockIdx.y * j_stride;
  double2* outr = out + blockIdx.y * o_stride;
  for (int i = threadIdx.x; i < S * d.L; i += blockDim.x) {
    const int ss = i / d.L, x = i - ss * d.L;
    const int row = row0 + ss;
    if (row >= rows) continue;
    const long long g3 = (long long)row * d.L + x;
    const int k = inv[g3];
    if (k < 0) continue;
    const double2 v = cvt<double2>(buf[x * ES + ss]);
    const double2 jv = Jr[k];
    const double2 A_k = ep.a ? ep.a[k] : ep.a_s;
    double2 r = cmul(A_k, jv);
    if (ep.conjout) {
      r.x -= v.x;
      r.y += v.y;
    } else {
      const double2 B_k = ep.b ? ep.b[k] : ep.b_s;
      r = csub(r, cmul(B_k, v));
    }
    outr[k] = r;
  }
}

// ---------------------------------------------------------------------------
// cols: transform along the middle (y) axis for S consecutive kx columns.
//   in [kx + Lp*y + in_w*w], y < n_in      out [kx + Lp*y + out_w*w], y < n_out
// grid.x = Lp / S, grid.y = number of w, grid.z = rhs
// ---------------------------------------------------------------------------
template <typename T> struct ColS { static constexpr int S = 128 / (int)sizeof(cplx<T>); };

template <typename T, int NC, bool INV>
__global__ void __launch_bounds__(ColS<T>::S * FFT<cplx<T>, NC, INV>::T)
k_cols(const cplx<T>* __restrict__ in, long long in_w, long long in_rhs, int n_in,
       cplx<T>* __restrict__ out, long long out_w, long long out_rhs, int n_out, int Lp,
       const cplx<T>* __restrict__ tw) {
  using V = cplx<T>;
  using F = FFT<V, NC, INV>;
  constexpr int S = ColS<T>::S;
  constexpr int ES = S + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* tw_s = reinterpret_cast<V*>(smem_raw);
  V* buf = tw_s + NC;
  const int kx0 = blockIdx.x * S;
  const long long w = blockIdx.y;
  const V* inp = in + blockIdx.z * in_rhs + w * in_w + kx0;
  V* outp = out + blockIdx.z * out_rhs + w * out_w + kx0;
  stage_twiddles(tw_s, tw, NC);
  for (int i = threadIdx.x; i < S * n_in; i += blockDim.x) {
    const int y = i / S, s = i - y * S;
    buf[y * ES + s] = (kx0 + s < Lp) ? inp[(long long)y * Lp + s] : mk<V>(0, 0);
  }
  __syncthreads();
  const int s = threadIdx.x % S, t = threadIdx.x / S;
  V reg[F::E];
  if (!INV && 2 * n_in <= NC)
    F::load_half(reg, buf + s, ES, t, n_in);
  else
    F::load(reg, buf + s, ES, t, n_in);
  F::run(reg, buf + s, ES, t, tw_s);
  __syncthreads();
  F::store(reg, buf + s, ES, t);
  __syncthreads();
  for (int i = threadIdx.x; i < S * n_out; i += blockDim.x) {
    const int y = i / S, ss = i - y * S;
    if (kx0 + ss < Lp) outp[(long long)y * Lp + ss] = buf[y * ES + ss];
  }
}

// ---------------------------------------------------------------------------
// zmul: per (kx, ky) column: forward z transform of the three components,
// symmetric 3x3 multiply by fN, inverse z transform, keep z < N.  In place.
// B[c][z][ky][kx], fN[q][kz][ky][kx].  grid.x = Lp / S, grid.y = Mp, grid.z = rhs
// ---------------------------------------------------------------------------
template <typename T, int NZ> struct ZS {
  static constexpr int S0 = ColS<T>::S;
  static constexpr long long bytes(int s) { return (long long)(NZ + 3 * NZ * (s + 1)) * sizeof(cplx<T>); }
  static constexpr int S = bytes(S0) <= 220 * 1024 ? S0 : (bytes(S0 / 2) <= 220 * 1024 ? S0 / 2 : S0 / 4);
  static constexpr int THREADS = S * FFT<cplx<T>, NZ, false>::T;
};

template <typename T, int NZ>
__global__ void __launch_bounds__(ZS<T, NZ>::THREADS)
k_zmul(cplx<T>* __restrict__ B, long long b_rhs, const cplx<T>* __restrict__ fN, Dims d,
       const cplx<T>* __restrict__ tw) {
  using V = cplx<T>;
  using FF = FFT<V, NZ, false>;
  using FI = FFT<V, NZ, true>;
  constexpr int S = ZS<T, NZ>::S;
  constexpr int ES = S + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* tw_s = reinterpret_cast<V*>(smem_raw);
  V* buf = tw_s + NZ;  // 3 components x NZ x ES
  const int kx0 = blockIdx.x * S;
  const int ky = blockIdx.y;
  const long long plane = (long long)d.Lp * d.Mp;            // one z-plane of B
  const long long comp = plane * d.N;                        // one component of B
  V* Bp = B + blockIdx.z * b_rhs + (long long)ky * d.Lp + kx0;
  stage_twiddles(tw_s, tw, NZ);
  for (int i = threadIdx.x; i < 3 * S * d.N; i += blockDim.x) {
    const int c = i / (S * d.N);
    const int rem = i - c * S * d.N;
    const int z = rem / S, s = rem - z * S;
    buf[(c * NZ + z) * ES + s] = (kx0 + s < d.Lp) ? Bp[c * comp + z * plane + s] : mk<V>(0, 0);
  }
  __syncthreads();
  const int s = threadIdx.x % S, t = threadIdx.x / S;
  V reg[FF::E];
#pragma unroll 1
  for (int c = 0; c < 3; ++c) {
    V* base = buf + c * NZ * ES + s;
    FF::load_half(reg, base, ES, t, d.N);
    FF::run(reg, base, ES, t, tw_s);
    __syncthreads();
    FF::store(reg, base, ES, t);
    __syncthreads();
  }
  // symmetric tensor multiply
  const long long fq = (long long)d.Lp * d.Mp * d.Np;
  const V* fp = fN + (long long)ky * d.Lp + kx0;
  for (int i = threadIdx.x; i < S * NZ; i += blockDim.x) {
    const int kz = i / S, ss = i - kz * S;
    const long long o = (long long)kz * plane + ss;
    if (kx0 + ss >= d.Lp) continue;
    const V nxx = fp[o], nxy = fp[fq + o], nxz = fp[2 * fq + o];
    const V nyy = fp[3 * fq + o], nyz = fp[4 * fq + o], nzz = fp[5 * fq + o];
    V* e = buf + kz * ES + ss;
    const V jx = e[0], jy = e[NZ * ES], jz = e[2 * NZ * ES];
    e[0] = cadd(cadd(cmul(nxx, jx), cmul(nxy, jy)), cmul(nxz, jz));
    e[NZ * ES] = cadd(cadd(cmul(nxy, jx), cmul(nyy, jy)), cmul(nyz, jz));
    e[2 * NZ * ES] = cadd(cadd(cmul(nxz, jx), cmul(nyz, jy)), cmul(nzz, jz));
  }
  __syncthreads();
#pragma unroll 1
  for (int c = 0; c < 3; ++c) {
    V* base = buf + c * NZ * ES + s;
    FI::load(reg, base, ES, t, NZ);
    FI::run(reg, base, ES, t, tw_s);
    __syncthreads();
    FI::store(reg, base, ES, t);
    __syncthreads();
  }
  for (int i = threadIdx.x; i < 3 * S * d.N; i += blockDim.x) {
    const int c = i / (S * d.N);
    const int rem = i - c * S * d.N;
    const int z = rem / S, ss = rem - z * S;
    if (kx0 + ss < d.Lp) Bp[c * comp + z * plane + ss] = buf[(c * NZ + z) * ES + ss];
  }
}

}  // namespace marie
