// Operator assembly on the device: getOPERATORS(r, f, 'N')
// (src_vie/src_operators/getOPERATORS.m:1-127) in FP64.
//
//   Toeplitz G_mn(mx,my,mz,1..6) = (1/4pi) * sum_ij J_mn(i,j) P(i,j,k)
//     J_mn: 6x6 face-pair integrals of exp(-j k0 R)/R over the faces of the
//     observation voxel at offset m and the source voxel at the origin
//     (assembly_nop.m:37-136, cubature_nop.cpp:8-125):
//       far    : every offset, 4-point Gauss-Legendre per face direction
//       medium : offsets < 5 per axis, 10-point rule (overrides far)
//       near   : offsets < 2 per axis, 20-point rule with the weakly singular
//                pairs replaced by the self / edge / vertex integrals
//                (nearby_correct.m), overriding medium
//     Only 21 face pairs are integrated; the other 15 are copies
//     (cubature_nop.cpp:100-115).  The far loop skips offsets that the medium
//     loop overwrites.
//   circulant embedding 2L x 2M x 2N with per-axis parities (circulant_nop.m,
//     gperiodic_coeff_nop.m) and the 3-D FFT of each of the 6 components.
//
// The singular integrals come from the reference's own scheme by default:
// singular = 'D' runs DIRECTFN at Np_1D = 20 (directfn.cu), as
// assembly_nop.m:16,96-98 does.  singular = 'C' is an opt-in that is not in
// the reference: each square-square integral reduced to relative coordinates
// (the overlap of two unit intervals is a hat function) with the 1/R point
// singularity removed by a Duffy (polar-type) substitution, after which tensor
// Gauss-Legendre converges to machine precision; it differs from DIRECTFN at
// Np_1D = 20 by up to 3.4e-5 (the truncation error of DIRECTFN at that order).
// singular = 'U' takes the five values from the caller.
#include <cmath>
#include <vector>

#include "matvec_launch.cuh"
#include "plan.h"

namespace marie {

// --------------------------------------------------------------------------
// Gauss-Legendre nodes on [-1, 1] (ascending), Newton on P_n in long double.
// --------------------------------------------------------------------------
void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  for (int i = 0; i < n; ++i) {
    long double z = std::cos((long double)M_PI * (i + 0.75L) / (n + 0.5L));
    long double dp = 0;
    for (int it = 0; it < 100; ++it) {
      long double p0 = 1, p1 = z;
      for (int k = 2; k <= n; ++k) {
        long double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
        p0 = p1;
        p1 = p2;
      }
      if (n == 1) { p1 = z; p0 = 1; }
      dp = n * (z * p1 - p0) / (z * z - 1);
      long double dz = p1 / dp;
      z -= dz;
      if (std::fabs((double)dz) < 1e-19) break;
    }
    long double p0 = 1, p1 = z;
    for (int k = 2; k <= n; ++k) {
      long double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
      p0 = p1;
      p1 = p2;
    }
    dp = n * (z * p1 - p0) / (z * z - 1);
    x[n - 1 - i] = (double)z;
    w[n - 1 - i] = (double)(2.0L / ((1 - z * z) * dp * dp));
  }
}

// gauss_2d.m: tensor rule on [0,1]^2, I outer, J inner, w/4
static void gauss_2d(int n1, std::vector<double>& w, std::vector<double>& u, std::vector<double>& v) {
  std::vector<double> x1, w1;
  gauss_legendre(n1, x1, w1);
  w.clear(); u.clear(); v.clear();
  for (int i = 0; i < n1; ++i)
    for (int j = 0; j < n1; ++j) {
      w.push_back(0.25 * w1[i] * w1[j]);
      u.push_back((x1[i] + 1) / 2);
      v.push_back((x1[j] + 1) / 2);
    }
}

// --------------------------------------------------------------------------
// face geometry (cube_faces.m): face f = 2*axis + side; corner 1 at origin of
// the face, a = edge along the first in-plane axis, b = along the second.
// --------------------------------------------------------------------------
struct FaceGeom {
  double o[6][3], a[6][3], b[6][3];
};

static FaceGeom make_faces(double d) {
  FaceGeom g{};
  // (axis, in-plane axis of edge a, in-plane axis of edge b) as in cube_faces.m
  const int ea[3] = {1, 0, 0};
  const int eb[3] = {2, 2, 1};
  for (int f = 0; f < 6; ++f) {
    const int ax = f / 2, side = f % 2;
    for (int c = 0; c < 3; ++c) g.o[f][c] = g.a[f][c] = g.b[f][c] = 0;
    g.o[f][ax] = side * d;
    g.a[f][ea[ax]] = d;
    g.b[f][eb[ax]] = d;
  }
  return g;
}

// the 21 integrated (obs, src) pairs and the 15 copies, cubature_nop.cpp:24-26,100-115
__constant__ int c_pair_obs[21] = {0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 4, 4, 5};
__constant__ int c_pair_src[21] = {0, 1, 2, 3, 4, 5, 0, 2, 3, 4, 5, 2, 3, 4, 5, 2, 4, 5, 4, 5, 4};
__constant__ int c_copy_dst[15][2] = {{1, 1}, {2, 0}, {2, 1}, {3, 0}, {3, 1}, {3, 3}, {4, 0}, {4, 1},
                                      {4, 2}, {4, 3}, {5, 0}, {5, 1}, {5, 2}, {5, 3}, {5, 5}};
__constant__ int c_copy_src[15][2] = {{0, 0}, {1, 3}, {0, 3}, {1, 2}, {0, 2}, {2, 2}, {1, 5}, {0, 5},
                                      {3, 5}, {2, 5}, {1, 4}, {0, 4}, {3, 4}, {2, 4}, {4, 4}};

struct CubArgs {
  double face_o[6][3], face_a[6][3], face_b[6][3];
  double P[6][6][6];  // vector_projection.m: P(i,j,k)
  double2 sing[5];    // ST, EAc, EAo, VAc, VAo
  double ko, dx, scale;  // K: the factor dx^4 / (j k0)^2 / (4 pi) of assembly_kop.m
  int L, M, N;
};

// vector_projection.m:10-25 with face normals [-x,+x,-y,+y,-z,+z]
static void make_projection(double P[6][6][6]) {
  const double nrm[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};
  const int comp[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
  auto cross = [](const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
  };
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j)
      for (int k = 0; k < 6; ++k) {
        double ea[3] = {0, 0, 0}, eb[3] = {0, 0, 0}, c1[3], c2[3];
        ea[comp[k][0]] = 1;
        eb[comp[k][1]] = 1;
        cross(nrm[i], ea, c1);
        cross(nrm[j], eb, c2);
        P[i][j][k] = c1[0] * c2[0] + c1[1] * c2[1] + c1[2] * c2[2];
      }
}

// Singular class of face pair (obs face i of the voxel at offset m in {0,1}^3,
// src face j of the voxel at the origin), derived from the geometry:
// 0 regular, 1 ST (coincident), 2 EAc, 3 EAo, 4 VAc, 5 VAo.
__host__ __device__ inline int near_class(int mx, int my, int mz, int i, int j) {
  const int m[3] = {mx, my, mz};
  const int ai = i / 2, si = i % 2, aj = j / 2, sj = j % 2;
  if (ai == aj) {
    if (m[ai] + si != sj) return 0;
    int shifted = 0;
    for (int b = 0; b < 3; ++b)
      if (b != ai) shifted += m[b];
    return shifted == 0 ? 1 : (shifted == 1 ? 2 : 4);
  }
  const int ci = m[ai] + si;  // plane of face i along axis ai
  const int cj = sj;          // plane of face j along axis aj
  if (!(cj >= m[aj] && cj <= m[aj] + 1)) return 0;
  if (!(ci >= 0 && ci <= 1)) return 0;
  const int b = 3 - ai - aj;
  return m[b] == 0 ? 3 : 5;
}

__device__ __forceinline__ double2 warp_sum2(double2 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
  }
  return v;
}

// Quadrature points of face f: X[i] = o + a u_i + b v_i, stored [i][3].
__device__ __forceinline__ void face_points(const CubArgs& A, int f, const double* __restrict__ u,
                                            const double* __restrict__ v, int Np, double* X, int t0, int nt) {
  for (int i = t0; i < Np; i += nt) {
    const double ui = u[i], vi = v[i];
    for (int c = 0; c < 3; ++c) X[3 * i + c] = A.face_o[f][c] + A.face_a[f][c] * ui + A.face_b[f][c] * vi;
  }
}

// Sum over Np x Np point pairs of w_p w_q exp(-j ko R)/R for one face pair
// (points of the observation face P, of the source face Q, both [i][3] in
// shared memory; the observation voxel is displaced by rm); threads t0,
// t0 + nt, ... split the pairs.  1/R comes from one reciprocal square root
// (R = R^2 / R), not a square root and a division: the FP64 pipe is the limit.
__device__ double2 face_pair_sum(const double* __restrict__ P, const double* __restrict__ Q,
                                 const double* __restrict__ w, int Np, double ko, const double rm[3], int t0,
                                 int nt) {
  double2 acc = mk<double2>(0, 0);
  const int tot = Np * Np;
  for (int t = t0; t < tot; t += nt) {
    const int ip = t / Np, iq = t - ip * Np;
    const double dx0 = Q[3 * iq] - (P[3 * ip] + rm[0]);
    const double dx1 = Q[3 * iq + 1] - (P[3 * ip + 1] + rm[1]);
    const double dx2 = Q[3 * iq + 2] - (P[3 * ip + 2] + rm[2]);
    const double R2 = dx0 * dx0 + dx1 * dx1 + dx2 * dx2;
    const double Ri = rsqrt(R2);
    double s, c;
    sincos(ko * (R2 * Ri), &s, &c);
    const double wt = w[ip] * w[iq] * Ri;
    acc.x += wt * c;
    acc.y -= wt * s;
  }
  return acc;
}

// Mirror, optional near-field correction, projection and scaling of one
// offset's 21 integrals J21 (already multiplied by nothing); writes G (6 comps).
__device__ void finish_offset(const CubArgs& A, const double2* J21, int mx, int my, int mz, bool near,
                              double2* __restrict__ G, long long V, long long off) {
  double2 J[6][6];
  for (int i = 0; i < 6; ++i)
    for (int j = 0; j < 6; ++j) J[i][j] = mk<double2>(0, 0);
  for (int p = 0; p < 21; ++p) J[c_pair_obs[p]][c_pair_src[p]] = cscale(J21[p], A.dx * A.dx * A.dx * A.dx);
  for (int c = 0; c < 15; ++c) J[c_copy_dst[c][0]][c_copy_dst[c][1]] = J[c_copy_src[c][0]][c_copy_src[c][1]];
  if (near) {
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) {
        const int cls = near_class(mx, my, mz, i, j);
        if (cls > 0) J[i][j] = A.sing[cls - 1];
      }
  }
  const double s = 1.0 / (4.0 * M_PI);
  for (int k = 0; k < 6; ++k) {
    double2 g = mk<double2>(0, 0);
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j) {
        const double pp = A.P[i][j][k];
        if (pp != 0.0) g = cadd(g, cscale(J[i][j], pp));
      }
    G[k * V + off] = cscale(g, s);
  }
}

// far field: one warp per offset outside the medium region
__global__ void k_cub_far(CubArgs A, const double* __restrict__ gw, const double* __restrict__ gu,
                          const double* __restrict__ gv, int Np, int n_medium, double2* __restrict__ G) {
  __shared__ double w[16], u[16], v[16];
  __shared__ double X[6][16 * 3];  // quadrature points of the six faces
  if (threadIdx.x < Np) {
    w[threadIdx.x] = gw[threadIdx.x];
    u[threadIdx.x] = gu[threadIdx.x];
    v[threadIdx.x] = gv[threadIdx.x];
  }
  __syncthreads();
  for (int f = 0; f < 6; ++f) face_points(A, f, u, v, Np, X[f], threadIdx.x, blockDim.x);
  __syncthreads();
  const long long V = (long long)A.L * A.M * A.N;
  const int lane = threadIdx.x & 31;
  const long long wpb = blockDim.x >> 5;
  for (long long off = blockIdx.x * wpb + (threadIdx.x >> 5); off < V; off += (long long)gridDim.x * wpb) {
    const int mx = (int)(off % A.L);
    const int my = (int)((off / A.L) % A.M);
    const int mz = (int)(off / ((long long)A.L * A.M));
    if (mx < n_medium && my < n_medium && mz < n_medium) continue;
    const double rm[3] = {mx * A.dx, my * A.dx, mz * A.dx};
    double2 J21[21];
    for (int p = 0; p < 21; ++p)
      J21[p] = warp_sum2(face_pair_sum(X[c_pair_obs[p]], X[c_pair_src[p]], w, Np, A.ko, rm, lane, 32));
    if (lane == 0) finish_offset(A, J21, mx, my, mz, false, G, V, off);
  }
}

// medium / near: one block per (offset, pair); offsets enumerated in [0,nr)^3
__global__ void k_cub_region(CubArgs A, const double* __restrict__ gw, const double* __restrict__ gu,
                             const double* __restrict__ gv, int Np, int nr, double2* __restrict__ J21out) {
  extern __shared__ double sh[];
  double* w = sh;
  double* u = sh + Np;
  double* v = sh + 2 * Np;
  double* P = sh + 3 * Np;  // points of the observation face, [i][3]
  double* Q = P + 3 * Np;   // points of the source face
  for (int i = threadIdx.x; i < Np; i += blockDim.x) {
    w[i] = gw[i];
    u[i] = gu[i];
    v[i] = gv[i];
  }
  __syncthreads();
  const int pair = blockIdx.y;
  face_points(A, c_pair_obs[pair], u, v, Np, P, threadIdx.x, blockDim.x);
  face_points(A, c_pair_src[pair], u, v, Np, Q, threadIdx.x, blockDim.x);
  __syncthreads();
  const int o = blockIdx.x;
  const int mx = o % nr, my = (o / nr) % nr, mz = o / (nr * nr);
  const double rm[3] = {mx * A.dx, my * A.dx, mz * A.dx};
  double2 acc = face_pair_sum(P, Q, w, Np, A.ko, rm, threadIdx.x, blockDim.x);
  acc = warp_sum2(acc);
  __shared__ double2 ws[32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double2 t = mk<double2>(0, 0);
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t = cadd(t, ws[i]);
    J21out[(long long)o * 21 + pair] = t;
  }
}

__global__ void k_region_finish(CubArgs A, const double2* __restrict__ J21, int nr, bool near, double2* __restrict__ G) {
  const long long V = (long long)A.L * A.M * A.N;
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= nr * nr * nr) return;
  const int mx = o % nr, my = (o / nr) % nr, mz = o / (nr * nr);
  if (mx >= A.L || my >= A.M || mz >= A.N) return;
  const long long off = mx + (long long)A.L * (my + (long long)A.M * mz);
  double2 j21[21];
  for (int p = 0; p < 21; ++p) j21[p] = J21[(long long)o * 21 + p];
  finish_offset(A, j21, mx, my, mz, near, G, V, off);
}

// circulant_nop.m:23-40: index L of each axis stays zero; reflected blocks take
// the product of the per-axis parities of the component.
__global__ void k_circulant(const double2* __restrict__ G, int L, int M, int N, double2* __restrict__ C) {
  // parity per component [xx,xy,xz,yy,yz,zz] per axis (x, y, z): -1 odd
  const int par[6][3] = {{1, 1, 1}, {-1, -1, 1}, {-1, 1, -1}, {1, 1, 1}, {1, -1, -1}, {1, 1, 1}};
  const long long Lp = 2LL * L, Mp = 2LL * M, Np = 2LL * N;
  const long long P = Lp * Mp * Np;
  const long long V = (long long)L * M * N;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < 6 * P; t += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(t / P);
    long long r = t - q * P;
    const int ix = (int)(r % Lp);
    r /= Lp;
    const int iy = (int)(r % Mp);
    const int iz = (int)(r / Mp);
    double sgn = 1.0;
    int sx = ix, sy = iy, sz = iz;
    bool zero = false;
    if (ix == L) zero = true; else if (ix > L) { sx = (int)(Lp - ix); sgn *= par[q][0]; }
    if (iy == M) zero = true; else if (iy > M) { sy = (int)(Mp - iy); sgn *= par[q][1]; }
    if (iz == N) zero = true; else if (iz > N) { sz = (int)(Np - iz); sgn *= par[q][2]; }
    double2 val = mk<double2>(0, 0);
    if (!zero) {
      val = G[q * V + sx + (long long)L * (sy + (long long)M * sz)];
      val = mk<double2>(sgn * val.x, sgn * val.y);
    }
    C[t] = val;
  }
}

// plain in-place forward FFT of contiguous rows of length NL (full input)
template <int NL>
__global__ void __launch_bounds__(RowCfg<double2, NL>::THREADS)
k_rows_full(double2* __restrict__ data, long long rows, const double2* __restrict__ tw) {
  using V = double2;
  using F = FFT<V, NL, false>;
  constexpr int S = RowCfg<double2, NL>::S;
  constexpr int ES = S + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* tw_s = reinterpret_cast<V*>(smem_raw);
  V* buf = tw_s + NL;
  const long long row0 = (long long)blockIdx.x * S;
  stage_twiddles(tw_s, tw, NL);
  for (int i = threadIdx.x; i < S * NL; i += blockDim.x) {
    const int s = i / NL, x = i - s * NL;
    buf[x * ES + s] = (row0 + s < rows) ? data[(row0 + s) * NL + x] : mk<V>(0, 0);
  }
  __syncthreads();
  const int s = threadIdx.x % S, t = threadIdx.x / S;
  V reg[F::E];
  F::load(reg, buf + s, ES, t, NL);
  F::run(reg, buf + s, ES, t, tw_s);
  __syncthreads();
  F::store(reg, buf + s, ES, t);
  __syncthreads();
  for (int i = threadIdx.x; i < S * NL; i += blockDim.x) {
    const int ss = i / NL, x = i - ss * NL;
    if (row0 + ss < rows) data[(row0 + ss) * NL + x] = buf[x * ES + ss];
  }
}

static cudaError_t rows_full(int NL, double2* data, long long rows, const double2* tw, cudaStream_t st) {
  switch (NL) {
#define MARIE_CASE(n_)                                                                                   \
  case n_: {                                                                                             \
    constexpr int S = RowCfg<double2, n_>::S;                                                                     \
    const size_t smem = (size_t)(n_ + n_ * (S + 1)) * sizeof(double2);                                   \
    cudaError_t e = opt_in_smem(k_rows_full<n_>, smem);                                                  \
    if (e != cudaSuccess) return e;                                                                      \
    k_rows_full<n_><<<(unsigned)((rows + S - 1) / S), RowCfg<double2, n_>::THREADS, smem, st>>>(data, rows, tw); \
    count_launch();                                                                                      \
    return cudaGetLastError();                                                                           \
  }
    MARIE_FFT_LENGTHS(MARIE_CASE)
#undef MARIE_CASE
  }
  return cudaErrorInvalidValue;
}

// --------------------------------------------------------------------------
// converged singular integrals (singular = 'C'): relative coordinates + Duffy
// substitution; not a reference method
// --------------------------------------------------------------------------
struct SingArgs {
  double ko, a;
  int n;
};

__device__ __forceinline__ double2 cexpm(double phase) {  // exp(-j*phase)
  double s, c;
  sincos(phase, &s, &c);
  return mk<double2>(c, -s);
}

// one block per term; term t accumulates into out[t]
//  0: ST      8a^3  E2 (1-s)(1-st)
//  1: EAc-a   2a^3  E2 [s(1-st) + st(1-s)]
//  2: EAc-b   2a^2  f(|u|)(2a-u1)(a-u2),  u1=a(1+s), u2=at
//  3: EAo     2a^3  E3 [s(1-st1) + s(1-s) + s(1-st2)]
//  4: VAc-a   2a^3  E2 s^2 t
//  5: VAc-b   2a^2  f(|u|)(2a-u1) u2,     u1=a(1+s), u2=at
//  6: VAc-c    a^2  f(|u|)(2a-u1)(2a-u2), u1=a(1+s), u2=a(1+t)
//  7: VAo-a    a^3  E3 s^2 (t1 + 1 + t2)
//  8: VAo-b    a^3  f(|u|)(2a-u2),        u1=as, u2=a(1+t1), u3=at2
__global__ void k_singular(SingArgs S, const double* __restrict__ x01, const double* __restrict__ w01,
                           double2* __restrict__ out) {
  const int term = blockIdx.x;
  const int n = S.n;
  const bool three = (term == 3 || term == 7 || term == 8);
  const long long tot = three ? (long long)n * n * n : (long long)n * n;
  const double a = S.a, k = S.ko;
  double2 acc = mk<double2>(0, 0);
  for (long long t = threadIdx.x; t < tot; t += blockDim.x) {
    const int i = (int)(t % n);
    const int j = (int)((t / n) % n);
    const int l = (int)(t / ((long long)n * n));
    const double s = x01[i], tt = x01[j], t2 = three ? x01[l] : 0.0;
    const double wt = w01[i] * w01[j] * (three ? w01[l] : 1.0);
    double2 val = mk<double2>(0, 0);
    switch (term) {
      case 0: case 1: case 4: {
        const double rho = sqrt(1.0 + tt * tt);
        double g;
        if (term == 0) g = 8.0 * (1 - s) * (1 - s * tt);
        else if (term == 1) g = 2.0 * (s * (1 - s * tt) + s * tt * (1 - s));
        else g = 2.0 * s * s * tt;
        val = cscale(cexpm(k * a * s * rho), a * a * a * g / rho);
        break;
      }
      case 3: case 7: {
        const double rho = sqrt(1.0 + tt * tt + t2 * t2);
        const double g = term == 3 ? 2.0 * (s * (1 - s * tt) + s * (1 - s) + s * (1 - s * t2))
                                   : s * s * (tt + 1.0 + t2);
        val = cscale(cexpm(k * a * s * rho), a * a * a * g / rho);
        break;
      }
      case 2: case 5: case 6: {
        const double u1 = a * (1 + s);
        const double u2 = term == 6 ? a * (1 + tt) : a * tt;
        const double R = sqrt(u1 * u1 + u2 * u2);
        double g;
        if (term == 2) g = 2.0 * (2 * a - u1) * (a - u2);
        else if (term == 5) g = 2.0 * (2 * a - u1) * u2;
        else g = (2 * a - u1) * (2 * a - u2);
        val = cscale(cexpm(k * R), a * a * g / R);
        break;
      }
      case 8: {
        const double u1 = a * s, u2 = a * (1 + tt), u3 = a * t2;
        const double R = sqrt(u1 * u1 + u2 * u2 + u3 * u3);
        val = cscale(cexpm(k * R), a * a * a * (2 * a - u2) / R);
        break;
      }
    }
    acc = cadd(acc, cscale(val, wt));
  }
  acc = warp_sum2(acc);
  __shared__ double2 ws[32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double2 tsum = mk<double2>(0, 0);
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) tsum = cadd(tsum, ws[i]);
    out[term] = tsum;
  }
}

static int converged_integrals(double ko, double dx, int n, double2 out[5], cudaStream_t st) {
  std::vector<double> x, w;
  gauss_legendre(n, x, w);
  for (int i = 0; i < n; ++i) {
    x[i] = 0.5 * (x[i] + 1.0);
    w[i] *= 0.5;
  }
  DBuf dxn, dwn, dout;
  MARIE_TRY(dxn.alloc(n * sizeof(double), st));
  MARIE_TRY(dwn.alloc(n * sizeof(double), st));
  MARIE_TRY(dout.alloc(9 * sizeof(double2), st));
  MARIE_CUDA_TRY(cudaMemcpyAsync(dxn.p, x.data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
  MARIE_CUDA_TRY(cudaMemcpyAsync(dwn.p, w.data(), n * sizeof(double), cudaMemcpyHostToDevice, st));
  SingArgs S{ko, dx, n};
  k_singular<<<9, 512, 0, st>>>(S, dxn.as<double>(), dwn.as<double>(), dout.as<double2>());
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  double2 t[9];
  MARIE_CUDA_TRY(cudaMemcpyAsync(t, dout.p, sizeof(t), cudaMemcpyDeviceToHost, st));
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  out[0] = t[0];
  out[1] = cadd(t[1], t[2]);
  out[2] = t[3];
  out[3] = cadd(cadd(t[4], t[5]), t[6]);
  out[4] = cadd(t[7], t[8]);
  return MARIE_OK;
}

// Toeplitz G (L x M x N x 6) on the device.
static int assemble_toeplitz(int L, int M, int N, double dx, double ko, const double2 sing[5], double2* G,
                             cudaStream_t st) {
  CubArgs A{};
  const FaceGeom fg = make_faces(dx);
  for (int f = 0; f < 6; ++f)
    for (int c = 0; c < 3; ++c) {
      A.face_o[f][c] = fg.o[f][c];
      A.face_a[f][c] = fg.a[f][c];
      A.face_b[f][c] = fg.b[f][c];
    }
  make_projection(A.P);
  for (int i = 0; i < 5; ++i) A.sing[i] = sing[i];
  A.ko = ko;
  A.dx = dx;
  A.L = L; A.M = M; A.N = N;
  const int n_medium = 5;
  struct Rule { DBuf w, u, v; int Np; };
  Rule rules[3];
  const int orders[3] = {4, 10, 20};
  for (int r = 0; r < 3; ++r) {
    std::vector<double> w, u, v;
    gauss_2d(orders[r], w, u, v);
    rules[r].Np = (int)w.size();
    MARIE_TRY(rules[r].w.alloc(w.size() * sizeof(double), st));
    MARIE_TRY(rules[r].u.alloc(w.size() * sizeof(double), st));
    MARIE_TRY(rules[r].v.alloc(w.size() * sizeof(double), st));
    MARIE_CUDA_TRY(cudaMemcpyAsync(rules[r].w.p, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    MARIE_CUDA_TRY(cudaMemcpyAsync(rules[r].u.p, u.data(), u.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    MARIE_CUDA_TRY(cudaMemcpyAsync(rules[r].v.p, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, st));
  }
  const long long V = (long long)L * M * N;
  {
    const int warps = 8;
    long long blocks = (V + warps - 1) / warps;
    if (blocks > 152 * 64) blocks = 152 * 64;
    k_cub_far<<<(unsigned)blocks, 32 * warps, 0, st>>>(A, rules[0].w.as<double>(), rules[0].u.as<double>(),
                                                       rules[0].v.as<double>(), rules[0].Np, n_medium, G);
    count_launch();
    MARIE_CUDA_TRY(cudaGetLastError());
  }
  // medium (10-point) then near (20-point, corrected); MATLAB loops run 1:5 and
  // 1:2 per axis; offsets beyond the grid are dropped here.
  for (int pass = 0; pass < 2; ++pass) {
    const int nr = pass == 0 ? n_medium : 2;
    Rule& R = rules[pass + 1];
    const int nO = nr * nr * nr;
    DBuf J21;
    MARIE_TRY(J21.alloc((size_t)nO * 21 * sizeof(double2), st));
    dim3 grid(nO, 21);
    const size_t smem = 9 * R.Np * sizeof(double);  // w, u, v and the two faces' points
    if (smem > 48 * 1024)
      MARIE_CUDA_TRY(cudaFuncSetAttribute(k_cub_region, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_cub_region<<<grid, 256, smem, st>>>(A, R.w.as<double>(), R.u.as<double>(), R.v.as<double>(), R.Np, nr,
                                          J21.as<double2>());
    count_launch();
    MARIE_CUDA_TRY(cudaGetLastError());
    k_region_finish<<<(nO + 127) / 128, 128, 0, st>>>(A, J21.as<double2>(), nr, pass == 1, G);
    count_launch();
    MARIE_CUDA_TRY(cudaGetLastError());
    MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  }
  return MARIE_OK;
}

// Forward 3-D FFT in place of the nq components of a 2L x 2M x 2N circulant.
static int fft_operator(double2* C, int Lp, int Mp, int Np, cudaStream_t st, int nq = 6) {
  std::vector<double2*> tw(3, nullptr);
  const int lens[3] = {Lp, Mp, Np};
  std::vector<DBuf> twb(3);
  for (int a = 0; a < 3; ++a) {
    std::vector<double2> h(lens[a]);
    for (int k = 0; k < lens[a]; ++k) {
      const double ang = 2.0 * M_PI * k / lens[a];
      h[k] = mk<double2>(std::cos(ang), -std::sin(ang));
    }
    MARIE_TRY(twb[a].alloc(lens[a] * sizeof(double2), st));
    MARIE_CUDA_TRY(cudaMemcpyAsync(twb[a].p, h.data(), lens[a] * sizeof(double2), cudaMemcpyHostToDevice, st));
    tw[a] = twb[a].as<double2>();
  }
  const long long P = (long long)Lp * Mp * Np;
  MARIE_CUDA_TRY(rows_full(Lp, C, nq * P / Lp, tw[0], st));
  using ML = MatvecLaunch<double>;
  // y: columns of S consecutive x, stride Lp, w = (z, q)
  MARIE_CUDA_TRY(ML::cols(false, Mp, C, (long long)Lp * Mp, 0, Mp, C, (long long)Lp * Mp, 0, Mp, Lp, nq * Np,
                          tw[1], 1, st));
  // z: columns over the contiguous (x, y) plane, stride Lp*Mp, w = q
  MARIE_CUDA_TRY(ML::cols(false, Np, C, P, 0, Np, C, P, 0, Np, Lp * Mp, nq, tw[2], 1, st));
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  return MARIE_OK;
}

// --------------------------------------------------------------------------
// K operator: getOPERATORS(r, f, 'K') (getOPERATORS.m:101-120)
//   Toeplitz IK_mn(mx,my,mz,1..3) = dx^4 / (j k0)^2 / (4 pi) * I(m) with
//   (assembly_kop.m:7-120)
//     far    : every offset, 4-point rule, the 12 signed face pairs of
//              cubature_kop.cpp:30-32 of sum w_p w_q G(R) (r_p - r_q),
//              G = (1 - exp(-j k0 R)(1 + j k0 R)) / R^3
//     medium : offsets < 5 per axis, the same with the 10-point rule
//     near   : offsets < 2 per axis, 20-point rule on all 36 face pairs (21
//              integrated, 15 copies as for N), the coincident pairs dropped
//              (nearby_correct_kop.m) and the face-normal combination of
//              cubature_kop_near_sym.m:91-105
//   circulant with component c odd along axis c (circulant_kop.m,
//   gperiodic_coeff_kop.m), then the FFT of the 3 components.
// --------------------------------------------------------------------------
__constant__ int c_kop_obs[12] = {0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5};
__constant__ int c_kop_src[12] = {0, 1, 0, 1, 2, 3, 2, 3, 4, 5, 4, 5};
__constant__ double c_kop_sign[12] = {1, -1, -1, 1, 1, -1, -1, 1, 1, -1, -1, 1};

// sum over point pairs of w_p w_q G(R) (r_p - r_q) for one face pair (points
// of the observation face P and of the source face Q in shared memory, [i][3];
// R and 1/R^3 from one reciprocal square root, as in face_pair_sum)
__device__ void kop_pair_sum(const double* __restrict__ P, const double* __restrict__ Q,
                             const double* __restrict__ w, int Np, double ko, const double rm[3], int lane, int nl,
                             double2 out[3]) {
  out[0] = out[1] = out[2] = mk<double2>(0, 0);
  const int tot = Np * Np;
  for (int t = lane; t < tot; t += nl) {
    const int ip = t / Np, iq = t - ip * Np;
    double d[3];
    for (int c = 0; c < 3; ++c) d[c] = (P[3 * ip + c] + rm[c]) - Q[3 * iq + c];
    const double R2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const double Ri = rsqrt(R2);
    const double kR = ko * (R2 * Ri);
    double sn, cs;
    sincos(kR, &sn, &cs);
    // 1 - exp(-j kR) (1 + j kR) = (1 - cs - kR sn) - j (kR cs - sn)
    const double wt = w[ip] * w[iq] * (Ri * Ri * Ri);
    const double gr = wt * (1.0 - cs - kR * sn), gi = -wt * (kR * cs - sn);
    for (int c = 0; c < 3; ++c) {
      out[c].x += gr * d[c];
      out[c].y += gi * d[c];
    }
  }
}

// far field: one warp per offset outside the medium region; writes I (3 comps)
__global__ void k_kop_far(CubArgs A, const double* __restrict__ gw, const double* __restrict__ gu,
                          const double* __restrict__ gv, int Np, int n_medium, double2* __restrict__ K) {
  __shared__ double w[16], u[16], v[16];
  __shared__ double X[6][16 * 3];  // quadrature points of the six faces
  if (threadIdx.x < Np) {
    w[threadIdx.x] = gw[threadIdx.x];
    u[threadIdx.x] = gu[threadIdx.x];
    v[threadIdx.x] = gv[threadIdx.x];
  }
  __syncthreads();
  for (int f = 0; f < 6; ++f) face_points(A, f, u, v, Np, X[f], threadIdx.x, blockDim.x);
  __syncthreads();
  const long long V = (long long)A.L * A.M * A.N;
  const int lane = threadIdx.x & 31;
  const long long wpb = blockDim.x >> 5;
  for (long long off = blockIdx.x * wpb + (threadIdx.x >> 5); off < V; off += (long long)gridDim.x * wpb) {
    const int mx = (int)(off % A.L);
    const int my = (int)((off / A.L) % A.M);
    const int mz = (int)(off / ((long long)A.L * A.M));
    if (mx < n_medium && my < n_medium && mz < n_medium) continue;
    const double rm[3] = {mx * A.dx, my * A.dx, mz * A.dx};
    // signed lane sums over the 12 pairs, one warp reduction per component
    double2 acc[3] = {mk<double2>(0, 0), mk<double2>(0, 0), mk<double2>(0, 0)};
    for (int p = 0; p < 12; ++p) {
      double2 o[3];
      kop_pair_sum(X[c_kop_obs[p]], X[c_kop_src[p]], w, Np, A.ko, rm, lane, 32, o);
      for (int c = 0; c < 3; ++c) acc[c] = cadd(acc[c], cscale(o[c], c_kop_sign[p]));
    }
    for (int c = 0; c < 3; ++c) acc[c] = warp_sum2(acc[c]);
    if (lane == 0)
      for (int c = 0; c < 3; ++c) K[c * V + off] = cscale(acc[c], A.scale);
  }
}

// medium (near = false: the 12 signed pairs) or near (the 21 pairs of the
// symmetric set): one block per (offset, pair); out[o][pair][3]
__global__ void k_kop_region(CubArgs A, const double* __restrict__ gw, const double* __restrict__ gu,
                             const double* __restrict__ gv, int Np, int nr, bool near, double2* __restrict__ out) {
  extern __shared__ double sh[];
  double* w = sh;
  double* u = sh + Np;
  double* v = sh + 2 * Np;
  double* P = sh + 3 * Np;  // points of the observation face, [i][3]
  double* Q = P + 3 * Np;   // points of the source face
  for (int i = threadIdx.x; i < Np; i += blockDim.x) {
    w[i] = gw[i];
    u[i] = gu[i];
    v[i] = gv[i];
  }
  __syncthreads();
  const int pair = blockIdx.y;
  const int io = near ? c_pair_obs[pair] : c_kop_obs[pair];
  const int is = near ? c_pair_src[pair] : c_kop_src[pair];
  face_points(A, io, u, v, Np, P, threadIdx.x, blockDim.x);
  face_points(A, is, u, v, Np, Q, threadIdx.x, blockDim.x);
  __syncthreads();
  const int o = blockIdx.x;
  const int mx = o % nr, my = (o / nr) % nr, mz = o / (nr * nr);
  const double rm[3] = {mx * A.dx, my * A.dx, mz * A.dx};
  double2 acc[3];
  kop_pair_sum(P, Q, w, Np, A.ko, rm, threadIdx.x, blockDim.x, acc);
  __shared__ double2 ws[3][32];
  for (int c = 0; c < 3; ++c) {
    const double2 r = warp_sum2(acc[c]);
    if ((threadIdx.x & 31) == 0) ws[c][threadIdx.x >> 5] = r;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double2 t = mk<double2>(0, 0);
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t = cadd(t, ws[threadIdx.x][i]);
    out[((long long)o * (near ? 21 : 12) + pair) * 3 + threadIdx.x] = t;
  }
}

__global__ void k_kop_finish(CubArgs A, const double2* __restrict__ I, int nr, bool near, double2* __restrict__ K) {
  const long long V = (long long)A.L * A.M * A.N;
  const int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= nr * nr * nr) return;
  const int mx = o % nr, my = (o / nr) % nr, mz = o / (nr * nr);
  if (mx >= A.L || my >= A.M || mz >= A.N) return;
  const long long off = mx + (long long)A.L * (my + (long long)A.M * mz);
  double2 r[3] = {mk<double2>(0, 0), mk<double2>(0, 0), mk<double2>(0, 0)};
  if (!near) {
    for (int p = 0; p < 12; ++p)
      for (int c = 0; c < 3; ++c) r[c] = cadd(r[c], cscale(I[((long long)o * 12 + p) * 3 + c], c_kop_sign[p]));
  } else {
    // I(6,6,3): the 21 integrated pairs, the 15 copies, coincident pairs dropped
    double2 F[6][6][3];
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j)
        for (int c = 0; c < 3; ++c) F[i][j][c] = mk<double2>(0, 0);
    for (int p = 0; p < 21; ++p)
      for (int c = 0; c < 3; ++c) F[c_pair_obs[p]][c_pair_src[p]][c] = I[((long long)o * 21 + p) * 3 + c];
    for (int q = 0; q < 15; ++q)
      for (int c = 0; c < 3; ++c) F[c_copy_dst[q][0]][c_copy_dst[q][1]][c] = F[c_copy_src[q][0]][c_copy_src[q][1]][c];
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 6; ++j)
        if (near_class(mx, my, mz, i, j) == 1)
          for (int c = 0; c < 3; ++c) F[i][j][c] = mk<double2>(0, 0);
    // J(i,:) = -/+ I(i,:,axis(i)); IK_c = sum_i J(i, 2c+1) - J(i, 2c)
    for (int i = 0; i < 6; ++i) {
      const double sg = (i % 2) ? 1.0 : -1.0;
      for (int c = 0; c < 3; ++c) r[c] = cadd(r[c], cscale(csub(F[i][2 * c + 1][i / 2], F[i][2 * c][i / 2]), sg));
    }
  }
  for (int c = 0; c < 3; ++c) K[c * V + off] = cscale(r[c], A.scale);
}

// circulant_kop.m:17-41: component c odd along axis c; index L stays zero
__global__ void k_circulant_k(const double2* __restrict__ G, int L, int M, int N, double2* __restrict__ C) {
  const long long Lp = 2LL * L, Mp = 2LL * M, Np = 2LL * N;
  const long long P = Lp * Mp * Np;
  const long long V = (long long)L * M * N;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < 3 * P; t += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(t / P);
    long long r = t - q * P;
    const int ix = (int)(r % Lp);
    r /= Lp;
    const int iy = (int)(r % Mp);
    const int iz = (int)(r / Mp);
    double sgn = 1.0;
    int sx = ix, sy = iy, sz = iz;
    bool zero = false;
    if (ix == L) zero = true; else if (ix > L) { sx = (int)(Lp - ix); if (q == 0) sgn = -sgn; }
    if (iy == M) zero = true; else if (iy > M) { sy = (int)(Mp - iy); if (q == 1) sgn = -sgn; }
    if (iz == N) zero = true; else if (iz > N) { sz = (int)(Np - iz); if (q == 2) sgn = -sgn; }
    double2 val = mk<double2>(0, 0);
    if (!zero) {
      val = G[q * V + sx + (long long)L * (sy + (long long)M * sz)];
      val = mk<double2>(sgn * val.x, sgn * val.y);
    }
    C[t] = val;
  }
}

// Toeplitz K (L x M x N x 3) on the device.
static int assemble_toeplitz_k(int L, int M, int N, double dx, double ko, double2* K, cudaStream_t st) {
  CubArgs A{};
  const FaceGeom fg = make_faces(dx);
  for (int f = 0; f < 6; ++f)
    for (int c = 0; c < 3; ++c) {
      A.face_o[f][c] = fg.o[f][c];
      A.face_a[f][c] = fg.a[f][c];
      A.face_b[f][c] = fg.b[f][c];
    }
  A.ko = ko;
  A.dx = dx;
  A.scale = -dx * dx * dx * dx / (4.0 * M_PI * ko * ko);  // dx^4 / (j k0)^2 / (4 pi)
  A.L = L; A.M = M; A.N = N;
  const int n_medium = 5;
  struct Rule { DBuf w, u, v; int Np; };
  Rule rules[3];
  const int orders[3] = {4, 10, 20};
  for (int r = 0; r < 3; ++r) {
    std::vector<double> w, u, v;
    gauss_2d(orders[r], w, u, v);
    rules[r].Np = (int)w.size();
    MARIE_TRY(rules[r].w.alloc(w.size() * sizeof(double), st));
    MARIE_TRY(rules[r].u.alloc(w.size() * sizeof(double), st));
    MARIE_TRY(rules[r].v.alloc(w.size() * sizeof(double), st));
    MARIE_CUDA_TRY(cudaMemcpyAsync(rules[r].w.p, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    MARIE_CUDA_TRY(cudaMemcpyAsync(rules[r].u.p, u.data(), u.size() * sizeof(double), cudaMemcpyHostToDevice, st));
    MARIE_CUDA_TRY(cudaMemcpyAsync(rules[r].v.p, v.data(), v.size() * sizeof(double), cudaMemcpyHostToDevice, st));
  }
  const long long V = (long long)L * M * N;
  {
    const int warps = 8;
    long long blocks = (V + warps - 1) / warps;
    if (blocks > 152 * 64) blocks = 152 * 64;
    k_kop_far<<<(unsigned)blocks, 32 * warps, 0, st>>>(A, rules[0].w.as<double>(), rules[0].u.as<double>(),
                                                       rules[0].v.as<double>(), rules[0].Np, n_medium, K);
    count_launch();
    MARIE_CUDA_TRY(cudaGetLastError());
  }
  // medium (10-point rule, 12 pairs) then near (20-point rule, 21 pairs); the
  // MATLAB loops run 1:5 and 1:2 per axis, offsets beyond the grid are dropped
  for (int pass = 0; pass < 2; ++pass) {
    const bool near = pass == 1;
    const int nr = near ? 2 : n_medium;
    const int npairs = near ? 21 : 12;
    Rule& R = rules[pass + 1];
    const int nO = nr * nr * nr;
    DBuf I;
    MARIE_TRY(I.alloc((size_t)nO * npairs * 3 * sizeof(double2), st));
    dim3 grid(nO, npairs);
    const size_t smem = 9 * R.Np * sizeof(double);  // w, u, v and the two faces' points
    if (smem > 48 * 1024)
      MARIE_CUDA_TRY(cudaFuncSetAttribute(k_kop_region, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_kop_region<<<grid, 256, smem, st>>>(A, R.w.as<double>(), R.u.as<double>(), R.v.as<double>(), R.Np, nr, near,
                                          I.as<double2>());
    count_launch();
    MARIE_CUDA_TRY(cudaGetLastError());
    k_kop_finish<<<(nO + 127) / 128, 128, 0, st>>>(A, I.as<double2>(), nr, near, K);
    count_launch();
    MARIE_CUDA_TRY(cudaGetLastError());
    MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  }
  return MARIE_OK;
}

int assemble_k_device(int L, int M, int N, double dx, double freq, char type, double2* out, cudaStream_t st) {
  const double ko = 2.0 * M_PI / 299792458.0 * freq;  // getOPERATORS.m:48
  const long long V = (long long)L * M * N;
  if (type == 'T') return assemble_toeplitz_k(L, M, N, dx, ko, out, st);
  DBuf G;
  MARIE_TRY(G.alloc(3 * V * sizeof(double2), st));
  MARIE_TRY(assemble_toeplitz_k(L, M, N, dx, ko, G.as<double2>(), st));
  const long long P = 8 * V;
  k_circulant_k<<<(unsigned)std::min<long long>((3 * P + 255) / 256, 152 * 32), 256, 0, st>>>(G.as<double2>(), L, M,
                                                                                              N, out);
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  if (type == 'C') {
    MARIE_CUDA_TRY(cudaStreamSynchronize(st));
    return MARIE_OK;
  }
  return fft_operator(out, 2 * L, 2 * M, 2 * N, st, 3);
}

// The reference's Np_1D for the singular integrals (Np_DEMCEM, assembly_nop.m:16).
constexpr int kNpSingular = 20;
// Gauss order of the converged quadrature of singular = 'C'.
constexpr int kNpConverged = 32;

// singular: 'D' DIRECTFN at order np (0: the reference's 20), 'C' the converged
// quadrature at order np (0: 32), 'U' the caller's five values.  The
// reference's other method, DEMCEM, is not built.
static int singular_values(char singular, int np, const double* user, double ko, double dx, double2 s[5],
                           cudaStream_t st) {
  switch (singular) {
    case 'U': case 'u':
      if (!user) return set_error(MARIE_EINVAL, "singular = 'U' needs the five singular values");
      for (int i = 0; i < 5; ++i) s[i] = mk<double2>(user[2 * i], user[2 * i + 1]);
      return MARIE_OK;
    case 'D': case 'd':
      return directfn_integrals(ko, dx, np ? np : kNpSingular, s, st);
    case 'C': case 'c':
      if (np < 0 || np > 128) return set_error(MARIE_EINVAL, "order of the converged quadrature out of range");
      return converged_integrals(ko, dx, np ? np : kNpConverged, s, st);
    case 'E': case 'e':
      return set_error(MARIE_EINVAL, "singular = DEMCEM is not built; use 'D' (DIRECTFN, the reference default)");
    default:
      return set_error(MARIE_EINVAL, "singular must be 'D', 'C' or 'U'");
  }
}

static int get_sing(char singular, const double* user, double ko, double dx, double2 s[5], cudaStream_t st) {
  return singular_values(singular, 0, user, ko, dx, s, st);
}

int assemble_operator_device(int L, int M, int N, double dx, double freq, char singular, const double* user_sing,
                             char type, double2* out, cudaStream_t st) {
  const double ko = 2.0 * M_PI / 299792458.0 * freq;  // getOPERATORS.m:48
  double2 sing[5];
  MARIE_TRY(get_sing(singular, user_sing, ko, dx, sing, st));
  const long long V = (long long)L * M * N;
  if (type == 'T') return assemble_toeplitz(L, M, N, dx, ko, sing, out, st);
  DBuf G;
  MARIE_TRY(G.alloc(6 * V * sizeof(double2), st));
  MARIE_TRY(assemble_toeplitz(L, M, N, dx, ko, sing, G.as<double2>(), st));
  const long long P = 8 * V;
  k_circulant<<<(unsigned)std::min<long long>((6 * P + 255) / 256, 152 * 32), 256, 0, st>>>(G.as<double2>(), L, M, N,
                                                                                             out);
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  if (type == 'C') {
    MARIE_CUDA_TRY(cudaStreamSynchronize(st));
    return MARIE_OK;
  }
  return fft_operator(out, 2 * L, 2 * M, 2 * N, st);
}

}  // namespace marie

using namespace marie;

extern "C" {

int marie_singular_integrals_ex(double ko, double dx, char method, int np_1d, double* out10) {
  if (!out10 || !(dx > 0)) return set_error(MARIE_EINVAL, "bad argument");
  if (method == 'U' || method == 'u') return set_error(MARIE_EINVAL, "method must be 'D' or 'C'");
  double2 s[5];
  MARIE_TRY(singular_values(method, np_1d, nullptr, ko, dx, s, 0));
  for (int i = 0; i < 5; ++i) {
    out10[2 * i] = s[i].x;
    out10[2 * i + 1] = s[i].y;
  }
  return MARIE_OK;
}

int marie_singular_integrals(double ko, double dx, double* out10) {
  return marie_singular_integrals_ex(ko, dx, 'D', 0, out10);
}

int marie_get_operators(const double* r, int64_t L, int64_t M, int64_t N, double f, char op, char type,
                        char singular, const double* singular_values, double* op_out) {
  if (!r || !op_out) return set_error(MARIE_EINVAL, "NULL argument");
  if (op != 'N' && op != 'K') return set_error(MARIE_EINVAL, "op must be 'N' or 'K'");
  if (type != 'F' && type != 'C' && type != 'T') return set_error(MARIE_EINVAL, "type must be 'F', 'C' or 'T'");
  if (L < 2) return set_error(MARIE_EINVAL, "L must be >= 2 to read dx from r");
  MARIE_TRACE("getOPERATORS");
  if (type != 'T' && (!fft_length_supported((int)(2 * L)) || !fft_length_supported((int)(2 * M)) ||
                      !fft_length_supported((int)(2 * N))))
    return set_error(MARIE_EUNSUPPORTED, "padded FFT length not supported");
  double r0[2];
  MARIE_CUDA_TRY(cudaMemcpy(r0, r, 2 * sizeof(double), cudaMemcpyDefault));
  const double dx = r0[1] - r0[0];  // getOPERATORS.m:47
  if (!(dx > 0)) return set_error(MARIE_EINVAL, "r must have increasing x coordinates");
  cudaStream_t st = 0;
  const long long V = L * M * N;
  const long long nq = op == 'N' ? 6 : 3;
  const size_t bytes = (type == 'T' ? nq * V : 8 * nq * V) * sizeof(double2);
  DBuf tmp;
  void* dev;
  MARIE_TRY(stage_out(op_out, bytes, st, tmp, &dev));
  if (op == 'K')
    MARIE_TRY(assemble_k_device((int)L, (int)M, (int)N, dx, f, type, (double2*)dev, st));
  else
    MARIE_TRY(assemble_operator_device((int)L, (int)M, (int)N, dx, f, singular, singular_values, type,
                                       (double2*)dev, st));
  MARIE_TRY(finish_out(op_out, dev, bytes, st));
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  return MARIE_OK;
}

int marie_plan_assemble(marie_plan* p, double dx, double freq, char singular, const double* singular_values) {
  if (!p) return set_error(MARIE_EINVAL, "NULL plan");
  if (!(dx > 0) || !(freq > 0)) return set_error(MARIE_EINVAL, "dx and freq must be positive");
  MARIE_TRACE("getOPERATORS N");
  DBuf F;
  MARIE_TRY(F.alloc((size_t)48 * p->d.V * sizeof(double2), p->stream));
  MARIE_TRY(assemble_operator_device(p->d.L, p->d.M, p->d.N, dx, freq, singular, singular_values, 'F',
                                     F.as<double2>(), p->stream));
  return install_operator(p, F.as<double2>());
}

int marie_plan_assemble_k(marie_plan* p, double dx, double freq) {
  if (!p) return set_error(MARIE_EINVAL, "NULL plan");
  if (!(dx > 0) || !(freq > 0)) return set_error(MARIE_EINVAL, "dx and freq must be positive");
  MARIE_TRACE("getOPERATORS K");
  DBuf F;
  MARIE_TRY(F.alloc((size_t)24 * p->d.V * sizeof(double2), p->stream));
  MARIE_TRY(assemble_k_device(p->d.L, p->d.M, p->d.N, dx, freq, 'F', F.as<double2>(), p->stream));
  return install_operator(p, F.as<double2>(), 1);
}

}  // extern "C"
