// DIRECTFN weakly singular integrals on the device, FP64.
//
// The reference computes the five singular square-square integrals of
// exp(-j ko R)/R that nearby_correct.m substitutes (ST, EAc, EAo, VAc, VAo)
// by splitting each square face into two triangles and calling the DIRECTFN
// cores for constant basis functions on triangle pairs
// (src_vie/src_operators/cubatures/singular_st.m:14-17, singular_ea.m:17-28,
// singular_va.m:20-34) at Np_1D = 20 Gauss-Legendre points per dimension
// (assembly_nop.m:16):
//   coincident triangles       mexcubatures/directfn_ws_st_const.cpp:48-183
//   edge-adjacent triangles    mexcubatures/directfn_ws_ea_const.cpp:48-182
//   vertex-adjacent triangles  mexcubatures/directfn_ws_va_const.cpp:47-243
// The method (Polimeridis & Mosig, IJNME 83, 2010; Polimeridis, Vipiana,
// Mosig & Wilton, IEEE TAP 61(6), 2013) maps both triangles onto the
// equilateral triangle (eta, xi) with vertices (-1,0), (1,0), (0,sqrt 3),
// changes to polar-type relative coordinates, splits the angular ranges into
// subdomains in which the radial limit is one straight edge, and integrates
// all four dimensions with Gauss-Legendre rules.  Here the two outer
// dimensions of each subdomain (and the sub-triangle or sign branch) form one
// work item per warp; the warp's lanes share the inner two dimensions, and a
// second kernel sums the items of each output in a fixed order, so results
// repeat bit for bit.  The subdomain limits, the nesting of the rules and the
// MEX gateways' vertex order (the EA gateway hands the core the second
// triangle as (r4, r2, r1), directfn_ws_ea_const_mex.cpp:50; the VA gateway
// as (r4, r5, r1), directfn_ws_va_const_mex.cpp:51) are the reference's: they
// define the quadrature, and another split changes its value at Np_1D = 20 by
// up to 3e-5.
#include <array>
#include <cmath>
#include <vector>

#include "plan.h"

namespace marie {

namespace {

constexpr double kSq3 = 1.7320508075688772935;
constexpr double kPi = 3.14159265358979323846;

// one triangle-pair call of a DIRECTFN core
struct DfnPair {
  double p[3][3], q[3][3];  // vertices in the order the core receives them
  double jac;               // (area_p / sqrt 3) * (area_q / sqrt 3)
  int kind;                 // 0 coincident, 1 edge-adjacent, 2 vertex-adjacent
  int slot;                 // output the pair adds to
  long long first;          // index of its first work item
};

__host__ __device__ inline long long items_of(int kind, int n) {
  const long long n2 = (long long)n * n;
  return kind == 0 ? 24 * n2 : kind == 1 ? 18 * n2 : 2 * n2;
}

__host__ __device__ __forceinline__ void tri_point(const double v[3][3], double eta, double xi, double r[3]) {
  const double w1 = (kSq3 * (1.0 - eta) - xi) / (2.0 * kSq3);
  const double w2 = (kSq3 * (1.0 + eta) - xi) / (2.0 * kSq3);
  const double w3 = xi / kSq3;
#pragma unroll
  for (int c = 0; c < 3; ++c) r[c] = w1 * v[0][c] + w2 * v[1][c] + w3 * v[2][c];
}

// exp(-j ko R) / R between the points (ep, xp) of P and (eq, xq) of Q
__host__ __device__ __forceinline__ double2 green(const DfnPair& t, double ko, double ep, double xp, double eq, double xq) {
  double a[3], b[3];
  tri_point(t.p, ep, xp, a);
  tri_point(t.q, eq, xq, b);
  const double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
  const double R = sqrt(dx * dx + dy * dy + dz * dz);
  double s, c;
  sincos(ko * R, &s, &c);
  const double ir = 1.0 / R;
  return mk<double2>(c * ir, -s * ir);
}

// coincident triangles: sub-triangle rotations (directfn_ws_st_const.cpp:519-538)
__host__ __device__ __forceinline__ void st_rotate(int kk, double& eta, double& xi) {
  if (kk == 0) return;
  const double e = eta, x = xi;
  if (kk == 1) {
    eta = 0.5 - 0.5 * e - 0.5 * kSq3 * x;
    xi = 0.5 * kSq3 + 0.5 * kSq3 * e - 0.5 * x;
  } else {
    eta = -0.5 - 0.5 * e + 0.5 * kSq3 * x;
    xi = 0.5 * kSq3 - 0.5 * kSq3 * e - 0.5 * x;
  }
}

// one work item: returns its contribution (all outer weights applied) on lane 0
__host__ __device__ double2 item_st(const DfnPair& t, double ko, int n, const double* x, const double* w, long long loc,
                           int lane) {
  // loc = ((kk * 8 + m) * n + i) * n + j: sub-triangle kk, subdomain m, psi_i, eta_j
  const int j = (int)(loc % n), i = (int)((loc / n) % n);
  const int m = (int)((loc / ((long long)n * n)) % 8), kk = (int)(loc / (8LL * n * n));
  // psi ranges in units of pi/3 (directfn_ws_st_const.cpp:189-229)
  const int pa = (m == 0 || m == 4 || m == 5) ? 0 : (m == 1 || m == 6) ? 1 : 2;
  const double psA = pa * kPi / 3.0, psB = (pa + 1) * kPi / 3.0;
  const double hps = 0.5 * (psB - psA);
  const double psi = hps * x[i] + 0.5 * (psB + psA);
  const double wps = hps * w[i];
  // eta ranges (:233-287)
  double eA, eB;
  switch (m) {
    case 0: case 1: eA = 0.0; eB = 1.0; break;
    case 2: case 3: {
      const double b1 = tan(kPi - psi) / kSq3, a1 = (1.0 - b1) / (1.0 + b1);
      if (m == 2) { eA = a1; eB = 1.0; } else { eA = 0.0; eB = a1; }
      break;
    }
    case 4: case 5: {
      const double b2 = tan(psi) / kSq3, a2 = -(1.0 - b2) / (1.0 + b2);
      if (m == 4) { eA = a2; eB = 0.0; } else { eA = -1.0; eB = a2; }
      break;
    }
    default: eA = -1.0; eB = 0.0;
  }
  const double het = 0.5 * (eB - eA);
  const double eta = het * x[j] + 0.5 * (eB + eA);
  const double wet = het * w[j];
  double sp, cp;
  sincos(psi, &sp, &cp);
  // radial limit (:291-464): L1 for m = 0, 4; L2 for 1, 2; L3 for 3, 7; L4 for 5, 6
  double Lam;
  if (m == 0 || m == 4) Lam = (1.0 - eta) / cp;
  else if (m == 1 || m == 2) Lam = kSq3 * (1.0 - eta) / sp;
  else if (m == 3 || m == 7) Lam = -(1.0 + eta) / cp;
  else Lam = kSq3 * (1.0 + eta) / sp;
  // inner lambda x rho rule (:468-515): rho in [0, lambda], Jacobian rho
  double2 acc = mk<double2>(0.0, 0.0);
  for (int e = lane; e < n * n; e += 32) {
    const int a = e / n, b = e - a * n;
    const double hl = 0.5 * Lam;
    const double lam = hl * x[a] + hl, wl = hl * w[a];
    const double hr = 0.5 * lam;
    const double rho = hr * x[b] + hr, wr = hr * w[b];
    double ep = eta, xp = lam * sp;
    double eq = rho * cp + ep, xq = -rho * sp + xp;
    st_rotate(kk, ep, xp);
    st_rotate(kk, eq, xq);
    acc = cadd(acc, cscale(green(t, ko, ep, xp, eq, xq), wl * wr * rho));
  }
  return cscale(acc, t.jac * wps * wet * sp);
}

__host__ __device__ double2 item_ea(const DfnPair& t, double ko, int n, const double* x, const double* w, long long loc,
                           int lane) {
  // loc = ((piece * 2 + B) * n + i) * n + j: eta piece of a subdomain, sign branch B, theta_i, psi_j
  const int j = (int)(loc % n), i = (int)((loc / n) % n);
  const int B = (int)((loc / ((long long)n * n)) % 2), piece = (int)(loc / (2LL * n * n));
  // pieces: subdomains 1, 2, 3 have two eta pieces each, 4, 5, 6 one
  const int m = piece < 6 ? piece / 2 : piece - 3;  // 0-based subdomain
  const int half = piece < 6 ? (piece & 1) : 0;
  // theta ranges (directfn_ws_ea_const.cpp:188-218)
  const double h2 = 0.5 * kPi, h3 = kPi / 3.0;
  const double thA = (m == 0 || m == 4) ? 0.0 : (m == 1 || m == 2) ? h3 : h2;
  const double thB = m == 0 ? h3 : (m == 1 || m == 2 || m == 4) ? h2 : kPi;
  const double hth = 0.5 * (thB - thA);
  const double th = hth * x[i] + 0.5 * (thB + thA);
  const double wth = hth * w[i];
  double st, ct;
  sincos(th, &st, &ct);
  // psi ranges (:224-260)
  const double PsA = atan(st - kSq3 * ct), PsB = atan(st + kSq3 * ct);
  double pA, pB;
  switch (m) {
    case 0: pA = 0.0; pB = PsB; break;
    case 1: pA = PsA; pB = PsB; break;
    case 2: case 3: pA = 0.0; pB = PsA; break;
    case 4: pA = PsB; pB = h2; break;
    default: pA = PsA; pB = h2;
  }
  const double hps = 0.5 * (pB - pA);
  const double psi = hps * x[j] + 0.5 * (pB + pA);
  const double wps = hps * w[j];
  double sp, cp;
  sincos(psi, &sp, &cp);
  // eta pieces and their radial limits (:266-456)
  double eA = 0.0, eB = 1.0;
  int lim;  // 1: L1, 2: L2, 3: L3
  if (m <= 1) {
    const double g = tan(psi) / (st + kSq3 * ct), hs = (1.0 - g) / (1.0 + g);
    if (half == 0) { eB = hs; lim = 3; } else { eA = hs; lim = 2; }
  } else if (m == 2) {
    const double hs = kSq3 / tan(th);
    if (half == 0) { eB = hs; lim = 3; } else { eA = hs; lim = 1; }
  } else if (m == 3) {
    lim = 1;
  } else {
    lim = 2;
  }
  const double het = 0.5 * (eB - eA), cet = 0.5 * (eB + eA);
  const double sgn = B == 0 ? 1.0 : -1.0;
  double2 acc = mk<double2>(0.0, 0.0);
  for (int e = lane; e < n * n; e += 32) {
    const int a = e / n, b = e - a * n;
    const double eta = het * x[a] + cet, wet = het * w[a];
    double Lam;
    if (lim == 3) Lam = kSq3 * (1.0 + eta) / (cp * (st + kSq3 * ct));
    else if (lim == 2) Lam = kSq3 * (1.0 - fabs(eta)) / sp;
    else Lam = kSq3 * (1.0 - fabs(eta)) / (cp * (st - kSq3 * ct));
    const double hl = 0.5 * Lam;
    const double lam = hl * x[b] + hl, wl = hl * w[b];
    // parameter points (:504-546), Jacobian lambda^2 (:462-498)
    const double ep = sgn * eta, xp = lam * sp;
    const double eq = sgn * (lam * cp * ct - eta), xq = lam * cp * st;
    acc = cadd(acc, cscale(green(t, ko, ep, xp, eq, xq), wet * wl * lam * lam));
  }
  return cscale(acc, t.jac * wth * wps * cp);
}

__host__ __device__ double2 item_va(const DfnPair& t, double ko, int n, const double* x, const double* w, long long loc,
                           int lane) {
  // loc = (part * n + i) * n + j: psi part, theta_p index i, theta_q index j
  // (directfn_ws_va_const.cpp:129-228)
  const int j = (int)(loc % n), i = (int)((loc / n) % n), part = (int)(loc / ((long long)n * n));
  const double h = kPi / 6.0;  // half-length of [0, pi/3]
  const double tp = h * x[i] + h, tq = h * x[j] + h;
  const double wtp = h * w[i], wtq = h * w[j];
  double stp, ctp, stq, ctq;
  sincos(tp, &stp, &ctp);
  sincos(tq, &stq, &ctq);
  const double Lp = 2.0 * kSq3 / (stp + kSq3 * ctp), Lq = 2.0 * kSq3 / (stq + kSq3 * ctq);
  const double split = atan(Lq / Lp);
  const double pA = part == 0 ? 0.0 : split, pB = part == 0 ? split : 0.5 * kPi;
  const double hps = 0.5 * (pB - pA), cps = 0.5 * (pB + pA);
  double2 acc = mk<double2>(0.0, 0.0);
  for (int e = lane; e < n * n; e += 32) {
    const int a = e / n, b = e - a * n;
    const double psi = hps * x[a] + cps, wps = hps * w[a];
    double sp, cp;
    sincos(psi, &sp, &cp);
    const double Lam = part == 0 ? Lp / cp : Lq / sp;
    const double hl = 0.5 * Lam;
    const double lam = hl * x[b] + hl, wl = hl * w[b];
    // parameter points (:249-266), Jacobian lambda^3 sin(psi) cos(psi)
    const double ep = lam * cp * ctp - 1.0, xp = lam * cp * stp;
    const double eq = lam * sp * ctq - 1.0, xq = lam * sp * stq;
    acc = cadd(acc, cscale(green(t, ko, ep, xp, eq, xq), wps * wl * lam * lam * lam * sp * cp));
  }
  return cscale(acc, t.jac * wtp * wtq);
}

__device__ __forceinline__ double2 warp_sum(double2 v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
  }
  return v;
}

// one warp per work item
__global__ void __launch_bounds__(256) k_directfn_items(const DfnPair* __restrict__ pairs, int npairs, double ko,
                                                         int n, const double* __restrict__ x,
                                                         const double* __restrict__ w, long long total,
                                                         double2* __restrict__ part) {
  const long long item = (long long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (item >= total) return;
  int k = 0;
  while (k + 1 < npairs && pairs[k + 1].first <= item) ++k;
  const DfnPair t = pairs[k];
  const long long loc = item - t.first;
  double2 v;
  if (t.kind == 0) v = item_st(t, ko, n, x, w, loc, lane);
  else if (t.kind == 1) v = item_ea(t, ko, n, x, w, loc, lane);
  else v = item_va(t, ko, n, x, w, loc, lane);
  v = warp_sum(v);
  if (lane == 0) part[item] = v;
}

// one block per output: the items of every pair of that slot, fixed order
__global__ void __launch_bounds__(256) k_directfn_sum(const DfnPair* __restrict__ pairs, int npairs, int n,
                                                       const double2* __restrict__ part, double2* __restrict__ out) {
  const int slot = blockIdx.x;
  double2 acc = mk<double2>(0.0, 0.0);
  for (int k = 0; k < npairs; ++k) {
    if (pairs[k].slot != slot) continue;
    const long long f = pairs[k].first, cnt = items_of(pairs[k].kind, n);
    for (long long i = threadIdx.x; i < cnt; i += blockDim.x) acc = cadd(acc, part[f + i]);
  }
  acc = warp_sum(acc);
  __shared__ double2 ws[8];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double2 s = mk<double2>(0.0, 0.0);
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s = cadd(s, ws[i]);
    out[slot] = s;
  }
}

double tri_jac(const double v[3][3]) {
  double a[3], b[3];
  for (int c = 0; c < 3; ++c) {
    a[c] = v[1][c] - v[0][c];
    b[c] = v[2][c] - v[0][c];
  }
  const double cx = a[1] * b[2] - a[2] * b[1], cy = a[2] * b[0] - a[0] * b[2], cz = a[0] * b[1] - a[1] * b[0];
  return 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz) / kSq3;
}

using Vec3 = std::array<double, 3>;

DfnPair make_pair(int kind, int slot, const Vec3& p1, const Vec3& p2, const Vec3& p3, const Vec3& q1, const Vec3& q2,
                  const Vec3& q3) {
  DfnPair t{};
  const Vec3* P[3] = {&p1, &p2, &p3};
  const Vec3* Q[3] = {&q1, &q2, &q3};
  for (int i = 0; i < 3; ++i)
    for (int c = 0; c < 3; ++c) {
      t.p[i][c] = (*P[i])[c];
      t.q[i][c] = (*Q[i])[c];
    }
  t.jac = tri_jac(t.p) * tri_jac(t.q);
  t.kind = kind;
  t.slot = slot;
  return t;
}

// the MEX gateways' vertex orders (directfn_ws_{st,ea,va}_const_mex.cpp)
DfnPair gw_st(int slot, const Vec3& r1, const Vec3& r2, const Vec3& r3) {
  return make_pair(0, slot, r1, r2, r3, r1, r2, r3);
}
DfnPair gw_ea(int slot, const Vec3& r1, const Vec3& r2, const Vec3& r3, const Vec3& r4) {
  return make_pair(1, slot, r1, r2, r3, r4, r2, r1);
}
DfnPair gw_va(int slot, const Vec3& r1, const Vec3& r2, const Vec3& r3, const Vec3& r4, const Vec3& r5) {
  return make_pair(2, slot, r1, r2, r3, r4, r5, r1);
}

int run_pairs(std::vector<DfnPair>& pairs, int nslots, double ko, int n, double2* out, cudaStream_t st) {
  long long total = 0;
  for (auto& t : pairs) {
    t.first = total;
    total += items_of(t.kind, n);
  }
  std::vector<double> x, w;
  gauss_legendre(n, x, w);
  const size_t pb = pairs.size() * sizeof(DfnPair);
  DBuf dp, dxw, dpart, dout;
  MARIE_TRY(dp.alloc(pb, st));
  MARIE_TRY(dxw.alloc(2 * n * sizeof(double), st));
  MARIE_TRY(dpart.alloc(total * sizeof(double2), st));
  MARIE_TRY(dout.alloc(nslots * sizeof(double2), st));
  std::vector<double> xw(x);
  xw.insert(xw.end(), w.begin(), w.end());
  MARIE_CUDA_TRY(cudaMemcpyAsync(dp.p, pairs.data(), pb, cudaMemcpyHostToDevice, st));
  MARIE_CUDA_TRY(cudaMemcpyAsync(dxw.p, xw.data(), xw.size() * sizeof(double), cudaMemcpyHostToDevice, st));
  const unsigned blocks = (unsigned)((total + 7) / 8);
  k_directfn_items<<<blocks, 256, 0, st>>>(dp.as<DfnPair>(), (int)pairs.size(), ko, n, dxw.as<double>(),
                                          dxw.as<double>() + n, total, dpart.as<double2>());
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  k_directfn_sum<<<nslots, 256, 0, st>>>(dp.as<DfnPair>(), (int)pairs.size(), n, dpart.as<double2>(),
                                        dout.as<double2>());
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  std::vector<double2> h(nslots);
  MARIE_CUDA_TRY(cudaMemcpyAsync(h.data(), dout.p, nslots * sizeof(double2), cudaMemcpyDeviceToHost, st));
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  for (int s = 0; s < nslots; ++s) out[s] = h[s];
  return MARIE_OK;
}

}  // namespace

bool directfn_order_ok(int n) { return n >= 1 && n <= kDirectfnMaxOrder; }

// The 20 triangle-pair calls of singular_st/ea/va.m for cubic voxels of edge
// d, each adding to its output slot (0 ST, 1 EAc, 2 EAo, 3 VAc, 4 VAo).
static std::vector<DfnPair> square_pairs(double d) {
  const Vec3 r1{0, 0, 0}, r2{d, 0, 0}, r3{d, d, 0}, r4{0, d, 0};
  std::vector<DfnPair> P;
  // ST, singular_st.m:14-17
  P.push_back(gw_st(0, r1, r2, r3));
  P.push_back(gw_ea(0, r1, r3, r2, r4));
  P.push_back(gw_ea(0, r1, r3, r4, r2));
  P.push_back(gw_st(0, r1, r3, r4));
  // EAc, EAo, singular_ea.m:17-28
  const Vec3 e5{2 * d, 0, 0}, e6{2 * d, d, 0}, e5o{d, 0, d}, e6o{d, d, d};
  for (int o = 0; o < 2; ++o) {
    const Vec3& a = o ? e5o : e5;
    const Vec3& b = o ? e6o : e6;
    P.push_back(gw_ea(1 + o, r2, r3, r1, a));
    P.push_back(gw_va(1 + o, r3, r1, r2, a, b));
    P.push_back(gw_va(1 + o, r3, r4, r1, r2, a));
    P.push_back(gw_va(1 + o, r3, r4, r1, a, b));
  }
  // VAc, VAo, singular_va.m:20-34
  const Vec3 v5{2 * d, d, 0}, v6{2 * d, 2 * d, 0}, v7{d, 2 * d, 0};
  const Vec3 v5o{d, d, d}, v6o{d, 2 * d, d}, v7o{d, 2 * d, 0};
  for (int o = 0; o < 2; ++o) {
    const Vec3& a = o ? v5o : v5;
    const Vec3& b = o ? v6o : v6;
    const Vec3& c = o ? v7o : v7;
    P.push_back(gw_va(3 + o, r3, r1, r2, a, b));
    P.push_back(gw_va(3 + o, r3, r1, r2, b, c));
    P.push_back(gw_va(3 + o, r3, r4, r1, a, b));
    P.push_back(gw_va(3 + o, r3, r4, r1, b, c));
  }
  return P;
}

int directfn_integrals(double ko, double dx, int n, double2 out[5], cudaStream_t st) {
  if (!directfn_order_ok(n)) return set_error(MARIE_EINVAL, "Np_1D must be in [1, %d]", kDirectfnMaxOrder);
  std::vector<DfnPair> P = square_pairs(dx);
  return run_pairs(P, 5, ko, n, out, st);
}

int directfn_single(char kind, const double* r, double ko, int n, double2* out, cudaStream_t st) {
  if (!directfn_order_ok(n)) return set_error(MARIE_EINVAL, "Np_1D must be in [1, %d]", kDirectfnMaxOrder);
  Vec3 v[5];
  const int nv = kind == 'S' ? 3 : kind == 'E' ? 4 : kind == 'V' ? 5 : 0;
  if (!nv) return set_error(MARIE_EINVAL, "kind must be 'S', 'E' or 'V'");
  for (int i = 0; i < nv; ++i) v[i] = Vec3{r[3 * i], r[3 * i + 1], r[3 * i + 2]};
  std::vector<DfnPair> P;
  if (kind == 'S') P.push_back(gw_st(0, v[0], v[1], v[2]));
  else if (kind == 'E') P.push_back(gw_ea(0, v[0], v[1], v[2], v[3]));
  else P.push_back(gw_va(0, v[0], v[1], v[2], v[3], v[4]));
  return run_pairs(P, 1, ko, n, out, st);
}

}  // namespace marie

using namespace marie;

extern "C" int marie_directfn(char kind, const double* vertices, double ko, int np_1d, double* out2) {
  if (!vertices || !out2) return set_error(MARIE_EINVAL, "NULL argument");
  double2 v;
  MARIE_TRY(directfn_single(kind, vertices, ko, np_1d, &v, 0));
  out2[0] = v.x;
  out2[1] = v.y;
  return MARIE_OK;
}
