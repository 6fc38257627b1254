// JVIE_Solver (src_vie/src_solver/JVIE_Solver.m:1-521, solver 'G'), the total
// field E_field_Nop (src_vie/src_fields/src_op/E_field_Nop.m:59-84) and the
// incident-field generators (PlaneWave_Excitation.m:39-95, E_field_DGF.m:36-99),
// all on the device.
#include <chrono>
#include <cmath>
#include <vector>

#include "plan.h"

namespace marie {

// EMconstants.m:13-20
static constexpr double MU0 = 4e-7 * M_PI;
static constexpr double C0 = 299792458.0;
static inline double eps0() { return 1.0 / (C0 * C0 * MU0); }

static inline int grid_n(long long n) {
  long long g = (n + 255) / 256;
  if (g > 152 * 8) g = 152 * 8;
  return g < 1 ? 1 : (int)g;
}

// ---------------------------------------------------------------------------
// non-air voxel compaction: idxS = find(abs(Mc(:)) > 1e-12), in order
// ---------------------------------------------------------------------------
static constexpr int CMP_BLOCKS = 1024;

__device__ __forceinline__ bool non_air(const double2* er, long long v) {
  const double2 e = er[v];
  const double mx = e.x - 1.0, my = e.y;
  return sqrt(mx * mx + my * my) > 1e-12;
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
//   idx3[k]  = c*V + idxS[s] + 1                     (1-based, JVIE_Solver.m:148)
//   rhs[k]   = Gram * j*omega*eps0 * Mc * Einc        (JVIE_Solver.m:151-156)
//   form 2:  Mc <- Mc/Mr, rhs <- rhs/Mr, Mr <- 1      (JVIE_Solver.m:242-244)
//   a = Gram*Mr, b = Mc ; preconditioner pa = Gram/Mr, pb = 1/Mr - 1
__global__ void k_jvie_setup(const int* __restrict__ idxS, long long nS, long long V, const double2* __restrict__ er,
                             const double2* __restrict__ Einc, double Gram, double omega_eps0, int form,
                             int64_t* __restrict__ idx3, double2* __restrict__ rhs, double2* __restrict__ a,
                             double2* __restrict__ b, double2* __restrict__ pa, double2* __restrict__ pb) {
  const long long n = 3 * nS;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const long long c = k / nS, s = k - c * nS;
    const long long v = idxS[s];
    const long long g = c * V + v;
    idx3[k] = g + 1;
    double2 mr = er[v];
    double2 mc = mk<double2>(mr.x - 1.0, mr.y);
    const double2 tau = mk<double2>(-omega_eps0 * mc.y, omega_eps0 * mc.x);  // j*omega*eps0*Mc
    double2 r = cmul(tau, Einc[g]);
    r = mk<double2>(Gram * r.x, Gram * r.y);
    if (form != 1) {
      const double den = mr.x * mr.x + mr.y * mr.y;
      const double2 inv_mr = mk<double2>(mr.x / den, -mr.y / den);
      mc = cmul(mc, inv_mr);
      r = cmul(r, inv_mr);
      mr = mk<double2>(1.0, 0.0);
    }
    rhs[k] = r;
    a[k] = mk<double2>(Gram * mr.x, Gram * mr.y);
    b[k] = mc;
    const double den = mr.x * mr.x + mr.y * mr.y;
    const double2 imr = mk<double2>(mr.x / den, -mr.y / den);
    pa[k] = mk<double2>(Gram * imr.x, Gram * imr.y);
    pb[k] = mk<double2>(imr.x - 1.0, imr.y);
  }
}

__global__ void k_scatter_dofs(const double2* __restrict__ x, const int64_t* __restrict__ idx3, long long n,
                               double2* __restrict__ out) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    out[idx3[k] - 1] = x[k];
}

__global__ void k_diag_apply(const double2* __restrict__ a, const double2* __restrict__ x, double2* __restrict__ y,
                             long long n) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    y[k] = cmul(a[k], x[k]);
}

__global__ void k_all_zero(const double2* __restrict__ b, long long n, int* __restrict__ nonzero) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    if (b[k].x != 0.0 || b[k].y != 0.0) *nonzero = 1;
}

__global__ void k_identity_index(int* __restrict__ inv, long long n) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    inv[k] = (int)k;
}

__global__ void k_add_field(const double2* __restrict__ einc, double2* __restrict__ e, long long n) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    e[k] = cadd(e[k], einc[k]);
}

__global__ void k_sub(const double2* __restrict__ b, double2* __restrict__ y, long long n) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    y[k] = csub(b[k], y[k]);
}
__global__ void k_axpy1(const double2* __restrict__ x, double2* __restrict__ y, long long n) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    y[k] = cadd(y[k], x[k]);
}

// ---------------------------------------------------------------------------
// incident fields
// ---------------------------------------------------------------------------
// PlaneWave_Excitation.m:62-95: product of voxel-averaged 1-D factors, / (dx dy dz)
__global__ void k_plane_wave(const double* __restrict__ r, long long L, long long M, long long N, double kx, double ky,
                             double kz, double2 e0x, double2 e0y, double2 e0z, double dx, double dy, double dz,
                             double2* __restrict__ E) {
  const long long V = L * M * N;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
    const double kk[3] = {kx, ky, kz};
    const double dd[3] = {dx, dy, dz};
    double2 f = mk<double2>(1.0, 0.0);
    for (int a = 0; a < 3; ++a) {
      double2 fa;
      if (kk[a] != 0.0) {
        // exp(-j k r) * (exp(-j k d/2) - exp(j k d/2)) / (-j k) = exp(-j k r) * 2 sin(k d/2) / k
        double sr, cr;
        sincos(kk[a] * r[a * V + v], &sr, &cr);
        const double s = 2.0 * sin(kk[a] * dd[a] * 0.5) / kk[a];
        fa = mk<double2>(cr * s, -sr * s);
      } else {
        fa = mk<double2>(dd[a], 0.0);
      }
      f = cmul(f, fa);
    }
    const double inv = 1.0 / (dx * dy * dz);
    f = mk<double2>(f.x * inv, f.y * inv);
    E[v] = cmul(e0x, f);
    E[V + v] = cmul(e0y, f);
    E[2 * V + v] = cmul(e0z, f);
  }
}

// E_field_DGF.m:77-99, point-sampled dyadic Green function of electric dipoles
__global__ void k_dipole_field(const double* __restrict__ r, long long V, double ko, const double2* __restrict__ Jd,
                               const double* __restrict__ pos, int ndip, double2* __restrict__ E) {
  const double omega = ko * C0;
  for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += (long long)gridDim.x * blockDim.x) {
    double2 ex = mk<double2>(0, 0), ey = ex, ez = ex;
    const double ox = r[v], oy = r[V + v], oz = r[2 * V + v];
    for (int j = 0; j < ndip; ++j) {
      const double X = ox - pos[3 * j], Y = oy - pos[3 * j + 1], Z = oz - pos[3 * j + 2];
      const double R2 = X * X + Y * Y + Z * Z;
      const double R = sqrt(R2);
      const double R3 = R * R2;
      double sn, cs;
      sincos(ko * R, &sn, &cs);
      // chi = j*omega*mu*exp(-j ko R) / (4 pi ko^2 R^3)
      const double amp = omega * MU0 / (4.0 * M_PI * ko * ko * R3);
      const double2 chi = mk<double2>(amp * sn, amp * cs);
      const double2 P0 = mk<double2>(1.0, ko * R);           // P = j ko R + 1
      const double2 Q = mk<double2>(ko * ko * R2 - 1.0, -ko * R);  // Q = ko^2 R^2 - P
      const double2 Pn = mk<double2>((Q.x - 2.0 * P0.x) / R2, (Q.y - 2.0 * P0.y) / R2);
      const double2 Qc = cmul(chi, Q), Pc = cmul(chi, Pn);
      const double2 jx = Jd[3 * j], jy = Jd[3 * j + 1], jz = Jd[3 * j + 2];
      const double2 pxx = mk<double2>(Pc.x * X * X - Qc.x, Pc.y * X * X - Qc.y);
      const double2 pyy = mk<double2>(Pc.x * Y * Y - Qc.x, Pc.y * Y * Y - Qc.y);
      const double2 pzz = mk<double2>(Pc.x * Z * Z - Qc.x, Pc.y * Z * Z - Qc.y);
      const double2 pxy = cscale(Pc, X * Y), pxz = cscale(Pc, X * Z), pyz = cscale(Pc, Y * Z);
      ex = cadd(ex, cadd(cadd(cmul(pxx, jx), cmul(pxy, jy)), cmul(pxz, jz)));
      ey = cadd(ey, cadd(cadd(cmul(pxy, jx), cmul(pyy, jy)), cmul(pyz, jz)));
      ez = cadd(ez, cadd(cadd(cmul(pxz, jx), cmul(pyz, jy)), cmul(pzz, jz)));
    }
    E[v] = ex;
    E[V + v] = ey;
    E[2 * V + v] = ez;
  }
}

// ---------------------------------------------------------------------------
// J-VIE solve
// ---------------------------------------------------------------------------
struct JvieState {
  long long nS = 0, n = 0;
  DBuf idxS, idx3, inv, rhs, a, b, pa, pb;
};

static int jvie_setup(marie_plan* p, const double2* er, const double2* Einc, double dx, double freq, int form,
                      JvieState& S) {
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
  MARIE_TRY(S.rhs.alloc(n * sizeof(double2), st));
  MARIE_TRY(S.a.alloc(n * sizeof(double2), st));
  MARIE_TRY(S.b.alloc(n * sizeof(double2), st));
  MARIE_TRY(S.pa.alloc(n * sizeof(double2), st));
  MARIE_TRY(S.pb.alloc(n * sizeof(double2), st));
  MARIE_TRY(S.inv.alloc(3 * V * sizeof(int), st));
  const double Gram = dx * dx * dx;
  const double omega = 2.0 * M_PI * freq;
  k_jvie_setup<<<grid_n(n), 256, 0, st>>>(S.idxS.as<int>(), tot, V, er, Einc, Gram, omega * eps0(), form,
                                          S.idx3.as<int64_t>(), S.rhs.as<double2>(), S.a.as<double2>(),
                                          S.b.as<double2>(), S.pa.as<double2>(), S.pb.as<double2>());
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  MARIE_TRY(build_inverse_index(p, S.idx3.as<int64_t>(), n, S.inv.as<int>()));
  return MARIE_OK;
}

static int all_zero(marie_plan* p, const double2* b, long long n, bool* z) {
  DBuf f;
  MARIE_TRY(f.alloc(sizeof(int), p->stream));
  MARIE_CUDA_TRY(cudaMemsetAsync(f.p, 0, sizeof(int), p->stream));
  k_all_zero<<<grid_n(n), 256, 0, p->stream>>>(b, n, f.as<int>());
  count_launch();
  int h = 0;
  MARIE_CUDA_TRY(cudaMemcpyAsync(&h, f.p, sizeof(int), cudaMemcpyDeviceToHost, p->stream));
  MARIE_CUDA_TRY(cudaStreamSynchronize(p->stream));
  *z = (h == 0);
  return MARIE_OK;
}

// mv_AN operator on the solver's DOFs with coefficient arrays (a, b); a b that is
// identically zero reduces to the diagonal Gram*Mr product (the circulant
// term is multiplied by zero in mv_AN.m:127-131).
static DevOp make_op(marie_plan* p, int prec, const JvieState& S, const double2* a, const double2* b, bool diag_only) {
  const long long n = S.n;
  const int* inv = S.inv.as<int>();
  return [p, prec, n, inv, a, b, diag_only](const double2* x, double2* y) -> int {
    if (diag_only) {
      k_diag_apply<<<grid_n(n), 256, 0, p->stream>>>(a, x, y, n);
      count_launch();
      MARIE_CUDA_TRY(cudaGetLastError());
      return MARIE_OK;
    }
    Prologue pro{nullptr, 0};
    Epilogue ep{};
    ep.a = a;
    ep.b = b;
    return run_matvec(p, prec, x, y, n, 1, inv, pro, ep);
  };
}

}  // namespace marie

using namespace marie;

extern "C" {

int marie_jvie_solve(marie_plan* p, const double* Einc, const double* e_r, double dx, double freq, int form,
                     char precond, double tol, int inner_it, int outer_it, double* Je, int* flag, double* relres,
                     int* iter, double* resvec, int64_t resvec_cap, int64_t* resvec_len, double* solvert) {
  if (!p || !Einc || !e_r || !Je) return set_error(MARIE_EINVAL, "NULL argument");
  if (!p->has_op) return set_error(MARIE_ENOOP, "plan has no operator");
  if (!(dx > 0) || !(freq > 0)) return set_error(MARIE_EINVAL, "dx and freq must be positive");
  // JVIE_Solver.m:71-122 argument clamps
  if (tol < 1e-15 || tol >= 1) tol = 1e-3;
  if (form != 1) form = 2;
  if (precond != 'L' && precond != 'R') precond = 0;
  if (inner_it < 1) inner_it = 50;
  if (outer_it < 1) outer_it = 200;
  const auto t0 = std::chrono::steady_clock::now();
  cudaStream_t st = p->stream;
  const long long V = p->d.V;
  DBuf tE, tER, tJe;
  const void *E_d, *er_d;
  void* Je_d;
  MARIE_TRY(stage_in(Einc, 3 * V * sizeof(double2), st, tE, &E_d));
  MARIE_TRY(stage_in(e_r, V * sizeof(double2), st, tER, &er_d));
  MARIE_TRY(stage_out(Je, 3 * V * sizeof(double2), st, tJe, &Je_d));
  JvieState S;
  MARIE_TRY(jvie_setup(p, (const double2*)er_d, (const double2*)E_d, dx, freq, form, S));
  MARIE_CUDA_TRY(cudaMemsetAsync(Je_d, 0, 3 * V * sizeof(double2), st));
  GmresResult R;
  std::vector<double> rv;
  if (S.n > 0) {
    const long long n = S.n;
    bool pb_zero = false;
    MARIE_TRY(all_zero(p, S.pb.as<double2>(), n, &pb_zero));
    const int prec_main = (p->precision == MARIE_FP32) ? MARIE_FP32 : MARIE_FP64;
    DevOp A64 = make_op(p, prec_main, S, S.a.as<double2>(), S.b.as<double2>(), false);
    DevOp P64 = make_op(p, prec_main, S, S.pa.as<double2>(), S.pb.as<double2>(), pb_zero);
    DBuf x;
    MARIE_TRY(x.alloc(n * sizeof(double2), st));
    const DevOp* L1 = precond == 'L' ? &P64 : nullptr;
    const DevOp* R1 = precond == 'R' ? &P64 : nullptr;
    if (p->precision != MARIE_MIXED) {
      MARIE_TRY(gmres(p, A64, L1, nullptr, R1, nullptr, S.rhs.as<double2>(), n, inner_it, tol, outer_it, nullptr,
                      x.as<double2>(), R));
      rv = R.resvec;
    } else {
      // FP32 circulant matvec inside FP64 GMRES, refined with FP64 residuals.
      DevOp A32 = make_op(p, MARIE_FP32, S, S.a.as<double2>(), S.b.as<double2>(), false);
      DevOp P32 = make_op(p, MARIE_FP32, S, S.pa.as<double2>(), S.pb.as<double2>(), pb_zero);
      const DevOp* L1m = precond == 'L' ? &P32 : nullptr;
      const DevOp* R1m = precond == 'R' ? &P32 : nullptr;
      DBuf r, d;
      MARIE_TRY(r.alloc(n * sizeof(double2), st));
      MARIE_TRY(d.alloc(n * sizeof(double2), st));
      const double2* b = S.rhs.as<double2>();
      MARIE_CUDA_TRY(cudaMemsetAsync(x.p, 0, n * sizeof(double2), st));
      MARIE_CUDA_TRY(cudaMemcpyAsync(r.p, b, n * sizeof(double2), cudaMemcpyDeviceToDevice, st));
      double bn = 0, rn = 0;
      MARIE_TRY(dev_norm2(p, b, n, &bn));
      rn = bn;
      rv.push_back(rn / bn);
      int outer = 0, inner_total = 0, last_p = 0;
      R.relres = rn / bn;
      const int max_refine = 20;
      while (R.relres > tol && outer < max_refine) {
        ++outer;
        // inner target: half of what is still missing, not below the FP32 floor
        double inner_tol = 0.5 * tol * bn / rn;
        if (inner_tol < 1e-5) inner_tol = 1e-5;
        if (inner_tol > 0.5) inner_tol = 0.5;
        GmresResult Ri;
        MARIE_TRY(gmres(p, A32, L1m, nullptr, R1m, nullptr, r.as<double2>(), n, inner_it, inner_tol, outer_it,
                        nullptr, d.as<double2>(), Ri));
        for (size_t i = 1; i < Ri.resvec.size(); ++i) rv.push_back(Ri.resvec[i] * rn / bn);
        inner_total += Ri.iter[1];
        last_p = Ri.iter[0];
        k_axpy1<<<grid_n(n), 256, 0, st>>>(d.as<double2>(), x.as<double2>(), n);
        count_launch();
        // r = b - A64 x in FP64 (with the left preconditioner when asked, as pgmres does)
        MARIE_TRY(A64(x.as<double2>(), r.as<double2>()));
        k_sub<<<grid_n(n), 256, 0, st>>>(b, r.as<double2>(), n);
        count_launch();
        MARIE_CUDA_TRY(cudaGetLastError());
        MARIE_TRY(dev_norm2(p, r.as<double2>(), n, &rn));
        R.relres = rn / bn;
        rv.push_back(R.relres);
      }
      R.flag = R.relres <= tol ? 0 : 1;
      R.iter[0] = last_p;
      R.iter[1] = inner_total;
    }
    k_scatter_dofs<<<grid_n(n), 256, 0, st>>>(x.as<double2>(), S.idx3.as<int64_t>(), n, (double2*)Je_d);
    count_launch();
    MARIE_CUDA_TRY(cudaGetLastError());
  } else {
    R.flag = 0;
    R.relres = 0;
  }
  MARIE_TRY(finish_out(Je, Je_d, 3 * V * sizeof(double2), st));
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  const auto t1 = std::chrono::steady_clock::now();
  if (flag) *flag = R.flag;
  if (relres) *relres = R.relres;
  if (iter) {
    iter[0] = R.iter[0];
    iter[1] = R.iter[1];
  }
  if (resvec_len) *resvec_len = (int64_t)rv.size();
  if (resvec)
    for (int64_t i = 0; i < (int64_t)rv.size() && i < resvec_cap; ++i) resvec[i] = rv[i];
  if (solvert) *solvert = std::chrono::duration<double>(t1 - t0).count();
  return MARIE_OK;
}

int marie_e_field_nop(marie_plan* p, const double* J, double Gram, double freq, const double* Einc, double* Etot,
                      int precision) {
  if (!p || !J || !Etot) return set_error(MARIE_EINVAL, "NULL argument");
  if (precision != MARIE_FP64 && precision != MARIE_FP32) return set_error(MARIE_EINVAL, "bad precision");
  if (!p->has_op) return set_error(MARIE_ENOOP, "plan has no operator");
  cudaStream_t st = p->stream;
  const long long n = 3 * p->d.V;
  DBuf tJ, tE, tO, inv;
  const void *J_d, *E_d = nullptr;
  void* O_d;
  MARIE_TRY(stage_in(J, n * sizeof(double2), st, tJ, &J_d));
  if (Einc) MARIE_TRY(stage_in(Einc, n * sizeof(double2), st, tE, &E_d));
  MARIE_TRY(stage_out(Etot, n * sizeof(double2), st, tO, &O_d));
  MARIE_TRY(inv.alloc(n * sizeof(int), st));
  k_identity_index<<<grid_n(n), 256, 0, st>>>(inv.as<int>(), n);
  count_launch();
  // out = s*(N J - Gram J), s = 1/(Gram*j*omega*eps0) = -j/(Gram*omega*eps0)
  const double omega = 2.0 * M_PI * freq;
  const double2 s = mk<double2>(0.0, -1.0 / (Gram * omega * eps0()));
  Prologue pro{nullptr, 0};
  Epilogue ep{};
  ep.a_s = mk<double2>(-Gram * s.x, -Gram * s.y);
  ep.b_s = mk<double2>(-s.x, -s.y);
  MARIE_TRY(run_matvec(p, precision, (const double2*)J_d, (double2*)O_d, n, 1, inv.as<int>(), pro, ep));
  if (Einc) {
    k_add_field<<<grid_n(n), 256, 0, st>>>((const double2*)E_d, (double2*)O_d, n);
    count_launch();
  }
  MARIE_CUDA_TRY(cudaGetLastError());
  MARIE_TRY(finish_out(Etot, O_d, n * sizeof(double2), st));
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  return MARIE_OK;
}

int marie_plane_wave(const double* r, int64_t L, int64_t M, int64_t N, const double* k, const double* Eo,
                     double* E) {
  if (!r || !k || !Eo || !E || L < 2 || M < 2 || N < 2) return set_error(MARIE_EINVAL, "bad argument");
  cudaStream_t st = 0;
  const long long V = L * M * N;
  DBuf tr, tE;
  const void* r_d;
  void* E_d;
  MARIE_TRY(stage_in(r, 3 * V * sizeof(double), st, tr, &r_d));
  MARIE_TRY(stage_out(E, 3 * V * sizeof(double2), st, tE, &E_d));
  // PlaneWave_Excitation.m:45-47 spacing from the first neighbours of each axis
  std::vector<double> rh(3 * 3);
  const long long offs[3][2] = {{0, 1}, {V, V + L}, {2 * V, 2 * V + L * M}};
  for (int a = 0; a < 3; ++a) {
    MARIE_CUDA_TRY(cudaMemcpy(&rh[2 * a], (const double*)r_d + offs[a][0], sizeof(double), cudaMemcpyDefault));
    MARIE_CUDA_TRY(cudaMemcpy(&rh[2 * a + 1], (const double*)r_d + offs[a][1], sizeof(double), cudaMemcpyDefault));
  }
  const double dx = rh[1] - rh[0], dy = rh[3] - rh[2], dz = rh[5] - rh[4];
  k_plane_wave<<<grid_n(V), 256, 0, st>>>((const double*)r_d, L, M, N, k[0], k[1], k[2], mk<double2>(Eo[0], Eo[1]),
                                           mk<double2>(Eo[2], Eo[3]), mk<double2>(Eo[4], Eo[5]), dx, dy, dz,
                                           (double2*)E_d);
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  MARIE_TRY(finish_out(E, E_d, 3 * V * sizeof(double2), st));
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  return MARIE_OK;
}

int marie_dipole_field(const double* r, int64_t L, int64_t M, int64_t N, double ko, const double* Jd,
                       const double* pos, int64_t ndip, double* E) {
  if (!r || !Jd || !pos || !E || ndip < 1) return set_error(MARIE_EINVAL, "bad argument");
  cudaStream_t st = 0;
  const long long V = L * M * N;
  DBuf tr, tJ, tP, tE;
  const void *r_d, *J_d, *P_d;
  void* E_d;
  MARIE_TRY(stage_in(r, 3 * V * sizeof(double), st, tr, &r_d));
  MARIE_TRY(stage_in(Jd, 3 * ndip * sizeof(double2), st, tJ, &J_d));
  MARIE_TRY(stage_in(pos, 3 * ndip * sizeof(double), st, tP, &P_d));
  MARIE_TRY(stage_out(E, 3 * V * sizeof(double2), st, tE, &E_d));
  k_dipole_field<<<grid_n(V), 256, 0, st>>>((const double*)r_d, V, ko, (const double2*)J_d, (const double*)P_d,
                                             (int)ndip, (double2*)E_d);
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  MARIE_TRY(finish_out(E, E_d, 3 * V * sizeof(double2), st));
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  return MARIE_OK;
}

}  // extern "C"
