// Fields on the device: the total field E_field_Nop
// (src_vie/src_fields/src_op/E_field_Nop.m:59-84) and the incident-field
// generators PlaneWave_Excitation.m:39-95 and E_field_DGF.m:36-99.
#include <cmath>
#include <vector>

#include "plan.h"

namespace marie {

// EMconstants.m:13-20
static constexpr double MU0 = 4e-7 * M_PI;
static constexpr double C0 = 299792458.0;
static inline double eps0() { return 1.0 / (C0 * C0 * MU0); }

static inline int grid_n(long long n) { return grid_stride_blocks(n, 8); }

__global__ void k_identity_index(int* __restrict__ inv, long long n) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    inv[k] = (int)k;
}

__global__ void k_add_field(const double2* __restrict__ einc, double2* __restrict__ e, long long n) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    e[k] = cadd(e[k], einc[k]);
}

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
      const double2 P0 = mk<double2>(1.0, ko * R);                 // P = j ko R + 1
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

}  // namespace marie

using namespace marie;

extern "C" {

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
  return check_kernel_status(p);
}

int marie_h_field_kop(marie_plan* p, const double* J, double Gram, const double* Hinc, double* Htot,
                      int precision) {
  if (!p || !J || !Htot) return set_error(MARIE_EINVAL, "NULL argument");
  if (precision != MARIE_FP64 && precision != MARIE_FP32) return set_error(MARIE_EINVAL, "bad precision");
  if (!p->has_opK) return set_error(MARIE_ENOOP, "plan has no K operator");
  cudaStream_t st = p->stream;
  const long long n = 3 * p->d.V;
  DBuf tJ, tH, tO, inv;
  const void *J_d, *H_d = nullptr;
  void* O_d;
  MARIE_TRY(stage_in(J, n * sizeof(double2), st, tJ, &J_d));
  if (Hinc) MARIE_TRY(stage_in(Hinc, n * sizeof(double2), st, tH, &H_d));
  MARIE_TRY(stage_out(Htot, n * sizeof(double2), st, tO, &O_d));
  MARIE_TRY(inv.alloc(n * sizeof(int), st));
  k_identity_index<<<grid_n(n), 256, 0, st>>>(inv.as<int>(), n);
  count_launch();
  // out = mv_K(J) / Gram (H_field_Kop.m:74-76)
  Prologue pro{nullptr, 0};
  Epilogue ep{};
  ep.a_s = mk<double2>(0.0, 0.0);
  ep.b_s = mk<double2>(-1.0 / Gram, 0.0);
  MARIE_TRY(run_matvec(p, precision, (const double2*)J_d, n, (double2*)O_d, n, n, 1, inv.as<int>(), pro, ep,
                       nullptr, 0, 1));
  if (Hinc) {
    k_add_field<<<grid_n(n), 256, 0, st>>>((const double2*)H_d, (double2*)O_d, n);
    count_launch();
  }
  MARIE_CUDA_TRY(cudaGetLastError());
  MARIE_TRY(finish_out(Htot, O_d, n * sizeof(double2), st));
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
