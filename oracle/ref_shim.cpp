// extern "C" shims around the reference C++ cubature cores, so that the oracle
// can call them through ctypes.  TEST INFRASTRUCTURE ONLY: built into
// oracle/_ref/ from the reference sources where they lie (oracle/Makefile),
// never linked into the product library.
//
// One shared object is built per reference core because the three DIRECTFN
// translation units define clashing non-static symbols (GL_1D, Kernel, ...).
// The argument order follows the MEX gateways:
//   cubature_nop_mex.cpp:29-78   (Np, w, u, v, r_m, r_n, R_faces[3][4][6], ko, dx)
//   cubature_kop_mex.cpp          (Np, w, u, v, r_m, r_n, R_faces[3][4][6], ko)
//   directfn_ws_st_const_mex.cpp (r1, r2, r3, ko, Np_1D)
//   directfn_ws_ea_const_mex.cpp:50 passes (r1, r2, r3, r4, r2, r1, ko, Np_1D)
//   directfn_ws_va_const_mex.cpp:51 passes (r1, r2, r3, r4, r5, r1, ko, Np_1D)
#include <complex>
using std::complex;

#if defined(SHIM_CUBATURE_NOP)
void cubature_nop(const int Np, const double w[], const double u[], const double v[],
                  const double r_m[3], const double r_n[3], const double R_faces[3][4][6],
                  const double ko, const double dx, complex<double> I_mn[6][6]);
// R_faces_colmajor: MATLAB 3x4x6 array, column-major (as the gateway receives it).
// out: 6x6 complex, row-major [obs][src] as (re, im) pairs.
extern "C" void ref_cubature_nop(int Np, const double* w, const double* u, const double* v,
                                 const double* r_m, const double* r_n,
                                 const double* R_faces_colmajor, double ko, double dx,
                                 double* out) {
  double RR[3][4][6];
  for (int k = 0; k < 6; k++)
    for (int j = 0; j < 4; j++)
      for (int i = 0; i < 3; i++) RR[i][j][k] = R_faces_colmajor[i + 3 * j + 12 * k];
  complex<double> I[6][6];
  cubature_nop(Np, w, u, v, r_m, r_n, RR, ko, dx, I);
  for (int i = 0; i < 6; i++)
    for (int j = 0; j < 6; j++) {
      out[2 * (6 * i + j)] = I[i][j].real();
      out[2 * (6 * i + j) + 1] = I[i][j].imag();
    }
}
#endif

#if defined(SHIM_CUBATURE_KOP)
void cubature_kop(const int Np, const double w[], const double u[], const double v[], const double r_m[3],
                  const double r_n[3], const double R_faces[3][4][6], const double ko, complex<double> IK_mn[3]);
// out: 3 complex as (re, im) pairs
extern "C" void ref_cubature_kop(int Np, const double* w, const double* u, const double* v,
                                 const double* r_m, const double* r_n,
                                 const double* R_faces_colmajor, double ko, double* out) {
  double RR[3][4][6];
  for (int k = 0; k < 6; k++)
    for (int j = 0; j < 4; j++)
      for (int i = 0; i < 3; i++) RR[i][j][k] = R_faces_colmajor[i + 3 * j + 12 * k];
  complex<double> I[3];
  cubature_kop(Np, w, u, v, r_m, r_n, RR, ko, I);
  for (int i = 0; i < 3; i++) {
    out[2 * i] = I[i].real();
    out[2 * i + 1] = I[i].imag();
  }
}
#endif

#if defined(SHIM_DIRECTFN_ST)
complex<double> directfn_ws_st_const(const double r1[], const double r2[], const double r3[],
                                     const double ko, const int Np_1D);
extern "C" void ref_directfn_st(const double* r1, const double* r2, const double* r3,
                                double ko, int Np, double* out) {
  complex<double> v = directfn_ws_st_const(r1, r2, r3, ko, Np);
  out[0] = v.real();
  out[1] = v.imag();
}
#endif

#if defined(SHIM_DIRECTFN_EA)
complex<double> directfn_ws_ea_const(const double r1[], const double r2[], const double r3[],
                                     const double r4[], const double rp[], const double rq[],
                                     const double ko, const int Np_1D);
extern "C" void ref_directfn_ea(const double* r1, const double* r2, const double* r3,
                                const double* r4, double ko, int Np, double* out) {
  complex<double> v = directfn_ws_ea_const(r1, r2, r3, r4, r2, r1, ko, Np);
  out[0] = v.real();
  out[1] = v.imag();
}
#endif

#if defined(SHIM_DIRECTFN_VA)
complex<double> directfn_ws_va_const(const double r1[], const double r2[], const double r3[],
                                     const double r4[], const double r5[], const double rq[],
                                     const double ko, const int Np_1D);
extern "C" void ref_directfn_va(const double* r1, const double* r2, const double* r3,
                                const double* r4, const double* r5, double ko, int Np,
                                double* out) {
  complex<double> v = directfn_ws_va_const(r1, r2, r3, r4, r5, r1, ko, Np);
  out[0] = v.real();
  out[1] = v.imag();
}
#endif
