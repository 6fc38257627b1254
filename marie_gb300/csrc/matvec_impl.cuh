// Definitions of the matvec launchers; included only by the two translation
// units that instantiate them (matvec_f32.cu, matvec_f64.cu).
#pragma once
#include "matvec_launch.cuh"

namespace marie {

template <typename T> struct MatvecImpl {
  using V = cplx<T>;

  template <int NL>
  static cudaError_t xfwd_n(const double2* J, long long js, const int* inv, Prologue pro, V* A, long long as,
                            const Dims& d, const V* tw, int nrhs, cudaStream_t st) {
    constexpr int S = RowCfg<NL>::S;
    const size_t smem = (size_t)(NL + NL * (S + 1)) * sizeof(V);
    cudaError_t e = opt_in_smem(k_xfwd<T, NL>, smem);
    if (e != cudaSuccess) return e;
    const int rows = d.M * d.N * 3;
    dim3 grid((rows + S - 1) / S, nrhs);
    k_xfwd<T, NL><<<grid, RowCfg<NL>::THREADS, smem, st>>>(J, js, inv, pro, A, as, d, tw);
    return cudaGetLastError();
  }
  template <int NL>
  static cudaError_t xinv_n(const V* A, long long as, const double2* J, long long js, const int* inv, Epilogue ep,
                            double2* out, long long os, const Dims& d, const V* tw, int nrhs, cudaStream_t st) {
    constexpr int S = RowCfg<NL>::S;
    const size_t smem = (size_t)(NL + NL * (S + 1)) * sizeof(V);
    cudaError_t e = opt_in_smem(k_xinv<T, NL>, smem);
    if (e != cudaSuccess) return e;
    const int rows = d.M * d.N * 3;
    dim3 grid((rows + S - 1) / S, nrhs);
    k_xinv<T, NL><<<grid, RowCfg<NL>::THREADS, smem, st>>>(A, as, J, js, inv, ep, out, os, d, tw);
    return cudaGetLastError();
  }
  template <int NC, bool INV>
  static cudaError_t cols_n(const V* in, long long in_w, long long in_rhs, int n_in, V* out, long long out_w,
                            long long out_rhs, int n_out, int Lp, int nw, const V* tw, int nrhs, cudaStream_t st) {
    constexpr int S = ColS<T>::S;
    const size_t smem = (size_t)(NC + NC * (S + 1)) * sizeof(V);
    cudaError_t e = opt_in_smem(k_cols<T, NC, INV>, smem);
    if (e != cudaSuccess) return e;
    dim3 grid((Lp + S - 1) / S, nw, nrhs);
    k_cols<T, NC, INV><<<grid, S * FFT<V, NC, INV>::T, smem, st>>>(in, in_w, in_rhs, n_in, out, out_w, out_rhs,
                                                                  n_out, Lp, tw);
    return cudaGetLastError();
  }
  template <int NZ>
  static cudaError_t zmul_n(V* B, long long bs, const V* fN, int oct, const Dims& d, const V* tw, int nrhs,
                            cudaStream_t st) {
    constexpr int S = ZS<T, NZ>::S;
    const size_t smem = (size_t)ZS<T, NZ>::bytes(S);
    cudaError_t e = opt_in_smem(k_zmul<T, NZ>, smem);
    if (e != cudaSuccess) return e;
    dim3 grid((d.Lp + S - 1) / S, d.Mp, nrhs);
    k_zmul<T, NZ><<<grid, ZS<T, NZ>::THREADS, smem, st>>>(B, bs, fN, oct, d, tw);
    return cudaGetLastError();
  }

  static cudaError_t xfwd(const double2* J, long long js, const int* inv, Prologue pro, V* A, long long as,
                          const Dims& d, const V* tw, int nrhs, cudaStream_t st) {
    switch (d.Lp) {
#define MARIE_CASE(n_) case n_: return xfwd_n<n_>(J, js, inv, pro, A, as, d, tw, nrhs, st);
      MARIE_FFT_LENGTHS(MARIE_CASE)
#undef MARIE_CASE
    }
    return cudaErrorInvalidValue;
  }
  static cudaError_t xinv(const V* A, long long as, const double2* J, long long js, const int* inv, Epilogue ep,
                          double2* out, long long os, const Dims& d, const V* tw, int nrhs, cudaStream_t st) {
    switch (d.Lp) {
#define MARIE_CASE(n_) case n_: return xinv_n<n_>(A, as, J, js, inv, ep, out, os, d, tw, nrhs, st);
      MARIE_FFT_LENGTHS(MARIE_CASE)
#undef MARIE_CASE
    }
    return cudaErrorInvalidValue;
  }
  static cudaError_t cols(bool inv, int NC, const V* in, long long in_w, long long in_rhs, int n_in, V* out,
                          long long out_w, long long out_rhs, int n_out, int Lp, int nw, const V* tw, int nrhs,
                          cudaStream_t st) {
    if (inv) {
      switch (NC) {
#define MARIE_CASE(n_) \
  case n_: return cols_n<n_, true>(in, in_w, in_rhs, n_in, out, out_w, out_rhs, n_out, Lp, nw, tw, nrhs, st);
        MARIE_FFT_LENGTHS(MARIE_CASE)
#undef MARIE_CASE
      }
    } else {
      switch (NC) {
#define MARIE_CASE(n_) \
  case n_: return cols_n<n_, false>(in, in_w, in_rhs, n_in, out, out_w, out_rhs, n_out, Lp, nw, tw, nrhs, st);
        MARIE_FFT_LENGTHS(MARIE_CASE)
#undef MARIE_CASE
      }
    }
    return cudaErrorInvalidValue;
  }
  static cudaError_t zmul(V* B, long long bs, const V* fN, int oct, const Dims& d, const V* tw, int nrhs,
                          cudaStream_t st) {
    switch (d.Np) {
#define MARIE_CASE(n_) case n_: return zmul_n<n_>(B, bs, fN, oct, d, tw, nrhs, st);
      MARIE_FFT_LENGTHS(MARIE_CASE)
#undef MARIE_CASE
    }
    return cudaErrorInvalidValue;
  }
};


template <typename T>
cudaError_t MatvecLaunch<T>::xfwd(const double2* J, long long js, const int* inv, Prologue pro, V* A, long long as,
                                  const Dims& d, const V* tw, int nrhs, cudaStream_t st) {
  return MatvecImpl<T>::xfwd(J, js, inv, pro, A, as, d, tw, nrhs, st);
}
template <typename T>
cudaError_t MatvecLaunch<T>::xinv(const V* A, long long as, const double2* J, long long js, const int* inv,
                                  Epilogue ep, double2* out, long long os, const Dims& d, const V* tw, int nrhs,
                                  cudaStream_t st) {
  return MatvecImpl<T>::xinv(A, as, J, js, inv, ep, out, os, d, tw, nrhs, st);
}
template <typename T>
cudaError_t MatvecLaunch<T>::cols(bool inv, int NC, const V* in, long long in_w, long long in_rhs, int n_in, V* out,
                                  long long out_w, long long out_rhs, int n_out, int Lp, int nw, const V* tw,
                                  int nrhs, cudaStream_t st) {
  return MatvecImpl<T>::cols(inv, NC, in, in_w, in_rhs, n_in, out, out_w, out_rhs, n_out, Lp, nw, tw, nrhs, st);
}
template <typename T>
cudaError_t MatvecLaunch<T>::zmul(V* B, long long bs, const V* fN, int oct, const Dims& d, const V* tw, int nrhs,
                                  cudaStream_t st) {
  return MatvecImpl<T>::zmul(B, bs, fN, oct, d, tw, nrhs, st);
}

}  // namespace marie
