// Definitions of the matvec launchers; included only by the two translation
// units that instantiate them (matvec_f32.cu, matvec_f64.cu).
#pragma once
#include <cstring>

#include "matvec_fused.cuh"
#include "matvec_launch.cuh"

namespace marie {

template <typename T> struct MatvecImpl {
  using V = cplx<T>;

  template <int NL, typename IO>
  static cudaError_t xfwd_n(const IO* J, long long js, const int* inv, Prologue pro, V* A, long long as,
                            const Dims& d, const V* tw, int nrhs, cudaStream_t st) {
    constexpr int S = RowCfg<cplx<T>, NL>::S;
    const size_t smem = (size_t)(NL + NL * (S + 1)) * sizeof(V);
    cudaError_t e = opt_in_smem(k_xfwd<T, NL, IO>, smem);
    if (e != cudaSuccess) return e;
    const int rows = d.M * d.N * 3;
    dim3 grid((rows + S - 1) / S, nrhs);
    k_xfwd<T, NL, IO><<<grid, RowCfg<cplx<T>, NL>::THREADS, smem, st>>>(J, js, inv, pro, A, as, d, tw);
    return cudaGetLastError();
  }
  template <int NL, typename IO>
  static cudaError_t xinv_n(const V* A, long long as, const IO* J, long long js, const int* inv, Epilogue ep,
                            IO* out, long long os, const Dims& d, const V* tw, int nrhs, cudaStream_t st) {
    constexpr int S = RowCfg<cplx<T>, NL>::S;
    const size_t smem = (size_t)(NL + NL * (S + 1)) * sizeof(V);
    cudaError_t e = opt_in_smem(k_xinv<T, NL, IO>, smem);
    if (e != cudaSuccess) return e;
    const int rows = d.M * d.N * 3;
    dim3 grid((rows + S - 1) / S, nrhs);
    k_xinv<T, NL, IO><<<grid, RowCfg<cplx<T>, NL>::THREADS, smem, st>>>(A, as, J, js, inv, ep, out, os, d, tw);
    return cudaGetLastError();
  }
  template <int NC, bool INV>
  static cudaError_t cols_n(const V* in, long long in_w, long long in_rhs, int n_in, V* out, long long out_w,
                            long long out_rhs, int n_out, int Lp, int nw, const V* tw, int nrhs, cudaStream_t st,
                            const int* stop, int step) {
    constexpr int S = ColS<T>::S;
    const size_t smem = (size_t)(NC + NC * (S + 1)) * sizeof(V);
    cudaError_t e = opt_in_smem(k_cols<T, NC, INV>, smem);
    if (e != cudaSuccess) return e;
    dim3 grid((Lp + S - 1) / S, nw, nrhs);
    k_cols<T, NC, INV><<<grid, S * FFT<V, NC, INV>::T, smem, st>>>(in, in_w, in_rhs, n_in, out, out_w, out_rhs,
                                                                  n_out, Lp, tw, stop, step);
    return cudaGetLastError();
  }
  template <int NZ, int KIND, int VAR>
  static cudaError_t zmul_nk(V* B, long long bs, const V* fN, int oct, const Dims& d, const V* tw, int nrhs,
                             cudaStream_t st, const ZTile* zt) {
    using ZC = ZS<T, NZ, KIND, VAR>;
    constexpr int S = ZC::S;
    // the bulk-copy tile needs a tensor map whose box is S columns wide
    const int mi = S == 8 ? 0 : S == 4 ? 1 : S == 2 ? 2 : -1;
    int tma = (ZC::TMA && zt && zt->ok && oct && mi >= 0) ? 1 : 0;
    if (tma && take_tile_timeout_injection()) tma = 2;  // test: a wait that runs out
    CUtensorMap none;
    memset(&none, 0, sizeof(none));
    const CUtensorMap& tmap = tma ? zt->map[mi] : none;
    int* err = zt ? zt->err : nullptr;
    const size_t smem = (size_t)ZC::bytes(S);  // S columns, 3 component buffers, operator tile
    cudaError_t e = opt_in_smem(k_zmul<T, NZ, KIND, VAR>, smem);
    if (e != cudaSuccess) return e;
    // the pass waits (griddepcontrol) before reading the previous pass's output
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((d.Lp + S - 1) / S, d.Mp, nrhs);
    cfg.blockDim = dim3(ZC::THREADS, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_zmul<T, NZ, KIND, VAR>, B, bs, fN, oct, d, tw, tmap, tma, err);
  }
  template <int NZ>
  static cudaError_t zmul_n(V* B, long long bs, const V* fN, int oct, const Dims& d, const V* tw, int nrhs,
                            cudaStream_t st, int kind, int var, const ZTile* zt) {
    if (kind == 1) return zmul_nk<NZ, 1, 0>(B, bs, fN, oct, d, tw, nrhs, st, nullptr);
    if constexpr (sizeof(T) == 4) {
      if constexpr (HasWide<NZ>::value)
        if (var == 1) return zmul_nk<NZ, 0, 1>(B, bs, fN, oct, d, tw, nrhs, st, zt);
      if (var == 2) return zmul_nk<NZ, 0, 2>(B, bs, fN, oct, d, tw, nrhs, st, zt);
    }
    return zmul_nk<NZ, 0, 0>(B, bs, fN, oct, d, tw, nrhs, st, zt);
  }

  template <typename IO>
  static cudaError_t xfwd(const IO* J, long long js, const int* inv, Prologue pro, V* A, long long as,
                          const Dims& d, const V* tw, int nrhs, cudaStream_t st) {
    switch (d.Lp) {
#define MARIE_CASE(n_) case n_: return xfwd_n<n_, IO>(J, js, inv, pro, A, as, d, tw, nrhs, st);
      MARIE_FFT_LENGTHS(MARIE_CASE)
#undef MARIE_CASE
    }
    return cudaErrorInvalidValue;
  }
  template <typename IO>
  static cudaError_t xinv(const V* A, long long as, const IO* J, long long js, const int* inv, Epilogue ep,
                          IO* out, long long os, const Dims& d, const V* tw, int nrhs, cudaStream_t st) {
    switch (d.Lp) {
#define MARIE_CASE(n_) case n_: return xinv_n<n_, IO>(A, as, J, js, inv, ep, out, os, d, tw, nrhs, st);
      MARIE_FFT_LENGTHS(MARIE_CASE)
#undef MARIE_CASE
    }
    return cudaErrorInvalidValue;
  }
  static cudaError_t cols(bool inv, int NC, const V* in, long long in_w, long long in_rhs, int n_in, V* out,
                          long long out_w, long long out_rhs, int n_out, int Lp, int nw, const V* tw, int nrhs,
                          cudaStream_t st, const int* stop, int step) {
    if (inv) {
      switch (NC) {
#define MARIE_CASE(n_) \
  case n_: return cols_n<n_, true>(in, in_w, in_rhs, n_in, out, out_w, out_rhs, n_out, Lp, nw, tw, nrhs, st, stop, step);
        MARIE_FFT_LENGTHS(MARIE_CASE)
#undef MARIE_CASE
      }
    } else {
      switch (NC) {
#define MARIE_CASE(n_) \
  case n_: return cols_n<n_, false>(in, in_w, in_rhs, n_in, out, out_w, out_rhs, n_out, Lp, nw, tw, nrhs, st, stop, step);
        MARIE_FFT_LENGTHS(MARIE_CASE)
#undef MARIE_CASE
      }
    }
    return cudaErrorInvalidValue;
  }
  static cudaError_t zmul(V* B, long long bs, const V* fN, int oct, const Dims& d, const V* tw, int nrhs,
                          cudaStream_t st, int kind, int var, const ZTile* zt) {
    switch (d.Np) {
#define MARIE_CASE(n_) case n_: return zmul_n<n_>(B, bs, fN, oct, d, tw, nrhs, st, kind, var, zt);
      MARIE_FFT_LENGTHS(MARIE_CASE)
#undef MARIE_CASE
    }
    return cudaErrorInvalidValue;
  }
};


// (2L, 2M, cluster size) of the grids with fused x+y passes
#define MARIE_FUSED_PAIRS(X) X(64, 64, 2) X(96, 96, 2) X(128, 128, 4) X(192, 192, 4) X(256, 256, 8) X(512, 384, 8)

template <typename T> struct FusedImpl {
  using V = cplx<T>;
  template <int NL, int NM, int CS> static constexpr bool usable() {
    using C = XYCfg<T, NL, NM, CS>;
    // FP64 is FP64-pipe bound on GB300: the fused kernels' lower occupancy costs
    // more than the saved spectrum traffic, so FP64 keeps the five-pass path.
    return sizeof(T) == 4 && C::ok && C::fwd_smem <= 220 * 1024 && C::inv_smem <= 220 * 1024;
  }
  template <typename K>
  static cudaError_t launch(K kern, int CS, int nblocks, int nrhs, size_t smem, cudaStream_t st, void** args) {
    cudaError_t e = opt_in_smem(kern, smem);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nblocks, nrhs, 1);
    cfg.blockDim = dim3(256, 1, 1);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)CS;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    // the pass waits (griddepcontrol) before reading the previous pass's output
    attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[1].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 2;
    return cudaLaunchKernelExC(&cfg, (const void*)kern, args);
  }
  template <int NL, int NM, int CS, bool NARROW, typename IO>
  static cudaError_t xyfwd_nv(const IO* J, long long js, const int* inv, Prologue pro, V* B, long long bs,
                              Dims d, const V* twx, const V* twy, int nrhs, cudaStream_t st) {
    void* args[] = {(void*)&J, (void*)&js, (void*)&inv, (void*)&pro, (void*)&B, (void*)&bs, (void*)&d,
                    (void*)&twx, (void*)&twy};
    return launch(k_xyfwd<T, NL, NM, CS, NARROW, IO>, CS, CS * 3 * d.N, nrhs, XYCfg<T, NL, NM, CS, NARROW>::fwd_smem,
                  st, args);
  }
  template <int NL, int NM, int CS, bool NARROW, typename IO>
  static cudaError_t yxinv_nv(const V* B, long long bs, const IO* J, long long js, const int* inv, Epilogue ep,
                              IO* out, long long os, Dims d, const V* twx, const V* twy, int nrhs,
                              cudaStream_t st) {
    void* args[] = {(void*)&B, (void*)&bs, (void*)&J, (void*)&js, (void*)&inv, (void*)&ep, (void*)&out,
                    (void*)&os, (void*)&d, (void*)&twx, (void*)&twy};
    return launch(k_yxinv<T, NL, NM, CS, NARROW, IO>, CS, CS * 3 * d.N, nrhs, XYCfg<T, NL, NM, CS, NARROW>::inv_smem,
                  st, args);
  }
  // a narrow variant exists where either transform has a wide schedule
  template <int NL, int NM> static constexpr bool has_narrow() {
    return sizeof(T) == 4 && (HasWide<NL>::value || HasWide<NM>::value);
  }
  template <int NL, int NM, int CS, typename IO>
  static cudaError_t xyfwd_n(const IO* J, long long js, const int* inv, Prologue pro, V* B, long long bs,
                             Dims d, const V* twx, const V* twy, int nrhs, cudaStream_t st, int fvar) {
    if constexpr (usable<NL, NM, CS>()) {
      if constexpr (has_narrow<NL, NM>())
        if (fvar == 1) return xyfwd_nv<NL, NM, CS, true, IO>(J, js, inv, pro, B, bs, d, twx, twy, nrhs, st);
      if constexpr (CS >= 4 && usable<NL, NM, CS / 2>())
        if (fvar == 2) return xyfwd_nv<NL, NM, CS / 2, false, IO>(J, js, inv, pro, B, bs, d, twx, twy, nrhs, st);
      return xyfwd_nv<NL, NM, CS, false, IO>(J, js, inv, pro, B, bs, d, twx, twy, nrhs, st);
    } else {
      return cudaErrorNotSupported;
    }
  }
  template <int NL, int NM, int CS, typename IO>
  static cudaError_t yxinv_n(const V* B, long long bs, const IO* J, long long js, const int* inv, Epilogue ep,
                             IO* out, long long os, Dims d, const V* twx, const V* twy, int nrhs,
                             cudaStream_t st, int fvar) {
    if constexpr (usable<NL, NM, CS>()) {
      if constexpr (has_narrow<NL, NM>())
        if (fvar == 1) return yxinv_nv<NL, NM, CS, true, IO>(B, bs, J, js, inv, ep, out, os, d, twx, twy, nrhs, st);
      if constexpr (CS >= 4 && usable<NL, NM, CS / 2>())
        if (fvar == 2)
          return yxinv_nv<NL, NM, CS / 2, false, IO>(B, bs, J, js, inv, ep, out, os, d, twx, twy, nrhs, st);
      return yxinv_nv<NL, NM, CS, false, IO>(B, bs, J, js, inv, ep, out, os, d, twx, twy, nrhs, st);
    } else {
      return cudaErrorNotSupported;
    }
  }
};

template <typename T> bool MatvecLaunch<T>::fused(const Dims& d) {
#define MARIE_CASE(a_, b_, c_) \
  if (d.Lp == a_ && d.Mp == b_) return FusedImpl<T>::template usable<a_, b_, c_>();
  MARIE_FUSED_PAIRS(MARIE_CASE)
#undef MARIE_CASE
  return false;
}
template <typename T>
template <typename IO>
cudaError_t MatvecLaunch<T>::xyfwd(const IO* J, long long js, const int* inv, Prologue pro, V* B, long long bs,
                                   const Dims& d, const V* twx, const V* twy, int nrhs, cudaStream_t st, int fvar) {
#define MARIE_CASE(a_, b_, c_)    \
  if (d.Lp == a_ && d.Mp == b_) \
    return FusedImpl<T>::template xyfwd_n<a_, b_, c_, IO>(J, js, inv, pro, B, bs, d, twx, twy, nrhs, st, fvar);
  MARIE_FUSED_PAIRS(MARIE_CASE)
#undef MARIE_CASE
  return cudaErrorNotSupported;
}
template <typename T>
template <typename IO>
cudaError_t MatvecLaunch<T>::yxinv(const V* B, long long bs, const IO* J, long long js, const int* inv,
                                   Epilogue ep, IO* out, long long os, const Dims& d, const V* twx, const V* twy,
                                   int nrhs, cudaStream_t st, int fvar) {
#define MARIE_CASE(a_, b_, c_)    \
  if (d.Lp == a_ && d.Mp == b_) \
    return FusedImpl<T>::template yxinv_n<a_, b_, c_, IO>(B, bs, J, js, inv, ep, out, os, d, twx, twy, nrhs, st, \
                                                          fvar);
  MARIE_FUSED_PAIRS(MARIE_CASE)
#undef MARIE_CASE
  return cudaErrorNotSupported;
}

template <typename T>
template <typename IO>
cudaError_t MatvecLaunch<T>::xfwd(const IO* J, long long js, const int* inv, Prologue pro, V* A, long long as,
                                  const Dims& d, const V* tw, int nrhs, cudaStream_t st) {
  return MatvecImpl<T>::template xfwd<IO>(J, js, inv, pro, A, as, d, tw, nrhs, st);
}
template <typename T>
template <typename IO>
cudaError_t MatvecLaunch<T>::xinv(const V* A, long long as, const IO* J, long long js, const int* inv,
                                  Epilogue ep, IO* out, long long os, const Dims& d, const V* tw, int nrhs,
                                  cudaStream_t st) {
  return MatvecImpl<T>::template xinv<IO>(A, as, J, js, inv, ep, out, os, d, tw, nrhs, st);
}
template <typename T>
cudaError_t MatvecLaunch<T>::cols(bool inv, int NC, const V* in, long long in_w, long long in_rhs, int n_in, V* out,
                                  long long out_w, long long out_rhs, int n_out, int Lp, int nw, const V* tw,
                                  int nrhs, cudaStream_t st, const int* stop, int step) {
  return MatvecImpl<T>::cols(inv, NC, in, in_w, in_rhs, n_in, out, out_w, out_rhs, n_out, Lp, nw, tw, nrhs, st, stop,
                             step);
}
template <typename T>
cudaError_t MatvecLaunch<T>::zmul(V* B, long long bs, const V* fN, int oct, const Dims& d, const V* tw, int nrhs,
                                  cudaStream_t st, int kind, int var, const ZTile* zt) {
  return MatvecImpl<T>::zmul(B, bs, fN, oct, d, tw, nrhs, st, kind, var, zt);
}

}  // namespace marie
