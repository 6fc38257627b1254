// Host-side launchers for the matvec passes: runtime FFT length -> template
// instantiation, dynamic shared-memory opt-in, grid shapes.
#pragma once
#include "matvec_kernels.cuh"

namespace marie {

#define MARIE_FFT_LENGTHS(X) \
  X(8) X(16) X(24) X(32) X(40) X(48) X(64) X(80) X(96) X(128) X(160) X(192) X(256) X(320) X(384) X(512)

inline bool fft_length_supported(int n) {
#define MARIE_LEN_CASE(n_) if (n == n_) return true;
  MARIE_FFT_LENGTHS(MARIE_LEN_CASE)
#undef MARIE_LEN_CASE
  return false;
}

// Raises the kernel's dynamic shared-memory limit once per kernel and device
// (never again afterwards, so launches inside a stream capture stay pure).
bool smem_opted_in(const void* kernel, size_t bytes);
void smem_mark_opted_in(const void* kernel, size_t bytes);
template <typename K> inline cudaError_t opt_in_smem(K kernel, size_t bytes) {
  if (bytes <= 48 * 1024 || smem_opted_in((const void*)kernel, bytes)) return cudaSuccess;
  const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e == cudaSuccess) smem_mark_opted_in((const void*)kernel, bytes);
  return e;
}

// The z pass's operator tile by bulk tensor copy (FP32 N operator): tensor
// maps over the plan's copy of the operator stored full along x,
// fN32x[q][oz][oy][kx] (2L x (M+1) x (N+1) x 6), one per box width of 8, 4
// and 2 columns, and the device word a pass sets when a copy does not arrive.
struct ZTile {
  CUtensorMap map[3];
  int ok = 0;
  int* err = nullptr;
};

// IO: the type of the matvec's input and output vectors (double2, or float2
// for FP32 arithmetic T = float)
template <typename T> struct MatvecLaunch {
  using V = cplx<T>;
  template <typename IO>
  static cudaError_t xfwd(const IO* J, long long js, const int* inv, Prologue pro, V* A, long long as,
                          const Dims& d, const V* tw, int nrhs, cudaStream_t st);
  template <typename IO>
  static cudaError_t xinv(const V* A, long long as, const IO* J, long long js, const int* inv, Epilogue ep,
                          IO* out, long long os, const Dims& d, const V* tw, int nrhs, cudaStream_t st);
  static cudaError_t cols(bool inv, int NC, const V* in, long long in_w, long long in_rhs, int n_in, V* out,
                          long long out_w, long long out_rhs, int n_out, int Lp, int nw, const V* tw, int nrhs,
                          cudaStream_t st, const int* stop = nullptr, int step = 0);
  // kind 0: the symmetric N operator (6 components), 1: the K operator (3);
  // var: the z-pass variant chosen by the autotuner (FP32, N operator)
  // zt: the bulk-copy tile source of an FP32 N operator (null: per-thread copies)
  static cudaError_t zmul(V* B, long long bs, const V* fN, int oct, const Dims& d, const V* tw, int nrhs,
                          cudaStream_t st, int kind = 0, int var = 0, const ZTile* zt = nullptr);
  // fused x+y passes (thread-block clusters); fused() says whether this grid has them
  static bool fused(const Dims& d);
  // fvar: 0 the default x/y radix schedules, 1 the narrow (radix-8) ones
  template <typename IO>
  static cudaError_t xyfwd(const IO* J, long long js, const int* inv, Prologue pro, V* B, long long bs,
                           const Dims& d, const V* twx, const V* twy, int nrhs, cudaStream_t st, int fvar = 0);
  template <typename IO>
  static cudaError_t yxinv(const V* B, long long bs, const IO* J, long long js, const int* inv, Epilogue ep,
                           IO* out, long long os, const Dims& d, const V* twx, const V* twy, int nrhs,
                           cudaStream_t st, int fvar = 0);
};

}  // namespace marie
