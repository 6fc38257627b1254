// Shared helpers for the J-VIE kernels: complex arithmetic on float2/double2,
// status codes and CUDA error plumbing.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/marie_vie.h"

namespace marie {

template <typename T> struct cplx_of;
template <> struct cplx_of<float> { using type = float2; };
template <> struct cplx_of<double> { using type = double2; };
template <typename T> using cplx = typename cplx_of<T>::type;

template <typename V> __host__ __device__ __forceinline__ V mk(decltype(V::x) re, decltype(V::x) im) {
  V v; v.x = re; v.y = im; return v;
}
template <typename V> __host__ __device__ __forceinline__ V cadd(V a, V b) { return mk<V>(a.x + b.x, a.y + b.y); }
template <typename V> __host__ __device__ __forceinline__ V csub(V a, V b) { return mk<V>(a.x - b.x, a.y - b.y); }
template <typename V> __host__ __device__ __forceinline__ V cmul(V a, V b) {
  return mk<V>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename V> __host__ __device__ __forceinline__ V cmulc(V a, V b) {
  return mk<V>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename V> __host__ __device__ __forceinline__ V cconj(V a) { return mk<V>(a.x, -a.y); }
template <typename V> __host__ __device__ __forceinline__ V cscale(V a, decltype(V::x) s) { return mk<V>(a.x * s, a.y * s); }
// multiply by -i (forward) or +i (inverse)
template <bool INV, typename V> __host__ __device__ __forceinline__ V rot90(V a) {
  return INV ? mk<V>(-a.y, a.x) : mk<V>(a.y, -a.x);
}
template <typename VO, typename VI> __host__ __device__ __forceinline__ VO cvt(VI a) {
  VO o; o.x = (decltype(VO::x))a.x; o.y = (decltype(VO::x))a.y; return o;
}

// Sets the thread-local last-error text and returns the status code.
int set_error(int code, const char* fmt, ...);

// Counts kernel launches issued by this library (marie_launch_count).
void count_launch(long long n = 1);

// Test injection (marie_inject_tile_timeout): true once for each z-pass launch
// that should arm its tile barrier for more bytes than the copy delivers.
bool take_tile_timeout_injection();

// Counts GMRES calls whose restart cycles ran in one conditional-graph launch
// (marie_graph_loops).
void count_graph_loop();

// Streaming multiprocessors of the current device (queried once per device).
int sm_count();

// Blocks for a grid-stride loop over n elements: ceil(n / threads), at most
// per_sm blocks per streaming multiprocessor of the current device, at least 1.
inline int grid_stride_blocks(long long n, int per_sm, int threads = 256) {
  long long g = (n + threads - 1) / threads;
  const long long cap = (long long)sm_count() * per_sm;
  if (g > cap) g = cap;
  return g < 1 ? 1 : (int)g;
}

#define MARIE_CUDA_TRY(expr)                                                          \
  do {                                                                                \
    cudaError_t _e = (expr);                                                          \
    if (_e != cudaSuccess)                                                            \
      return ::marie::set_error(MARIE_ECUDA, "%s:%d %s: %s", __FILE__, __LINE__, #expr, \
                                cudaGetErrorString(_e));                              \
  } while (0)

#define MARIE_TRY(expr)          \
  do {                           \
    int _s = (expr);             \
    if (_s != MARIE_OK) return _s; \
  } while (0)

}  // namespace marie
