// C-ABI entry points for plans, operator upload and the matvecs, plus the
// host-side plumbing they share (pointer staging, workspaces, index maps).
#include <cmath>
#include <cstdarg>
#include <atomic>
#include <map>
#include <mutex>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "matvec_launch.cuh"
#include "plan.h"

namespace marie {

static thread_local char g_err[512] = "";
static std::atomic<long long> g_launches{0};

void count_launch(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

static std::atomic<long long> g_tile_timeouts{0};
static std::atomic<long long> g_graph_loops{0};
void count_graph_loop() { g_graph_loops.fetch_add(1, std::memory_order_relaxed); }
bool take_tile_timeout_injection() {
  long long left = g_tile_timeouts.load();
  while (left > 0 && !g_tile_timeouts.compare_exchange_weak(left, left - 1)) {
  }
  return left > 0;
}

int sm_count() {
  static std::atomic<int> cache[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  int v = cache[dev].load(std::memory_order_relaxed);
  if (v > 0) return v;
  if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) return 152;
  cache[dev].store(v, std::memory_order_relaxed);
  return v;
}

static std::mutex g_smem_mu;
static std::map<std::pair<const void*, int>, size_t> g_smem_set;  // (kernel, device) -> bytes

bool smem_opted_in(const void* kernel, size_t bytes) {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> g(g_smem_mu);
  auto it = g_smem_set.find({kernel, dev});
  return it != g_smem_set.end() && it->second >= bytes;
}
void smem_mark_opted_in(const void* kernel, size_t bytes) {
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> g(g_smem_mu);
  size_t& v = g_smem_set[{kernel, dev}];
  if (bytes > v) v = bytes;
}

int set_error(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

// host-side fault injection: the n-th allocation from now fails (0 = off)
static std::atomic<long long> g_fail_alloc_in{0};

// Library-owned stream-ordered memory pool per device.  Its release threshold
// keeps freed blocks mapped, so the per-solve buffers (the Krylov basis is
// ~1 GB at 128^3) are reused from the pool instead of being unmapped at every
// synchronisation and mapped again by the next solve, as the default pool
// (threshold 0) does.  The pool is separate from the device's default pool,
// which other libraries in the process keep using unchanged.
static std::mutex g_pool_mu;
static std::map<int, cudaMemPool_t> g_pools;

static cudaMemPool_t device_pool() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lock(g_pool_mu);
  auto it = g_pools.find(dev);
  if (it != g_pools.end()) return it->second;
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = dev;
  cudaMemPool_t pool = nullptr;
  if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  unsigned long long keep = ~0ULL;
  cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  g_pools[dev] = pool;
  return pool;
}

int DBuf::alloc(size_t bytes, cudaStream_t st) {
  s = st;
  if (bytes == 0) bytes = 16;
  long long left = g_fail_alloc_in.load();
  while (left > 0 && !g_fail_alloc_in.compare_exchange_weak(left, left - 1)) {
  }
  if (left == 1) {
    p = nullptr;
    return set_error(MARIE_ENOMEM, "device allocation of %zu bytes failed (injected)", bytes);
  }
  cudaMemPool_t pool = device_pool();
  cudaError_t e = pool ? cudaMallocFromPoolAsync(&p, bytes, pool, st) : cudaMallocAsync(&p, bytes, st);
  if (e != cudaSuccess && pool) {
    // blocks cached in the pool may be the wrong sizes: hand them back to the
    // device once and retry before reporting the failure
    cudaGetLastError();
    cudaStreamSynchronize(st);
    cudaMemPoolTrimTo(pool, 0);
    e = cudaMallocFromPoolAsync(&p, bytes, pool, st);
  }
  if (e != cudaSuccess) {
    p = nullptr;
    cudaGetLastError();
    return set_error(MARIE_ENOMEM, "device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
  }
  return MARIE_OK;
}

bool is_device_ptr(const void* ptr) { return ptr && host_kind(ptr) == HostKind::Device; }

int stage_in(const void* user, size_t bytes, cudaStream_t st, DBuf& tmp, const void** dev) {
  if (is_device_ptr(user)) {
    *dev = user;
    return MARIE_OK;
  }
  MARIE_TRY(tmp.alloc(bytes, st));
  MARIE_TRY(copy_to_device(tmp.p, user, bytes, st));
  *dev = tmp.p;
  return MARIE_OK;
}

int stage_out(void* user, size_t bytes, cudaStream_t st, DBuf& tmp, void** dev) {
  if (is_device_ptr(user)) {
    *dev = user;
    return MARIE_OK;
  }
  MARIE_TRY(tmp.alloc(bytes, st));
  *dev = tmp.p;
  return MARIE_OK;
}

int finish_out(void* user, const void* dev, size_t bytes, cudaStream_t st) {
  if (user != dev) MARIE_TRY(copy_to_host(user, dev, bytes, st));
  return MARIE_OK;
}

int ensure_workspace(marie_plan* p, int prec, long long nrhs, bool with_A) {
  const size_t es = (prec == MARIE_FP32) ? sizeof(float2) : sizeof(double2);
  const size_t need_A = with_A ? (size_t)p->elems_A() * es * nrhs : 0;
  const size_t need_B = (size_t)p->elems_B() * es * nrhs;
  if (need_A > p->ws_bytes_A) {
    if (p->wsA) cudaFreeAsync(p->wsA, p->stream);
    p->wsA = nullptr;
    p->ws_bytes_A = 0;
    if (cudaMallocAsync(&p->wsA, need_A, p->stream) != cudaSuccess) {
      cudaGetLastError();
      p->wsA = nullptr;
      return set_error(MARIE_ENOMEM, "workspace A (%zu bytes) allocation failed", need_A);
    }
    p->ws_bytes_A = need_A;
  }
  if (need_B > p->ws_bytes_B) {
    if (p->wsB) cudaFreeAsync(p->wsB, p->stream);
    p->wsB = nullptr;
    p->ws_bytes_B = 0;
    if (cudaMallocAsync(&p->wsB, need_B, p->stream) != cudaSuccess) {
      cudaGetLastError();
      p->wsB = nullptr;
      return set_error(MARIE_ENOMEM, "workspace B (%zu bytes) allocation failed", need_B);
    }
    p->ws_bytes_B = need_B;
  }
  return MARIE_OK;
}

int ensure_pinned(marie_plan* p, size_t n) {
  if (p->pinned_len >= n) return MARIE_OK;
  if (p->pinned) cudaFreeHost(p->pinned);
  p->pinned = nullptr;
  p->pinned_len = 0;
  MARIE_CUDA_TRY(cudaMallocHost(&p->pinned, n * sizeof(double)));
  p->pinned_len = n;
  return MARIE_OK;
}

// ---------------------------------------------------------------------------
// index map and coefficient kernels
// ---------------------------------------------------------------------------
__global__ void k_fill_int(int* a, long long n, int v) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    a[i] = v;
}

__global__ void k_scatter_inverse(const int64_t* idx, long long n, long long n3V, int* inv, int* err) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long g = idx[i] - 1;
    if (g < 0 || g >= n3V) {
      atomicOr(err, 1);
      continue;
    }
    const int old = atomicExch(&inv[g], (int)i);
    if (old != -1) atomicOr(err, 2);
  }
}

__global__ void k_coefficients(const int64_t* idx, long long n, long long V, const double2* Mr, const double2* Mc,
                               double Gram, int mode, double2* a, double2* b) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const long long v = (idx[i] - 1) % V;
    const double2 mr = Mr[v], mc = Mc[v];
    if (mode == 0) {
      a[i] = mk<double2>(Gram * mr.x, Gram * mr.y);
      b[i] = mc;
    } else {
      b[i] = mc;                                      // prologue factor
      a[i] = mk<double2>(Gram * mr.x, -Gram * mr.y);  // Gram * conj(Mr)
    }
  }
}

static inline int grid_for(long long n, int threads = 256) { return grid_stride_blocks(n, 16, threads); }

// autotuner input: J = a smooth pattern, the identity DOF map over the grid
__global__ void k_tune_fill(double2* __restrict__ J, int* __restrict__ inv, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    J[i] = mk<double2>(1.0 + 1e-3 * (double)(i % 97), -1e-3 * (double)(i % 89));
    inv[i] = (int)i;
  }
}

int build_inverse_index(marie_plan* p, const int64_t* idx_dev, long long n, int* inv) {
  const long long n3V = 3 * p->d.V;
  if (n < 0 || n > n3V) return set_error(MARIE_EINVAL, "n_idx = %lld outside [0, 3*L*M*N = %lld]", n, n3V);
  DBuf err;
  MARIE_TRY(err.alloc(sizeof(int), p->stream));
  MARIE_CUDA_TRY(cudaMemsetAsync(err.p, 0, sizeof(int), p->stream));
  k_fill_int<<<grid_for(n3V), 256, 0, p->stream>>>(inv, n3V, -1);
  count_launch();
  if (n > 0) {
    k_scatter_inverse<<<grid_for(n), 256, 0, p->stream>>>(idx_dev, n, n3V, inv, err.as<int>());
    count_launch();
  }
  MARIE_CUDA_TRY(cudaGetLastError());
  int herr = 0;
  MARIE_CUDA_TRY(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, p->stream));
  MARIE_CUDA_TRY(cudaStreamSynchronize(p->stream));
  if (herr & 1) return set_error(MARIE_EINVAL, "idx entry outside [1, 3*L*M*N]");
  if (herr & 2) return set_error(MARIE_EINVAL, "idx has repeated entries");
  return MARIE_OK;
}

int build_coefficients(marie_plan* p, const int64_t* idx_dev, long long n, const double2* Mr, const double2* Mc,
                       double Gram, int mode, double2* a, double2* b) {
  if (n == 0) return MARIE_OK;
  k_coefficients<<<grid_for(n), 256, 0, p->stream>>>(idx_dev, n, p->d.V, Mr, Mc, Gram, mode, a, b);
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  return MARIE_OK;
}

template <typename T, typename IO>
static int run_matvec_t(marie_plan* p, const IO* J, long long js, IO* out, long long os, long long n,
                        int nrhs, const int* inv, const Prologue& pro, const Epilogue& ep, const cplx<T>* fN,
                        cplx<T>* const* tw, const int* stop, int step, int kind) {
  const int oct = kind == 0 ? p->oct : p->octK;
  using ML = MatvecLaunch<T>;
  const int prec = sizeof(T) == 4 ? MARIE_FP32 : MARIE_FP64;
  const long long chunk_max = p->nrhs_max > 0 ? p->nrhs_max : 1;
  const bool fused = p->fuse && ML::fused(p->d);
  for (long long r0 = 0; r0 < nrhs; r0 += chunk_max) {
    const int nr = (int)((nrhs - r0) < chunk_max ? (nrhs - r0) : chunk_max);
    MARIE_TRY(ensure_workspace(p, prec, nr, !fused));
    Dims d = p->d;
    d.stop = stop ? stop + r0 : nullptr;
    d.step = step;
    cplx<T>* A = reinterpret_cast<cplx<T>*>(p->wsA);
    cplx<T>* B = reinterpret_cast<cplx<T>*>(p->wsB);
    const long long sA = p->elems_A(), sB = p->elems_B();
    const IO* Jc = J + r0 * js;
    IO* oc = out + r0 * os;
    const bool prof = p->profile;
    if (prof) MARIE_CUDA_TRY(cudaEventRecord(p->ev[0], p->stream));
    if (fused) {
      MARIE_CUDA_TRY(ML::xyfwd(Jc, js, inv, pro, B, sB, d, tw[0], tw[1], nr, p->stream, p->fvar));
      if (prof) {
        MARIE_CUDA_TRY(cudaEventRecord(p->ev[1], p->stream));
        MARIE_CUDA_TRY(cudaEventRecord(p->ev[2], p->stream));
      }
      MARIE_CUDA_TRY(ML::zmul(B, sB, fN, oct, d, tw[2], nr, p->stream, kind, kind == 0 ? p->zvar : 0,
                                    kind == 0 ? &p->zt : nullptr));
      if (prof) {
        MARIE_CUDA_TRY(cudaEventRecord(p->ev[3], p->stream));
        MARIE_CUDA_TRY(cudaEventRecord(p->ev[4], p->stream));
      }
      MARIE_CUDA_TRY(ML::yxinv(B, sB, Jc, js, inv, ep, oc, os, d, tw[0], tw[1], nr, p->stream, p->fvar));
      count_launch(3);
    } else {
      MARIE_CUDA_TRY(ML::xfwd(Jc, js, inv, pro, A, sA, d, tw[0], nr, p->stream));
      if (prof) MARIE_CUDA_TRY(cudaEventRecord(p->ev[1], p->stream));
      MARIE_CUDA_TRY(ML::cols(false, d.Mp, A, (long long)d.Lp * d.M, sA, d.M, B, (long long)d.Lp * d.Mp, sB, d.Mp,
                              d.Lp, 3 * d.N, tw[1], nr, p->stream, d.stop, step));
      if (prof) MARIE_CUDA_TRY(cudaEventRecord(p->ev[2], p->stream));
      MARIE_CUDA_TRY(ML::zmul(B, sB, fN, oct, d, tw[2], nr, p->stream, kind, kind == 0 ? p->zvar : 0,
                                    kind == 0 ? &p->zt : nullptr));
      if (prof) MARIE_CUDA_TRY(cudaEventRecord(p->ev[3], p->stream));
      MARIE_CUDA_TRY(ML::cols(true, d.Mp, B, (long long)d.Lp * d.Mp, sB, d.Mp, A, (long long)d.Lp * d.M, sA, d.M,
                              d.Lp, 3 * d.N, tw[1], nr, p->stream, d.stop, step));
      if (prof) MARIE_CUDA_TRY(cudaEventRecord(p->ev[4], p->stream));
      MARIE_CUDA_TRY(ML::xinv(A, sA, Jc, js, inv, ep, oc, os, d, tw[0], nr, p->stream));
      count_launch(5);
    }
    if (prof) {
      MARIE_CUDA_TRY(cudaEventRecord(p->ev[5], p->stream));
      MARIE_CUDA_TRY(cudaEventSynchronize(p->ev[5]));
      for (int k = 0; k < 5; ++k) {
        float ms = 0;
        MARIE_CUDA_TRY(cudaEventElapsedTime(&ms, p->ev[k], p->ev[k + 1]));
        p->pass_ms[k] += ms;
      }
      p->profiled += 1;
    }
  }
  return MARIE_OK;
}

int run_matvec(marie_plan* p, int prec, const double2* J, long long js, double2* out, long long os, long long n,
               int nrhs, const int* inv, const Prologue& pro, const Epilogue& ep, const int* stop, int step,
               int kind) {
  if (kind == 0 && !p->has_op)
    return set_error(MARIE_ENOOP, "plan has no operator: call marie_set_operator or marie_plan_assemble");
  if (kind == 1 && !p->has_opK)
    return set_error(MARIE_ENOOP, "plan has no K operator: call marie_set_operator_k or marie_plan_assemble_k");
  const float2* f32 = kind == 0 ? p->fN32 : p->fK32;
  const double2* f64 = kind == 0 ? p->fN64 : p->fK64;
  if (prec == MARIE_FP32) {
    if (!f32) return set_error(MARIE_EINVAL, "plan was not created with FP32 arithmetic");
    return run_matvec_t<float, double2>(p, J, js, out, os, n, nrhs, inv, pro, ep, f32, p->tw32, stop, step, kind);
  }
  if (!f64) return set_error(MARIE_EINVAL, "plan was not created with FP64 arithmetic");
  return run_matvec_t<double, double2>(p, J, js, out, os, n, nrhs, inv, pro, ep, f64, p->tw64, stop, step, kind);
}

int run_matvec32(marie_plan* p, const float2* J, long long js, float2* out, long long os, long long n, int nrhs,
                 const int* inv, const Prologue& pro, const Epilogue& ep, const int* stop, int step, int kind) {
  if (kind == 0 && !p->has_op)
    return set_error(MARIE_ENOOP, "plan has no operator: call marie_set_operator or marie_plan_assemble");
  if (kind == 1 && !p->has_opK)
    return set_error(MARIE_ENOOP, "plan has no K operator: call marie_set_operator_k or marie_plan_assemble_k");
  const float2* f32 = kind == 0 ? p->fN32 : p->fK32;
  if (!f32) return set_error(MARIE_EINVAL, "plan was not created with FP32 arithmetic");
  if ((ep.a && !ep.af) || (ep.b && !ep.bf))
    return set_error(MARIE_EINVAL, "FP32 matvec needs the FP32 copies of per-DOF coefficients");
  return run_matvec_t<float, float2>(p, J, js, out, os, n, nrhs, inv, pro, ep, f32, p->tw32, stop, step, kind);
}

int run_matvec(marie_plan* p, int prec, const double2* J, double2* out, long long n, int nrhs, const int* inv,
               const Prologue& pro, const Epilogue& ep) {
  return run_matvec(p, prec, J, n, out, n, n, nrhs, inv, pro, ep, nullptr, 0);
}

// twiddles exp(-2*pi*i*k/n), built in double on the host
template <typename V> static int make_twiddles(int n, V** out, cudaStream_t st) {
  std::vector<V> h(n);
  for (int k = 0; k < n; ++k) {
    const double a = 2.0 * M_PI * (double)k / (double)n;
    h[k].x = (decltype(V::x))std::cos(a);
    h[k].y = (decltype(V::x))(-std::sin(a));
  }
  MARIE_CUDA_TRY(cudaMalloc(out, n * sizeof(V)));
  MARIE_CUDA_TRY(cudaMemcpy(*out, h.data(), n * sizeof(V), cudaMemcpyHostToDevice));
  return MARIE_OK;
}

__global__ void k_scale_convert(const double2* in, long long n, double s, double2* o64, float2* o32) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double2 v = in[i];
    if (o64) o64[i] = mk<double2>(v.x * s, v.y * s);
    if (o32) o32[i] = mk<float2>((float)(v.x * s), (float)(v.y * s));
  }
}

// parity of component q along axis a (0 x, 1 y, 2 z): true = odd
// component q of operator kind (0: N, 6 components; 1: K, 3) odd along axis a
__host__ __device__ inline bool comp_odd(int kind, int q, int a) {
  return kind == 0 ? OpKind<0>::odd(q, a) : OpKind<1>::odd(q, a);
}
__host__ __device__ inline int comp_count(int kind) { return kind == 0 ? 6 : 3; }

// max |fN(k) - s fN(mirror k)| and max |fN(k)| over the full operator (as the
// bit patterns of non-negative doubles, which order like the values).
__global__ void k_symmetry_check(const double2* __restrict__ f, int L, int M, int N, int kind,
                                 unsigned long long* __restrict__ out) {
  const int NQ = comp_count(kind);
  const long long Lp = 2LL * L, Mp = 2LL * M, Np = 2LL * N, P = Lp * Mp * Np;
  double dev = 0, mx = 0;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < NQ * P; t += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(t / P);
    long long r = t - q * P;
    const long long ix = r % Lp;
    r /= Lp;
    const long long iy = r % Mp, iz = r / Mp;
    const long long jx = ix > L ? Lp - ix : ix, jy = iy > M ? Mp - iy : iy, jz = iz > N ? Np - iz : iz;
    const bool neg = ((ix > L) && comp_odd(kind, q, 0)) ^ ((iy > M) && comp_odd(kind, q, 1)) ^
                     ((iz > N) && comp_odd(kind, q, 2));
    const double2 a = f[t];
    double2 b = f[q * P + jx + Lp * (jy + Mp * jz)];
    if (neg) b = mk<double2>(-b.x, -b.y);
    dev = fmax(dev, hypot(a.x - b.x, a.y - b.y));
    mx = fmax(mx, hypot(a.x, a.y));
  }
  for (int o = 16; o > 0; o >>= 1) {
    dev = fmax(dev, __shfl_xor_sync(0xffffffffu, dev, o));
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&out[0], (unsigned long long)__double_as_longlong(dev));
    atomicMax(&out[1], (unsigned long long)__double_as_longlong(mx));
  }
}

// octant (L+1) x (M+1) x (N+1) x NQ of the full operator, scaled, in FP64 and/or FP32
__global__ void k_extract_octant(const double2* __restrict__ f, int L, int M, int N, int NQ, double s, double2* o64,
                                 float2* o32) {
  const long long Lp = 2LL * L, Mp = 2LL * M, Np = 2LL * N, P = Lp * Mp * Np;
  const long long Lo = L + 1, Mo = M + 1, No = N + 1, O = Lo * Mo * No;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < NQ * O; t += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(t / O);
    long long r = t - q * O;
    const long long ox = r % Lo;
    r /= Lo;
    const long long oy = r % Mo, oz = r / Mo;
    const double2 v = f[q * P + ox + Lp * (oy + Mp * oz)];
    if (o64) o64[t] = mk<double2>(v.x * s, v.y * s);
    if (o32) o32[t] = mk<float2>((float)(v.x * s), (float)(v.y * s));
  }
}

// the N operator full along x, half along y and z: fx[q][oz][oy][kx] =
// s * f[q][oz][oy][kx] for oy <= M, oz <= N, in FP32 (the z pass's bulk tile
// source; the full operator already carries the x-reflection signs)
__global__ void k_extract_fullx(const double2* __restrict__ f, int L, int M, int N, double s, float2* __restrict__ fx) {
  const long long Lp = 2LL * L, Mp = 2LL * M, Np = 2LL * N, P = Lp * Mp * Np;
  const long long Mo = M + 1, No = N + 1, X = Lp * Mo * No;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < 6 * X; t += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(t / X);
    long long r = t - q * X;
    const long long kx = r % Lp;
    r /= Lp;
    const long long oy = r % Mo, oz = r / Mo;
    const double2 v = f[q * P + kx + Lp * (oy + Mp * oz)];
    fx[t] = mk<float2>((float)(v.x * s), (float)(v.y * s));
  }
}

// full operator from the octant (inverse of k_extract_octant), scaled by s
__global__ void k_expand_octant(const double2* __restrict__ o, int L, int M, int N, int kind, double s,
                                double2* __restrict__ f) {
  const long long Lp = 2LL * L, Mp = 2LL * M, Np = 2LL * N, P = Lp * Mp * Np;
  const long long Lo = L + 1, Mo = M + 1, No = N + 1, O = Lo * Mo * No;
  const int NQ = comp_count(kind);
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < NQ * P; t += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(t / P);
    long long r = t - q * P;
    const long long ix = r % Lp;
    r /= Lp;
    const long long iy = r % Mp, iz = r / Mp;
    const long long jx = ix > L ? Lp - ix : ix, jy = iy > M ? Mp - iy : iy, jz = iz > N ? Np - iz : iz;
    const bool neg = ((ix > L) && comp_odd(kind, q, 0)) ^ ((iy > M) && comp_odd(kind, q, 1)) ^
                     ((iz > N) && comp_odd(kind, q, 2));
    double2 v = o[q * O + jx + Lo * (jy + Mo * jz)];
    const double sg = neg ? -s : s;
    f[t] = mk<double2>(v.x * sg, v.y * sg);
  }
}

// Installs an operator (full layout, device) into the plan: the octant when it
// has the circulant's parity symmetry to 1e-12 of its maximum (every operator
// built by getOPERATORS does), the full array otherwise.  Scaled by 1/(8LMN).
// kind 0: N (6 components, fN64/fN32), 1: K (3 components, fK64/fK32).
// cuTensorMapEncodeTiled from the driver (looked up once through the runtime;
// the library links no driver library)
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiledFn encode_tiled() {
  static std::once_flag once;
  static EncodeTiledFn fn = nullptr;
  std::call_once(once, [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(f);
    cudaGetLastError();
  });
  return fn;
}

// The z pass's bulk tile source of an FP32 octant N operator: fN32x and one
// tensor map per box width (8, 4, 2 columns) over (2L, M+1, N+1, 6) 8-byte
// elements.  Without the driver entry point, or with N + 1 > 256 (beyond the
// box limit), the plan keeps the per-thread tile copies.
static int build_zt(marie_plan* p, const double2* fN_dev) {
  const Dims& d = p->d;
  cudaFree(p->fN32x);
  p->fN32x = nullptr;
  p->zt.ok = 0;
  p->zt.err = p->kerr;
  EncodeTiledFn enc = encode_tiled();
  if (!enc || d.N + 1 > 256) return MARIE_OK;
  const long long X = (long long)d.Lp * (d.M + 1) * (d.N + 1);
  MARIE_CUDA_TRY(cudaMalloc(&p->fN32x, 6 * X * sizeof(float2)));
  const long long P = (long long)d.Lp * d.Mp * d.Np;
  k_extract_fullx<<<grid_for(6 * X), 256, 0, p->stream>>>(fN_dev, d.L, d.M, d.N, 1.0 / (double)P, p->fN32x);
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  const cuuint64_t gd[4] = {(cuuint64_t)d.Lp, (cuuint64_t)d.M + 1, (cuuint64_t)d.N + 1, 6};
  const cuuint64_t gs[3] = {(cuuint64_t)d.Lp * 8, (cuuint64_t)d.Lp * (d.M + 1) * 8,
                            (cuuint64_t)d.Lp * (d.M + 1) * (d.N + 1) * 8};
  const cuuint32_t es[4] = {1, 1, 1, 1};
  const int widths[3] = {8, 4, 2};
  for (int i = 0; i < 3; ++i) {
    const cuuint32_t bd[4] = {(cuuint32_t)widths[i], 1, (cuuint32_t)d.N + 1, 6};
    const CUresult r = enc(&p->zt.map[i], CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 4, p->fN32x, gd, gs, bd, es,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
      cudaFree(p->fN32x);
      p->fN32x = nullptr;
      return MARIE_OK;
    }
  }
  p->zt.ok = 1;
  return MARIE_OK;
}

int check_kernel_status(marie_plan* p) {
  if (!p || !p->kerr) return MARIE_OK;
  int h = 0;
  MARIE_CUDA_TRY(cudaMemcpyAsync(&h, p->kerr, sizeof(int), cudaMemcpyDeviceToHost, p->stream));
  MARIE_CUDA_TRY(cudaStreamSynchronize(p->stream));
  if (h) {
    MARIE_CUDA_TRY(cudaMemsetAsync(p->kerr, 0, sizeof(int), p->stream));
    MARIE_CUDA_TRY(cudaStreamSynchronize(p->stream));
    return set_error(MARIE_ETIMEOUT, "a z-pass operator tile copy did not arrive within its time limit");
  }
  return MARIE_OK;
}

int install_operator(marie_plan* p, const double2* fN_dev, int kind) {
  const Dims& d = p->d;
  const long long P = (long long)d.Lp * d.Mp * d.Np;
  const long long O = (long long)(d.L + 1) * (d.M + 1) * (d.N + 1);
  const int NQ = comp_count(kind);
  const bool need64 = p->precision != MARIE_FP32;
  const bool need32 = p->precision != MARIE_FP64;
  DBuf flags;
  MARIE_TRY(flags.alloc(2 * sizeof(unsigned long long), p->stream));
  MARIE_CUDA_TRY(cudaMemsetAsync(flags.p, 0, 2 * sizeof(unsigned long long), p->stream));
  k_symmetry_check<<<grid_for(NQ * P), 256, 0, p->stream>>>(fN_dev, d.L, d.M, d.N, kind,
                                                            flags.as<unsigned long long>());
  count_launch();
  unsigned long long h[2];
  MARIE_CUDA_TRY(cudaMemcpyAsync(h, flags.p, sizeof(h), cudaMemcpyDeviceToHost, p->stream));
  MARIE_CUDA_TRY(cudaStreamSynchronize(p->stream));
  double dev, mx;
  memcpy(&dev, &h[0], sizeof(double));
  memcpy(&mx, &h[1], sizeof(double));
  const int oct = (dev <= 1e-12 * mx) ? 1 : 0;
  const long long n = oct ? NQ * O : NQ * P;
  if (kind == 0) {
    release_cufft_state(p);  // its full copy of fN is stale now
    cudaFree(p->fN32x);
    p->fN32x = nullptr;
    p->zt.ok = 0;
  }
  double2*& f64 = kind == 0 ? p->fN64 : p->fK64;
  float2*& f32 = kind == 0 ? p->fN32 : p->fK32;
  cudaFree(f64);
  cudaFree(f32);
  f64 = nullptr;
  f32 = nullptr;
  if (kind == 0)
    p->has_op = false;
  else
    p->has_opK = false;
  if (need64) MARIE_CUDA_TRY(cudaMalloc(&f64, n * sizeof(double2)));
  if (need32) MARIE_CUDA_TRY(cudaMalloc(&f32, n * sizeof(float2)));
  if (oct) {
    k_extract_octant<<<grid_for(n), 256, 0, p->stream>>>(fN_dev, d.L, d.M, d.N, NQ, 1.0 / (double)P,
                                                         need64 ? f64 : nullptr, need32 ? f32 : nullptr);
  } else {
    k_scale_convert<<<grid_for(n), 256, 0, p->stream>>>(fN_dev, n, 1.0 / (double)P, need64 ? f64 : nullptr,
                                                         need32 ? f32 : nullptr);
  }
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  if (kind == 0 && oct && need32) MARIE_TRY(build_zt(p, fN_dev));
  MARIE_CUDA_TRY(cudaStreamSynchronize(p->stream));
  if (kind == 0) {
    p->oct = oct;
    p->has_op = true;
  } else {
    p->octK = oct;
    p->has_opK = true;
  }
  return MARIE_OK;
}

}  // namespace marie

using namespace marie;

static void free_bound(marie_plan* p) {
  cudaFree(p->bnd_idx);
  cudaFree(p->bnd_inv);
  cudaFree(p->bnd_a);
  cudaFree(p->bnd_b);
  cudaFree(p->bnd_af);
  cudaFree(p->bnd_bf);
  p->bnd_idx = nullptr;
  p->bnd_inv = nullptr;
  p->bnd_a = p->bnd_b = nullptr;
  p->bnd_af = p->bnd_bf = nullptr;
  p->bnd_n = 0;
}

// out[k] = (float2) in[k]
__global__ void k_to_f32(const double2* __restrict__ in, long long n, float2* __restrict__ out) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    out[k] = make_float2((float)in[k].x, (float)in[k].y);
}

namespace marie {

int bound_operator(marie_plan* p, long long n, DevOp* op) {
  if (!p->bnd_n) return set_error(MARIE_EINVAL, "NULL operator and no mv_AN bound to the plan (marie_plan_bind_mv_AN)");
  if (p->bnd_n != n) return set_error(MARIE_EINVAL, "vector length %lld differs from the bound mv_AN's %lld DOFs", n,
                                      p->bnd_n);
  const int prec = p->fN64 ? MARIE_FP64 : MARIE_FP32;
  *op = [p, n, prec](const double2* x, double2* y) -> int {
    Prologue pro{nullptr, 0};
    Epilogue ep{};
    if (p->bnd_transp == 0) {
      ep.a = p->bnd_a;
      ep.b = p->bnd_b;
    } else {
      pro.pre = p->bnd_b;
      pro.conjin = 1;
      ep.a = p->bnd_a;
      ep.conjout = 1;
    }
    return run_matvec(p, prec, x, y, n, 1, p->bnd_inv, pro, ep);
  };
  return MARIE_OK;
}
}  // namespace marie

extern "C" {

const char* marie_last_error(void) { return g_err; }
int marie_version(void) { return 1; }

int marie_plan_create(int64_t L, int64_t M, int64_t N, int precision, int64_t nrhs_max, void* stream,
                      marie_plan** out) {
  if (!out) return set_error(MARIE_EINVAL, "plan output pointer is NULL");
  *out = nullptr;
  if (L < 1 || M < 1 || N < 1) return set_error(MARIE_EINVAL, "grid dimensions must be positive");
  if (!fft_length_supported((int)(2 * L)) || !fft_length_supported((int)(2 * M)) ||
      !fft_length_supported((int)(2 * N)))
    return set_error(MARIE_EUNSUPPORTED,
                     "padded FFT lengths %lld x %lld x %lld: each must be one of 8 16 24 32 40 48 64 80 96 128 160 "
                     "192 256 320 384 512",
                     (long long)(2 * L), (long long)(2 * M), (long long)(2 * N));
  if (precision != MARIE_FP64 && precision != MARIE_FP32 && precision != MARIE_MIXED)
    return set_error(MARIE_EINVAL, "precision must be MARIE_FP64, MARIE_FP32 or MARIE_MIXED");
  marie_plan* p = new marie_plan();
  p->d.L = (int)L; p->d.M = (int)M; p->d.N = (int)N;
  p->d.Lp = (int)(2 * L); p->d.Mp = (int)(2 * M); p->d.Np = (int)(2 * N);
  p->d.V = L * M * N;
  p->precision = precision;
  p->nrhs_max = nrhs_max > 0 ? nrhs_max : 1;
  {
    const char* nf = getenv("MARIE_NO_FUSED");  // forces the five-pass matvec (comparison runs)
    p->fuse = !(nf && nf[0] == '1');
  }
  cudaGetDevice(&p->device);
  if (stream) {
    p->stream = (cudaStream_t)stream;
  } else {
    if (cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete p;
      return set_error(MARIE_ECUDA, "stream creation failed");
    }
    p->own_stream = true;
  }
  if (cudaMalloc(&p->kerr, sizeof(int)) != cudaSuccess || cudaMemset(p->kerr, 0, sizeof(int)) != cudaSuccess) {
    cudaGetLastError();
    marie_plan_destroy(p);
    return set_error(MARIE_ENOMEM, "plan status word allocation failed");
  }
  const int lens[3] = {p->d.Lp, p->d.Mp, p->d.Np};
  for (int a = 0; a < 3; ++a) {
    int s = MARIE_OK;
    if (precision != MARIE_FP32 && s == MARIE_OK) s = make_twiddles(lens[a], &p->tw64[a], p->stream);
    if (precision != MARIE_FP64 && s == MARIE_OK) s = make_twiddles(lens[a], &p->tw32[a], p->stream);
    if (s != MARIE_OK) {
      marie_plan_destroy(p);
      return s;
    }
  }
  *out = p;
  return MARIE_OK;
}

int marie_plan_bind_mv_AN(marie_plan* p, const double* Mr, const double* Mc, double Gram, int transp,
                          const int64_t* idx, int64_t n_idx) {
  if (!p || !Mr || !Mc || !idx || n_idx < 1) return set_error(MARIE_EINVAL, "NULL argument or n_idx < 1");
  if (transp != 0 && transp != 1) return set_error(MARIE_EINVAL, "transp must be 0 ('notransp') or 1 ('transp')");
  if (!p->has_op) return set_error(MARIE_ENOOP, "plan has no operator");
  MARIE_CUDA_TRY(cudaStreamSynchronize(p->stream));
  free_bound(p);
  const long long V = p->d.V, n = n_idx;
  DBuf tMr, tMc;
  const void *Mr_d, *Mc_d, *idx_d;
  DBuf tidx;
  MARIE_TRY(stage_in(Mr, V * sizeof(double2), p->stream, tMr, &Mr_d));
  MARIE_TRY(stage_in(Mc, V * sizeof(double2), p->stream, tMc, &Mc_d));
  MARIE_TRY(stage_in(idx, n * sizeof(int64_t), p->stream, tidx, &idx_d));
  if (cudaMalloc(&p->bnd_idx, n * sizeof(int64_t)) != cudaSuccess ||
      cudaMalloc(&p->bnd_inv, 3 * V * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&p->bnd_a, n * sizeof(double2)) != cudaSuccess ||
      cudaMalloc(&p->bnd_b, n * sizeof(double2)) != cudaSuccess) {
    cudaGetLastError();
    free_bound(p);
    return set_error(MARIE_ENOMEM, "bound mv_AN: device allocation failed");
  }
  MARIE_CUDA_TRY(cudaMemcpyAsync(p->bnd_idx, idx_d, n * sizeof(int64_t), cudaMemcpyDeviceToDevice, p->stream));
  int s = build_inverse_index(p, p->bnd_idx, n, p->bnd_inv);
  if (s == MARIE_OK)
    s = build_coefficients(p, p->bnd_idx, n, (const double2*)Mr_d, (const double2*)Mc_d, Gram, transp, p->bnd_a,
                           p->bnd_b);
  if (s == MARIE_OK && p->fN32) {
    // FP32 copies for the FP32 applications, whose epilogue runs in FP32
    if (cudaMalloc(&p->bnd_af, n * sizeof(float2)) != cudaSuccess ||
        cudaMalloc(&p->bnd_bf, n * sizeof(float2)) != cudaSuccess) {
      cudaGetLastError();
      s = set_error(MARIE_ENOMEM, "bound mv_AN: device allocation failed");
    } else {
      k_to_f32<<<grid_stride_blocks(n, 8), 256, 0, p->stream>>>(p->bnd_a, n, p->bnd_af);
      k_to_f32<<<grid_stride_blocks(n, 8), 256, 0, p->stream>>>(p->bnd_b, n, p->bnd_bf);
      count_launch(2);
    }
  }
  if (s == MARIE_OK && cudaStreamSynchronize(p->stream) != cudaSuccess) s = set_error(MARIE_ECUDA, "bind mv_AN failed");
  if (s != MARIE_OK) {
    free_bound(p);
    return s;
  }
  p->bnd_n = n;
  p->bnd_transp = transp;
  return MARIE_OK;
}

int marie_plan_destroy(marie_plan* p) {
  if (!p) return MARIE_OK;
  if (p->stream) cudaStreamSynchronize(p->stream);
  release_cufft_state(p);
  free_bound(p);
  if (p->wsA) cudaFreeAsync(p->wsA, p->stream);
  if (p->wsB) cudaFreeAsync(p->wsB, p->stream);
  if (p->stream) cudaStreamSynchronize(p->stream);
  cudaFree(p->fN64);
  cudaFree(p->fN32);
  cudaFree(p->fN32x);
  cudaFree(p->kerr);
  cudaFree(p->fK64);
  cudaFree(p->fK32);
  for (int a = 0; a < 3; ++a) {
    cudaFree(p->tw64[a]);
    cudaFree(p->tw32[a]);
  }
  if (p->pinned) cudaFreeHost(p->pinned);
  for (int k = 0; k < 6; ++k)
    if (p->ev[k]) cudaEventDestroy(p->ev[k]);
  if (p->own_stream) cudaStreamDestroy(p->stream);
  delete p;
  return MARIE_OK;
}

void* marie_plan_stream(marie_plan* p) { return p ? (void*)p->stream : nullptr; }

// Autotuner: times the FP32 matvec of this plan's grid for every candidate
// schedule (fused x+y passes with the default or the narrow radix schedule, or
// the five-pass form; the z pass with the wide or narrow radix schedule and
// with 8 or 4 columns per CTA), keeps the fastest on the plan and reports every
// candidate's time as {fuse, fvar, zvar, ms}.
int marie_plan_autotune(marie_plan* p, int* fuse_out, int* fvar_out, int* zvar_out, double* ms_out, int64_t cap,
                        int64_t* count) {
  if (!p) return set_error(MARIE_EINVAL, "NULL plan");
  if (count) *count = 0;
  if (!p->has_op || !p->fN32) return MARIE_OK;  // nothing to tune without the FP32 operator
  cudaStream_t st = p->stream;
  const long long n = 3 * p->d.V;
  DBuf J, out, inv;
  MARIE_TRY(J.alloc(n * sizeof(double2), st));
  MARIE_TRY(out.alloc(n * sizeof(double2), st));
  MARIE_TRY(inv.alloc(n * sizeof(int), st));
  k_tune_fill<<<grid_for(n), 256, 0, st>>>(J.as<double2>(), inv.as<int>(), n);
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  Prologue pro{nullptr, 0};
  Epilogue ep{};
  ep.a_s = mk<double2>(1.0, 0.0);
  ep.b_s = mk<double2>(1.0, 0.0);
  auto wide = [](int n) { return n == 16 || n == 128 || n == 256; };
  const bool can_fuse = MatvecLaunch<float>::fused(p->d);
  const bool narrow_xy = can_fuse && (wide(p->d.Lp) || wide(p->d.Mp));
  // half-size clusters exist for the grids fused with clusters of 4 or 8
  const bool half_cluster = can_fuse && p->d.Lp >= 128;
  struct Cand { int fuse, fvar, zvar; double ms; };
  std::vector<Cand> cands;
  for (int f = can_fuse ? 1 : 0; f >= 0; --f)
    for (int fv = 0; fv < (f ? 3 : 1); ++fv) {
      if ((fv == 1 && !narrow_xy) || (fv == 2 && !half_cluster)) continue;
      for (int z = 0; z < 3; ++z)
        if (z != 1 || wide(p->d.Np)) cands.push_back({f, fv, z, 0.0});
    }
  const bool fuse0 = p->fuse;
  const int fvar0 = p->fvar, zvar0 = p->zvar;
  cudaEvent_t e0, e1;
  MARIE_CUDA_TRY(cudaEventCreate(&e0));
  MARIE_CUDA_TRY(cudaEventCreate(&e1));
  int status = MARIE_OK;
  for (auto& c : cands) {
    p->fuse = c.fuse != 0;
    p->fvar = c.fvar;
    p->zvar = c.zvar;
    const int reps = 5;
    for (int r = 0; r < 2 + reps && status == MARIE_OK; ++r) {
      if (r == 2) cudaEventRecord(e0, st);
      status = run_matvec(p, MARIE_FP32, J.as<double2>(), out.as<double2>(), n, 1, inv.as<int>(), pro, ep);
    }
    if (status != MARIE_OK) break;
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    c.ms = ms / reps;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (status != MARIE_OK) {
    p->fuse = fuse0;
    p->fvar = fvar0;
    p->zvar = zvar0;
    return status;
  }
  const Cand* best = &cands[0];
  for (const auto& c : cands)
    if (c.ms < best->ms) best = &c;
  p->fuse = best->fuse != 0;
  p->fvar = best->fvar;
  p->zvar = best->zvar;
  if (fuse_out) *fuse_out = best->fuse;
  if (fvar_out) *fvar_out = best->fvar;
  if (zvar_out) *zvar_out = best->zvar;
  for (size_t i = 0; i < cands.size() && (int64_t)i < cap && ms_out; ++i) {
    ms_out[4 * i] = cands[i].fuse;
    ms_out[4 * i + 1] = cands[i].fvar;
    ms_out[4 * i + 2] = cands[i].zvar;
    ms_out[4 * i + 3] = cands[i].ms;
  }
  if (count) *count = (int64_t)cands.size();
  return check_kernel_status(p);
}

int marie_plan_set_schedule(marie_plan* p, int fuse, int fvar, int zvar) {
  if (!p) return set_error(MARIE_EINVAL, "NULL plan");
  if (fvar < 0 || fvar > 2) return set_error(MARIE_EINVAL, "fvar must be 0, 1 or 2");
  if (zvar < 0 || zvar > 2) return set_error(MARIE_EINVAL, "zvar must be 0, 1 or 2");
  p->fuse = fuse != 0;
  p->fvar = fvar;
  p->zvar = zvar;
  return MARIE_OK;
}

int marie_plan_set_inner_precision(marie_plan* p, int precision) {
  if (!p) return set_error(MARIE_EINVAL, "NULL plan");
  if (precision != MARIE_FP32 && precision != MARIE_FP64)
    return set_error(MARIE_EINVAL, "inner precision must be MARIE_FP32 or MARIE_FP64");
  p->inner_prec = precision;
  return MARIE_OK;
}

int marie_plan_set_inner_restart(marie_plan* p, int restart) {
  if (!p) return set_error(MARIE_EINVAL, "NULL plan");
  if (restart < 0 || restart > 127) return set_error(MARIE_EINVAL, "inner restart must be 0 or in [1, 127]");
  p->inner_restart = restart;
  return MARIE_OK;
}

int marie_plan_set_batch_groups(marie_plan* p, int groups) {
  if (!p) return set_error(MARIE_EINVAL, "NULL plan");
  if (groups != 1 && groups != 2) return set_error(MARIE_EINVAL, "batch groups must be 1 or 2");
  p->batch_groups = groups;
  return MARIE_OK;
}

int marie_plan_set_graph_refinement(marie_plan* p, int on) {
  if (!p) return set_error(MARIE_EINVAL, "NULL plan");
  if (on != 0 && on != 1) return set_error(MARIE_EINVAL, "graph refinement must be 0 or 1");
  p->graph_refine = on != 0;
  return MARIE_OK;
}

int marie_release_cached_memory(void) {
  // blocks freed by finished calls go back to the device; blocks in use stay
  std::lock_guard<std::mutex> lock(g_pool_mu);
  for (auto& kv : g_pools) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaSetDevice(kv.first);
    cudaDeviceSynchronize();
    const cudaError_t e = cudaMemPoolTrimTo(kv.second, 0);
    cudaSetDevice(dev);
    if (e != cudaSuccess) return set_error(MARIE_ECUDA, "trimming the memory pool failed: %s", cudaGetErrorString(e));
  }
  return MARIE_OK;
}

int64_t marie_launch_count(void) { return g_launches.load(); }

int64_t marie_graph_loops(void) { return g_graph_loops.load(); }

void marie_inject_alloc_failure(int64_t nth) { g_fail_alloc_in.store(nth > 0 ? nth : 0); }

void marie_inject_tile_timeout(int64_t n) { g_tile_timeouts.store(n > 0 ? n : 0); }

int marie_plan_profile(marie_plan* p, int enable, double* pass_ms, int64_t* count) {
  if (!p) return set_error(MARIE_EINVAL, "NULL plan");
  if (pass_ms) {
    for (int k = 0; k < 5; ++k) pass_ms[k] = p->profiled ? p->pass_ms[k] / (double)p->profiled : 0.0;
  }
  if (count) *count = p->profiled;
  for (int k = 0; k < 5; ++k) p->pass_ms[k] = 0;
  p->profiled = 0;
  if (enable && !p->ev[0])
    for (int k = 0; k < 6; ++k) MARIE_CUDA_TRY(cudaEventCreate(&p->ev[k]));
  p->profile = enable != 0;
  return MARIE_OK;
}

int marie_set_operator(marie_plan* p, const double* fN, int64_t Lf, int64_t Mf, int64_t Nf) {
  if (!p || !fN) return set_error(MARIE_EINVAL, "NULL plan or operator");
  if (Lf != p->d.Lp || Mf != p->d.Mp || Nf != p->d.Np)
    return set_error(MARIE_EINVAL, "operator is %lldx%lldx%lld, plan expects %dx%dx%d", (long long)Lf,
                     (long long)Mf, (long long)Nf, p->d.Lp, p->d.Mp, p->d.Np);
  const size_t bytes = (size_t)6 * Lf * Mf * Nf * sizeof(double2);
  DBuf tmp;
  const void* dev = nullptr;
  MARIE_TRY(stage_in(fN, bytes, p->stream, tmp, &dev));
  return install_operator(p, (const double2*)dev);
}

int marie_set_operator_k(marie_plan* p, const double* fK, int64_t Lf, int64_t Mf, int64_t Nf) {
  if (!p || !fK) return set_error(MARIE_EINVAL, "NULL plan or operator");
  if (Lf != p->d.Lp || Mf != p->d.Mp || Nf != p->d.Np)
    return set_error(MARIE_EINVAL, "operator is %lldx%lldx%lld, plan expects %dx%dx%d", (long long)Lf,
                     (long long)Mf, (long long)Nf, p->d.Lp, p->d.Mp, p->d.Np);
  const size_t bytes = (size_t)3 * Lf * Mf * Nf * sizeof(double2);
  DBuf tmp;
  const void* dev = nullptr;
  MARIE_TRY(stage_in(fK, bytes, p->stream, tmp, &dev));
  return install_operator(p, (const double2*)dev, 1);
}

int marie_get_plan_operator(marie_plan* p, double* fN_out) {
  if (!p || !fN_out) return set_error(MARIE_EINVAL, "NULL plan or output");
  if (!p->has_op || !p->fN64) return set_error(MARIE_ENOOP, "plan holds no FP64 operator");
  const long long P = (long long)p->d.Lp * p->d.Mp * p->d.Np;
  const size_t bytes = (size_t)6 * P * sizeof(double2);
  DBuf tmp;
  void* dev = nullptr;
  MARIE_TRY(stage_out(fN_out, bytes, p->stream, tmp, &dev));
  if (p->oct)
    k_expand_octant<<<grid_for(6 * P), 256, 0, p->stream>>>(p->fN64, p->d.L, p->d.M, p->d.N, 0, (double)P,
                                                            (double2*)dev);
  else
    k_scale_convert<<<grid_for(6 * P), 256, 0, p->stream>>>(p->fN64, 6 * P, (double)P, (double2*)dev, nullptr);
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  MARIE_TRY(finish_out(fN_out, dev, bytes, p->stream));
  return MARIE_OK;
}

static int check_prec(marie_plan* p, int precision) {
  if (precision != MARIE_FP64 && precision != MARIE_FP32)
    return set_error(MARIE_EINVAL, "matvec precision must be MARIE_FP64 or MARIE_FP32");
  if (precision == MARIE_FP32 && !p->fN32) return set_error(MARIE_EINVAL, "plan has no FP32 operator");
  if (precision == MARIE_FP64 && !p->fN64) return set_error(MARIE_EINVAL, "plan has no FP64 operator");
  return MARIE_OK;
}

int marie_mv_AN(marie_plan* p, const double* JIn0, const double* Mr, const double* Mc, double Gram, int transp,
                const int64_t* idx, int64_t n_idx, double* JOut, int64_t nrhs, int precision) {
  if (!p || !JIn0 || !Mr || !Mc || !JOut || (!idx && n_idx > 0)) return set_error(MARIE_EINVAL, "NULL argument");
  if (nrhs < 1) return set_error(MARIE_EINVAL, "nrhs must be >= 1");
  if (transp != 0 && transp != 1) return set_error(MARIE_EINVAL, "transp must be 0 ('notransp') or 1 ('transp')");
  MARIE_TRY(check_prec(p, precision));
  if (!p->has_op) return set_error(MARIE_ENOOP, "plan has no operator");
  const long long V = p->d.V, n = n_idx;
  DBuf tJ, tMr, tMc, tidx, tout, inv, ca, cb;
  const void *J_d, *Mr_d, *Mc_d, *idx_d;
  void* out_d;
  MARIE_TRY(stage_in(JIn0, n * nrhs * sizeof(double2), p->stream, tJ, &J_d));
  MARIE_TRY(stage_in(Mr, V * sizeof(double2), p->stream, tMr, &Mr_d));
  MARIE_TRY(stage_in(Mc, V * sizeof(double2), p->stream, tMc, &Mc_d));
  MARIE_TRY(stage_in(idx, n * sizeof(int64_t), p->stream, tidx, &idx_d));
  MARIE_TRY(stage_out(JOut, n * nrhs * sizeof(double2), p->stream, tout, &out_d));
  MARIE_TRY(inv.alloc(3 * V * sizeof(int), p->stream));
  MARIE_TRY(ca.alloc(n * sizeof(double2), p->stream));
  MARIE_TRY(cb.alloc(n * sizeof(double2), p->stream));
  MARIE_TRY(build_inverse_index(p, (const int64_t*)idx_d, n, inv.as<int>()));
  MARIE_TRY(build_coefficients(p, (const int64_t*)idx_d, n, (const double2*)Mr_d, (const double2*)Mc_d, Gram, transp,
                               ca.as<double2>(), cb.as<double2>()));
  Prologue pro{nullptr, 0};
  Epilogue ep{};
  if (transp == 0) {
    ep.a = ca.as<double2>();
    ep.b = cb.as<double2>();
    ep.conjout = 0;
  } else {
    pro.pre = cb.as<double2>();
    pro.conjin = 1;
    ep.a = ca.as<double2>();
    ep.conjout = 1;
  }
  if (n > 0)
    MARIE_TRY(run_matvec(p, precision, (const double2*)J_d, (double2*)out_d, n, (int)nrhs, inv.as<int>(), pro, ep));
  MARIE_TRY(finish_out(JOut, out_d, n * nrhs * sizeof(double2), p->stream));
  MARIE_CUDA_TRY(cudaStreamSynchronize(p->stream));
  return check_kernel_status(p);
}

int marie_plan_apply_mv_AN(marie_plan* p, const double* JIn0, double* JOut, int64_t nrhs, int precision) {
  if (!p || !JIn0 || !JOut) return set_error(MARIE_EINVAL, "NULL argument");
  if (nrhs < 1) return set_error(MARIE_EINVAL, "nrhs must be >= 1");
  if (!p->bnd_n) return set_error(MARIE_EINVAL, "no mv_AN bound to the plan (marie_plan_bind_mv_AN)");
  MARIE_TRY(check_prec(p, precision));
  const long long n = p->bnd_n;
  DBuf tJ, tout;
  const void* J_d;
  void* out_d;
  MARIE_TRY(stage_in(JIn0, n * nrhs * sizeof(double2), p->stream, tJ, &J_d));
  MARIE_TRY(stage_out(JOut, n * nrhs * sizeof(double2), p->stream, tout, &out_d));
  Prologue pro{nullptr, 0};
  Epilogue ep{};
  ep.a = p->bnd_a;
  if (p->bnd_transp == 0) {
    ep.b = p->bnd_b;
  } else {
    pro.pre = p->bnd_b;
    pro.conjin = 1;
    ep.conjout = 1;
  }
  if (precision == MARIE_FP32) {
    // the FP32 operator's epilogue in FP32, as in the solver's inner matvecs
    ep.af = p->bnd_af;
    ep.bf = p->bnd_bf;
  }
  MARIE_TRY(run_matvec(p, precision, (const double2*)J_d, (double2*)out_d, n, (int)nrhs, p->bnd_inv, pro, ep));
  if (out_d != JOut) {
    MARIE_TRY(finish_out(JOut, out_d, n * nrhs * sizeof(double2), p->stream));
    return check_kernel_status(p);
  }
  MARIE_CUDA_TRY(cudaGetLastError());
  return MARIE_OK;
}

int marie_mv_L(marie_plan* p, const double* JIn0, double Gram, const int64_t* idx, int64_t n_idx, double* JOut,
               int64_t nrhs, int precision) {
  if (!p || !JIn0 || !JOut || (!idx && n_idx > 0)) return set_error(MARIE_EINVAL, "NULL argument");
  if (nrhs < 1) return set_error(MARIE_EINVAL, "nrhs must be >= 1");
  MARIE_TRY(check_prec(p, precision));
  if (!p->has_op) return set_error(MARIE_ENOOP, "plan has no operator");
  const long long V = p->d.V, n = n_idx;
  DBuf tJ, tidx, tout, inv;
  const void *J_d, *idx_d;
  void* out_d;
  MARIE_TRY(stage_in(JIn0, n * nrhs * sizeof(double2), p->stream, tJ, &J_d));
  MARIE_TRY(stage_in(idx, n * sizeof(int64_t), p->stream, tidx, &idx_d));
  MARIE_TRY(stage_out(JOut, n * nrhs * sizeof(double2), p->stream, tout, &out_d));
  MARIE_TRY(inv.alloc(3 * V * sizeof(int), p->stream));
  MARIE_TRY(build_inverse_index(p, (const int64_t*)idx_d, n, inv.as<int>()));
  Prologue pro{nullptr, 0};
  Epilogue ep{};
  ep.a_s = mk<double2>(-Gram, 0.0);
  ep.b_s = mk<double2>(-1.0, 0.0);
  if (n > 0)
    MARIE_TRY(run_matvec(p, precision, (const double2*)J_d, (double2*)out_d, n, (int)nrhs, inv.as<int>(), pro, ep));
  MARIE_TRY(finish_out(JOut, out_d, n * nrhs * sizeof(double2), p->stream));
  MARIE_CUDA_TRY(cudaStreamSynchronize(p->stream));
  return check_kernel_status(p);
}

int marie_mv_K(marie_plan* p, const double* JIn0, const int64_t* idx, int64_t n_idx, double* JOut, int64_t nrhs,
               int precision) {
  if (!p || !JIn0 || !JOut || (!idx && n_idx > 0)) return set_error(MARIE_EINVAL, "NULL argument");
  if (nrhs < 1) return set_error(MARIE_EINVAL, "nrhs must be >= 1");
  if (precision != MARIE_FP64 && precision != MARIE_FP32)
    return set_error(MARIE_EINVAL, "precision must be MARIE_FP64 or MARIE_FP32");
  if (!p->has_opK) return set_error(MARIE_ENOOP, "plan has no K operator");
  const long long V = p->d.V, n = n_idx;
  DBuf tJ, tidx, tout, inv;
  const void *J_d, *idx_d;
  void* out_d;
  MARIE_TRY(stage_in(JIn0, n * nrhs * sizeof(double2), p->stream, tJ, &J_d));
  MARIE_TRY(stage_in(idx, n * sizeof(int64_t), p->stream, tidx, &idx_d));
  MARIE_TRY(stage_out(JOut, n * nrhs * sizeof(double2), p->stream, tout, &out_d));
  MARIE_TRY(inv.alloc(3 * V * sizeof(int), p->stream));
  MARIE_TRY(build_inverse_index(p, (const int64_t*)idx_d, n, inv.as<int>()));
  // out = crop(IFFT(fK x FFT(J))): no diagonal term
  Prologue pro{nullptr, 0};
  Epilogue ep{};
  ep.a_s = mk<double2>(0.0, 0.0);
  ep.b_s = mk<double2>(-1.0, 0.0);
  if (n > 0)
    MARIE_TRY(run_matvec(p, precision, (const double2*)J_d, n, (double2*)out_d, n, n, (int)nrhs, inv.as<int>(), pro,
                         ep, nullptr, 0, 1));
  MARIE_TRY(finish_out(JOut, out_d, n * nrhs * sizeof(double2), p->stream));
  MARIE_CUDA_TRY(cudaStreamSynchronize(p->stream));
  return MARIE_OK;
}

}  // extern "C"
