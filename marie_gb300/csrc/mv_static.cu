// marie_mv_AN_static: the circulant matvec for callers that cannot allocate
// device memory.
//
// marie_mv_AN takes its scratch (the grid-to-DOF index map, the per-DOF
// coefficients and the padded FFT spectra) from the plan's workspace, which it
// grows with cudaMalloc on demand.  Some callers cannot let a library allocate
// at the moment they ask for a matvec: a host whose device memory is owned by
// another allocator (MATLAB's gpuArray pool, a serving runtime with a fixed
// arena, where a cudaMalloc behind its back can fail or fragment its pool), or
// a real-time loop that must not block in the driver's allocator.  This entry
// point serves them without any allocation: its scratch is one file-scope
// __device__ array of kStaticScratchBytes, which every GPU that loads this
// library holds until the process exits.  Inputs and outputs stay the caller's
// device buffers; the plan (operator and twiddles) is created beforehand.
//
// Set-up: the first call for a device looks up the array's device address with
// cudaGetSymbolAddress, with that device (the plan's) current, and caches it.
// A call runs on the plan's device and stream whatever device is current, and
// restores the caller's current device before it returns.  Each call blocks
// the host until its stream is done (it reads the status of the index check,
// then finishes the product), so the entry point cannot be captured into a
// CUDA graph.  Every call shares the one array and it keeps the previous call's
// contents, so each call resets what must start clean (the error flag and the
// index map); two calls that overlap on the GPU (other streams, other threads,
// other plans on the same device) race on it.  The passes run with the plan's
// schedule (marie_plan_autotune / marie_plan_set_schedule), as marie_mv_AN's do.
#include <map>
#include <mutex>

#include "matvec_launch.cuh"
#include "plan.h"

namespace marie {
// index-map and coefficient kernels of capi.cu
__global__ void k_fill_int(int* a, long long n, int v);
__global__ void k_scatter_inverse(const int64_t* idx, long long n, long long n3V, int* inv, int* err);
__global__ void k_coefficients(const int64_t* idx, long long n, long long V, const double2* Mr, const double2* Mc,
                               double Gram, int mode, double2* a, double2* b);
}  // namespace marie

using namespace marie;

// 64 MiB: an FP32 matvec needs about 204 bytes per voxel on grids with the
// fused x+y passes and 252 on the others (up to 64^3 voxels fit); an FP64 one
// about 396 (up to about 160k voxels).
static constexpr size_t kStaticScratchBytes = 64ull << 20;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

// In host code g_static_scratch is only a host-side stand-in for the device
// symbol, never a device address: the address is looked up once per device.
static std::mutex g_scratch_mu;
static std::map<int, unsigned char*> g_scratch_addr;

// dev must be the current device
static int scratch_address(int dev, unsigned char** out) {
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  auto it = g_scratch_addr.find(dev);
  if (it != g_scratch_addr.end()) {
    *out = it->second;
    return MARIE_OK;
  }
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
  if (e != cudaSuccess || !p)
    return set_error(MARIE_ECUDA, "cudaGetSymbolAddress of the static scratch failed: %s", cudaGetErrorString(e));
  g_scratch_addr[dev] = static_cast<unsigned char*>(p);
  *out = static_cast<unsigned char*>(p);
  return MARIE_OK;
}

static size_t up256(size_t b) { return (b + 255) & ~size_t(255); }

template <typename T>
static int static_matvec(marie_plan* p, const double2* J, const double2* Mr, const double2* Mc, double Gram,
                         int transp, const int64_t* idx, long long n, double2* out, unsigned char* scratch) {
  using ML = MatvecLaunch<T>;
  using V = cplx<T>;
  const Dims d = p->d;
  const long long V3 = 3 * d.V;
  const bool fused = p->fuse && ML::fused(d);
  // scratch layout: error flag | inv[3V] | a[n] | b[n] | B spectra | A spectra (grids without fused passes)
  size_t off = 0;
  int* err = reinterpret_cast<int*>(scratch + off);
  off += 256;
  int* inv = reinterpret_cast<int*>(scratch + off);
  off += up256(V3 * sizeof(int));
  double2* ca = reinterpret_cast<double2*>(scratch + off);
  off += up256(n * sizeof(double2));
  double2* cb = reinterpret_cast<double2*>(scratch + off);
  off += up256(n * sizeof(double2));
  V* B = reinterpret_cast<V*>(scratch + off);
  off += up256(p->elems_B() * sizeof(V));
  V* A = reinterpret_cast<V*>(scratch + off);
  if (!fused) off += up256(p->elems_A() * sizeof(V));
  if (off > kStaticScratchBytes)
    return set_error(MARIE_EINVAL,
                     "marie_mv_AN_static: this grid and DOF count need %zu bytes of scratch, more than the %zu of "
                     "its static array; use marie_mv_AN",
                     off, kStaticScratchBytes);
  cudaStream_t st = p->stream;
  const int g = sm_count() * 8;
  // the array keeps the previous call's contents: reset the flag and the map
  MARIE_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));
  k_fill_int<<<g, 256, 0, st>>>(inv, V3, -1);
  count_launch();
  if (n > 0) {
    k_scatter_inverse<<<g, 256, 0, st>>>(idx, n, V3, inv, err);
    count_launch();
  }
  MARIE_CUDA_TRY(cudaGetLastError());
  int herr = 0;
  MARIE_CUDA_TRY(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  if (herr & 1) return set_error(MARIE_EINVAL, "idx entry outside [1, 3*L*M*N]");
  if (herr & 2) return set_error(MARIE_EINVAL, "idx has repeated entries");
  if (n == 0) return MARIE_OK;
  k_coefficients<<<g, 256, 0, st>>>(idx, n, d.V, Mr, Mc, Gram, transp, ca, cb);
  count_launch();
  MARIE_CUDA_TRY(cudaGetLastError());
  Prologue pro{nullptr, 0};
  Epilogue ep{};
  if (transp == 0) {
    ep.a = ca;
    ep.b = cb;
  } else {
    pro.pre = cb;
    pro.conjin = 1;
    ep.a = ca;
    ep.conjout = 1;
  }
  const V* fN = sizeof(T) == 4 ? reinterpret_cast<const V*>(p->fN32) : reinterpret_cast<const V*>(p->fN64);
  V* const* tw = sizeof(T) == 4 ? reinterpret_cast<V* const*>(p->tw32) : reinterpret_cast<V* const*>(p->tw64);
  const long long sA = p->elems_A(), sB = p->elems_B();
  if (fused) {
    MARIE_CUDA_TRY(ML::xyfwd(J, n, inv, pro, B, sB, d, tw[0], tw[1], 1, st, p->fvar));
    MARIE_CUDA_TRY(ML::zmul(B, sB, fN, p->oct, d, tw[2], 1, st, 0, p->zvar));
    MARIE_CUDA_TRY(ML::yxinv(B, sB, J, n, inv, ep, out, n, d, tw[0], tw[1], 1, st, p->fvar));
    count_launch(3);
  } else {
    MARIE_CUDA_TRY(ML::xfwd(J, n, inv, pro, A, sA, d, tw[0], 1, st));
    MARIE_CUDA_TRY(ML::cols(false, d.Mp, A, (long long)d.Lp * d.M, sA, d.M, B, (long long)d.Lp * d.Mp, sB, d.Mp,
                            d.Lp, 3 * d.N, tw[1], 1, st));
    MARIE_CUDA_TRY(ML::zmul(B, sB, fN, p->oct, d, tw[2], 1, st, 0, p->zvar));
    MARIE_CUDA_TRY(ML::cols(true, d.Mp, B, (long long)d.Lp * d.Mp, sB, d.Mp, A, (long long)d.Lp * d.M, sA, d.M,
                            d.Lp, 3 * d.N, tw[1], 1, st));
    MARIE_CUDA_TRY(ML::xinv(A, sA, J, n, inv, ep, out, n, d, tw[0], 1, st));
    count_launch(5);
  }
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  return MARIE_OK;
}

namespace {
// makes the plan's device current for one call and restores the caller's
struct DeviceScope {
  int prev = -1;
  bool switched = false;
  int enter(int dev) {
    MARIE_CUDA_TRY(cudaGetDevice(&prev));
    if (prev != dev) {
      MARIE_CUDA_TRY(cudaSetDevice(dev));
      switched = true;
    }
    return MARIE_OK;
  }
  ~DeviceScope() {
    if (switched) cudaSetDevice(prev);
  }
};
}  // namespace

static int mv_static_on_device(marie_plan* p, const double* JIn0, const double* Mr, const double* Mc, double Gram,
                               int transp, const int64_t* idx, int64_t n_idx, double* JOut, int precision);

extern "C" int marie_mv_AN_static(marie_plan* p, const double* JIn0, const double* Mr, const double* Mc, double Gram,
                                  int transp, const int64_t* idx, int64_t n_idx, double* JOut, int precision) {
  if (!p || !JIn0 || !Mr || !Mc || !JOut || (!idx && n_idx > 0)) return set_error(MARIE_EINVAL, "NULL argument");
  DeviceScope scope;
  MARIE_TRY(scope.enter(p->device));
  return mv_static_on_device(p, JIn0, Mr, Mc, Gram, transp, idx, n_idx, JOut, precision);
}

static int mv_static_on_device(marie_plan* p, const double* JIn0, const double* Mr, const double* Mc, double Gram,
                               int transp, const int64_t* idx, int64_t n_idx, double* JOut, int precision) {
  if (transp != 0 && transp != 1) return set_error(MARIE_EINVAL, "transp must be 0 ('notransp') or 1 ('transp')");
  if (!p->has_op) return set_error(MARIE_ENOOP, "plan has no operator");
  if (precision == MARIE_FP32 ? !p->fN32 : (precision == MARIE_FP64 ? !p->fN64 : true))
    return set_error(MARIE_EINVAL, "precision must be MARIE_FP64 or MARIE_FP32 and held by the plan");
  if (n_idx < 0 || n_idx > 3 * p->d.V) return set_error(MARIE_EINVAL, "n_idx outside [0, 3*L*M*N]");
  // host buffers would need staging allocations: device memory only
  if (!is_device_ptr(JIn0) || !is_device_ptr(Mr) || !is_device_ptr(Mc) || !is_device_ptr(JOut) ||
      (n_idx > 0 && !is_device_ptr(idx)))
    return set_error(MARIE_EINVAL, "marie_mv_AN_static takes device pointers only");
  unsigned char* scratch = nullptr;
  MARIE_TRY(scratch_address(p->device, &scratch));
  if (precision == MARIE_FP32)
    return static_matvec<float>(p, (const double2*)JIn0, (const double2*)Mr, (const double2*)Mc, Gram, transp, idx,
                                n_idx, (double2*)JOut, scratch);
  return static_matvec<double>(p, (const double2*)JIn0, (const double2*)Mr, (const double2*)Mc, Gram, transp, idx,
                               n_idx, (double2*)JOut, scratch);
}
