// The FP32 mv_AN ('notransp') built on cuFFT, timed beside the hand-written
// matvec as a comparison.  It is the sequence the reference runs through
// MATLAB's gpuArray fftn (mv_AN.m:101-131): scatter J into three zero-padded
// 2L x 2M x 2N arrays, batched 3-D forward transform, the symmetric 3x3
// product with the full operator, batched inverse transform, crop, and the
// epilogue Gram*Mr*J - Mc*(N J).  The cuFFT plan, the full FP32 operator and
// the padded arrays are kept with the plan after the first call.
#include <cufft.h>

#include <map>
#include <mutex>

#include "plan.h"

namespace marie {

__global__ void k_cf_scatter(const double2* __restrict__ J, const int64_t* __restrict__ idx, long long n, int L,
                             int M, int N, long long P, float2* __restrict__ X) {
  const long long V = (long long)L * M * N;
  const long long Lp = 2LL * L, Mp = 2LL * M;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const long long g = idx[k] - 1;
    const long long c = g / V, v = g - c * V;
    const long long x = v % L, y = (v / L) % M, z = v / ((long long)L * M);
    const double2 j = J[k];
    X[c * P + x + Lp * (y + Mp * z)] = mk<float2>((float)j.x, (float)j.y);
  }
}

// Y_c = sum_q N(c,q) X_q with the symmetric tensor [xx xy xz; xy yy yz; xz yz zz]
__global__ void k_cf_multiply(const float2* __restrict__ X, const float2* __restrict__ F, long long P,
                              float2* __restrict__ Y) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < P; t += (long long)gridDim.x * blockDim.x) {
    const float2 x0 = X[t], x1 = X[P + t], x2 = X[2 * P + t];
    const float2 xx = F[t], xy = F[P + t], xz = F[2 * P + t], yy = F[3 * P + t], yz = F[4 * P + t],
                 zz = F[5 * P + t];
    Y[t] = cadd(cadd(cmul(xx, x0), cmul(xy, x1)), cmul(xz, x2));
    Y[P + t] = cadd(cadd(cmul(xy, x0), cmul(yy, x1)), cmul(yz, x2));
    Y[2 * P + t] = cadd(cadd(cmul(xz, x0), cmul(yz, x1)), cmul(zz, x2));
  }
}

__global__ void k_cf_gather(const double2* __restrict__ J, const int64_t* __restrict__ idx, long long n, int L, int M,
                            int N, long long P, const float2* __restrict__ Y, const double2* __restrict__ Mr,
                            const double2* __restrict__ Mc, double Gram, double2* __restrict__ out) {
  const long long V = (long long)L * M * N;
  const long long Lp = 2LL * L, Mp = 2LL * M;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const long long g = idx[k] - 1;
    const long long c = g / V, v = g - c * V;
    const long long x = v % L, y = (v / L) % M, z = v / ((long long)L * M);
    const float2 f = Y[c * P + x + Lp * (y + Mp * z)];
    const double2 nj = mk<double2>(f.x, f.y);
    const double2 a = mk<double2>(Gram * Mr[v].x, Gram * Mr[v].y);
    out[k] = csub(cmul(a, J[k]), cmul(Mc[v], nj));
  }
}

// full FP32 operator from the plan's FP32 octant (already scaled by 1/(8LMN))
__global__ void k_cf_expand(const float2* __restrict__ o, int L, int M, int N, float2* __restrict__ f) {
  const long long Lp = 2LL * L, Mp = 2LL * M, Np = 2LL * N, P = Lp * Mp * Np;
  const long long Lo = L + 1, Mo = M + 1, No = N + 1, O = Lo * Mo * No;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < 6 * P; t += (long long)gridDim.x * blockDim.x) {
    const int q = (int)(t / P);
    long long r = t - q * P;
    const long long ix = r % Lp;
    r /= Lp;
    const long long iy = r % Mp, iz = r / Mp;
    const long long jx = ix > L ? Lp - ix : ix, jy = iy > M ? Mp - iy : iy, jz = iz > N ? Np - iz : iz;
    const bool neg = ((ix > L) && OpKind<0>::odd(q, 0)) ^ ((iy > M) && OpKind<0>::odd(q, 1)) ^
                     ((iz > N) && OpKind<0>::odd(q, 2));
    const float2 v = o[q * O + jx + Lo * (jy + Mo * jz)];
    f[t] = neg ? mk<float2>(-v.x, -v.y) : v;
  }
}

namespace {

struct CufftState {
  cufftHandle plan = 0;
  float2 *F = nullptr, *X = nullptr, *Y = nullptr;
  long long P = 0;
  ~CufftState() {
    if (plan) cufftDestroy(plan);
    cudaFree(F);
    cudaFree(X);
    cudaFree(Y);
  }
};

std::mutex g_cf_mu;
std::map<const marie_plan*, CufftState*> g_cf;

inline int grid_cf(long long n) { return grid_stride_blocks(n, 16); }

int cufft_state(marie_plan* p, CufftState** out) {
  std::lock_guard<std::mutex> lock(g_cf_mu);
  auto it = g_cf.find(p);
  if (it != g_cf.end()) {
    *out = it->second;
    return MARIE_OK;
  }
  auto* s = new CufftState();
  const Dims& d = p->d;
  s->P = (long long)d.Lp * d.Mp * d.Np;
  if (cudaMalloc(&s->F, 6 * s->P * sizeof(float2)) != cudaSuccess ||
      cudaMalloc(&s->X, 3 * s->P * sizeof(float2)) != cudaSuccess ||
      cudaMalloc(&s->Y, 3 * s->P * sizeof(float2)) != cudaSuccess) {
    delete s;
    cudaGetLastError();
    return set_error(MARIE_ENOMEM, "cuFFT comparison: device allocation failed");
  }
  // x fastest (column-major grid) = cuFFT's last dimension
  int n[3] = {d.Np, d.Mp, d.Lp};
  if (cufftPlanMany(&s->plan, 3, n, nullptr, 1, (int)s->P, nullptr, 1, (int)s->P, CUFFT_C2C, 3) != CUFFT_SUCCESS ||
      cufftSetStream(s->plan, p->stream) != CUFFT_SUCCESS) {
    delete s;
    return set_error(MARIE_ECUDA, "cuFFT comparison: plan creation failed");
  }
  if (p->oct) {
    k_cf_expand<<<grid_cf(6 * s->P), 256, 0, p->stream>>>(p->fN32, d.L, d.M, d.N, s->F);
    count_launch();
  } else {
    MARIE_CUDA_TRY(cudaMemcpyAsync(s->F, p->fN32, 6 * s->P * sizeof(float2), cudaMemcpyDeviceToDevice, p->stream));
  }
  MARIE_CUDA_TRY(cudaGetLastError());
  MARIE_CUDA_TRY(cudaStreamSynchronize(p->stream));
  g_cf[p] = s;
  *out = s;
  return MARIE_OK;
}

}  // namespace

void release_cufft_state(const marie_plan* p) {
  std::lock_guard<std::mutex> lock(g_cf_mu);
  auto it = g_cf.find(p);
  if (it == g_cf.end()) return;
  delete it->second;
  g_cf.erase(it);
}

}  // namespace marie

using namespace marie;

extern "C" int marie_mv_AN_cufft(marie_plan* p, const double* JIn0, const double* Mr, const double* Mc, double Gram,
                                 const int64_t* idx, int64_t n_idx, double* JOut, float* ms) {
  if (!p || !JIn0 || !Mr || !Mc || !JOut || !idx || n_idx < 1) return set_error(MARIE_EINVAL, "NULL argument");
  if (!p->has_op || !p->fN32) return set_error(MARIE_ENOOP, "plan holds no FP32 operator");
  if (n_idx > 3 * p->d.V) return set_error(MARIE_EINVAL, "n_idx outside [1, 3*L*M*N]");
  CufftState* s = nullptr;
  MARIE_TRY(cufft_state(p, &s));
  cudaStream_t st = p->stream;
  const long long V = p->d.V, n = n_idx;
  DBuf tJ, tMr, tMc, tidx, tout;
  const void *J_d, *Mr_d, *Mc_d, *idx_d;
  void* out_d;
  MARIE_TRY(stage_in(JIn0, n * sizeof(double2), st, tJ, &J_d));
  MARIE_TRY(stage_in(Mr, V * sizeof(double2), st, tMr, &Mr_d));
  MARIE_TRY(stage_in(Mc, V * sizeof(double2), st, tMc, &Mc_d));
  MARIE_TRY(stage_in(idx, n * sizeof(int64_t), st, tidx, &idx_d));
  MARIE_TRY(stage_out(JOut, n * sizeof(double2), st, tout, &out_d));
  cudaEvent_t e0, e1;
  MARIE_CUDA_TRY(cudaEventCreate(&e0));
  MARIE_CUDA_TRY(cudaEventCreate(&e1));
  MARIE_CUDA_TRY(cudaEventRecord(e0, st));
  MARIE_CUDA_TRY(cudaMemsetAsync(s->X, 0, 3 * s->P * sizeof(float2), st));
  k_cf_scatter<<<grid_cf(n), 256, 0, st>>>((const double2*)J_d, (const int64_t*)idx_d, n, p->d.L, p->d.M, p->d.N,
                                           s->P, s->X);
  const bool ok1 = cufftExecC2C(s->plan, (cufftComplex*)s->X, (cufftComplex*)s->X, CUFFT_FORWARD) == CUFFT_SUCCESS;
  k_cf_multiply<<<grid_cf(s->P), 256, 0, st>>>(s->X, s->F, s->P, s->Y);
  const bool ok2 = cufftExecC2C(s->plan, (cufftComplex*)s->Y, (cufftComplex*)s->Y, CUFFT_INVERSE) == CUFFT_SUCCESS;
  k_cf_gather<<<grid_cf(n), 256, 0, st>>>((const double2*)J_d, (const int64_t*)idx_d, n, p->d.L, p->d.M, p->d.N,
                                          s->P, s->Y, (const double2*)Mr_d, (const double2*)Mc_d, Gram,
                                          (double2*)out_d);
  count_launch(3);
  MARIE_CUDA_TRY(cudaEventRecord(e1, st));
  MARIE_CUDA_TRY(cudaGetLastError());
  MARIE_CUDA_TRY(cudaEventSynchronize(e1));
  float t = 0;
  MARIE_CUDA_TRY(cudaEventElapsedTime(&t, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!ok1 || !ok2) return set_error(MARIE_ECUDA, "cuFFT execution failed");
  if (ms) *ms = t;
  MARIE_TRY(finish_out(JOut, out_d, n * sizeof(double2), st));
  MARIE_CUDA_TRY(cudaStreamSynchronize(st));
  return MARIE_OK;
}
