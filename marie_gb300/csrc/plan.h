// Internal plan state shared by the C-ABI translation units.
#pragma once
#include <unistd.h>

#include <functional>
#include <memory>
#include <thread>
#include <vector>

#include "common.cuh"
#include "matvec_launch.cuh"
#include "trace.h"

struct marie_plan {
  marie::Dims d{};
  int precision = MARIE_FP64;
  long long nrhs_max = 1;
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;

  // Operator, pre-scaled by 1/(8LMN): octant or full 2L x 2M x 2N x 6 layout.
  double2* fN64 = nullptr;
  float2* fN32 = nullptr;
  bool has_op = false;
  bool fuse = true;  // fused x+y / y+x passes when the grid has them
  int fvar = 0;      // x/y radix schedule of the fused passes (set by marie_plan_autotune)
  int zvar = 0;      // z-pass variant of the FP32 N matvec (set by marie_plan_autotune)
  int inner_prec = MARIE_FP64;  // Krylov basis of the mixed-precision inner solves
  int inner_restart = 0;        // their restart length (0: the caller's inner_it)
  int batch_groups = 2;         // batched GMRES: systems split into this many groups on their own streams
  bool graph_refine = true;     // conditional-graph loops (refinement, restart cycles); host-driven when false
  int oct = 0;  // 1: fN64/fN32 hold the (L+1)(M+1)(N+1) octant, 0: the full array

  // The FP32 N operator stored full along x for the z pass's bulk tile copy
  // (fN32x[q][oz][oy][kx], 2L x (M+1) x (N+1) x 6, x reflections signed in),
  // with its tensor maps; built beside the octant when the operator has the
  // circulant parity symmetry and N + 1 <= 256.
  float2* fN32x = nullptr;
  marie::ZTile zt{};
  // Device status word of the kernels' bounded waits (1: a tile copy did not
  // arrive in time); read and cleared by check_kernel_status.
  int* kerr = nullptr;

  // K operator (mv_K, H_field_Kop), same scaling and layouts with 3 components.
  double2* fK64 = nullptr;
  float2* fK32 = nullptr;
  bool has_opK = false;
  int octK = 0;

  // Twiddle tables exp(-2*pi*i*k/n) for the three padded axis lengths.
  double2* tw64[3] = {nullptr, nullptr, nullptr};
  float2* tw32[3] = {nullptr, nullptr, nullptr};

  // Spectra workspaces (A: 3 x N x M x 2L, B: 3 x N x 2M x 2L per rhs).
  void* wsA = nullptr;
  void* wsB = nullptr;
  size_t ws_bytes_A = 0, ws_bytes_B = 0;

  // Optional per-pass timing of the matvec (events recorded between passes).
  bool profile = false;
  cudaEvent_t ev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
  float pass_ms[5] = {0, 0, 0, 0, 0};
  long long profiled = 0;

  // mv_AN bound by marie_plan_bind_mv_AN: the operator of marie_pgmres,
  // marie_pgmres_dr and marie_bicgstab when their A is NULL (DOF indices,
  // inverse map, epilogue / prologue coefficients; device, plan-owned).
  int64_t* bnd_idx = nullptr;
  int* bnd_inv = nullptr;
  double2* bnd_a = nullptr;
  double2* bnd_b = nullptr;
  float2* bnd_af = nullptr;  // FP32 copies of bnd_a / bnd_b (plans with an FP32 operator)
  float2* bnd_bf = nullptr;
  long long bnd_n = 0;
  int bnd_transp = 0;

  // Pinned host staging for small scalars (reductions, Hessenberg columns).
  double* pinned = nullptr;
  size_t pinned_len = 0;

  long long elems_A() const { return 3LL * d.Lp * d.M * d.N; }
  long long elems_B() const { return 3LL * d.Lp * d.Mp * d.N; }
};

namespace marie {

// Device buffer that is released on scope exit (stream-ordered).
struct DBuf {
  void* p = nullptr;
  cudaStream_t s = nullptr;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  ~DBuf() { if (p) cudaFreeAsync(p, s); }
  int alloc(size_t bytes, cudaStream_t st);
  template <typename T> T* as() const { return reinterpret_cast<T*>(p); }
};

// True when ptr is device (or managed) memory of the current device.
bool is_device_ptr(const void* ptr);

enum class HostKind { Device, Pinned, Pageable };
HostKind host_kind(const void* ptr);
// Host-to-device copy queued on st; pageable sources of 8 MB and more go
// through the library's pinned ring (the call returns once the source has
// been read).  Device-to-host copy that returns once `host` holds the data.
int copy_to_device(void* dev, const void* host, size_t bytes, cudaStream_t st);
int copy_to_host(void* host, const void* dev, size_t bytes, cudaStream_t st);

// Input view: device pointer to `bytes` of data, copying from host if needed.
int stage_in(const void* user, size_t bytes, cudaStream_t st, DBuf& tmp, const void** dev);
// Output view: device pointer to write to; finish_out copies back to host.
int stage_out(void* user, size_t bytes, cudaStream_t st, DBuf& tmp, void** dev);
int finish_out(void* user, const void* dev, size_t bytes, cudaStream_t st);

// Faults in the pages of a host output buffer on a helper thread (one write
// per page), so that the operating system's zero-fill of freshly mapped pages
// runs while the device solves instead of inside the final device-to-host
// copy.  Device pointers are left alone.  join() before writing the buffer.
struct HostPrefault {
  std::thread t;
  void start(void* user, size_t bytes) {
    if (!user || bytes == 0 || is_device_ptr(user)) return;
    t = std::thread([user, bytes] {
      const long pg = sysconf(_SC_PAGESIZE);
      const size_t step = pg > 0 ? (size_t)pg : 4096;
      volatile char* c = static_cast<volatile char*>(user);
      for (size_t off = 0; off < bytes; off += step) c[off] = 0;
      c[bytes - 1] = 0;
    });
  }
  void join() {
    if (t.joinable()) t.join();
  }
  ~HostPrefault() { join(); }
};

int ensure_workspace(marie_plan* p, int prec, long long nrhs, bool with_A = true);
int ensure_pinned(marie_plan* p, size_t n_doubles);

// Build the inverse map inv[g] = k for 1-based idx[k]; -1 elsewhere.  Fails on
// out-of-range or repeated indices.
int build_inverse_index(marie_plan* p, const int64_t* idx_dev, long long n, int* inv);

// One circulant matvec (nrhs columns of length n, device pointers).
int run_matvec(marie_plan* p, int prec, const double2* J, double2* out, long long n, int nrhs, const int* inv,
               const Prologue& pro, const Epilogue& ep);
// Same with column strides js / os and the batched-solve skip mask: column r
// is left untouched when stop[r] < step.
int run_matvec(marie_plan* p, int prec, const double2* J, long long js, double2* out, long long os, long long n,
               int nrhs, const int* inv, const Prologue& pro, const Epilogue& ep, const int* stop, int step,
               int kind = 0);
// FP32 matvec on FP32 vectors (FP32 arithmetic throughout, the epilogue's
// per-DOF coefficients from ep.af / ep.bf).
int run_matvec32(marie_plan* p, const float2* J, long long js, float2* out, long long os, long long n, int nrhs,
                 const int* inv, const Prologue& pro, const Epilogue& ep, const int* stop, int step, int kind = 0);

// Scale fN by 1/(8LMN) into the plan's FP64/FP32 copies (fN_dev: full layout).
// kind 0: the N operator (6 components), 1: the K operator (3 components).
int install_operator(marie_plan* p, const double2* fN_dev, int kind = 0);

// Reads the plan's kernel status word after the plan's stream has finished
// (a synchronising copy), clears it and returns MARIE_ETIMEOUT if a kernel's
// bounded wait ran out.
int check_kernel_status(marie_plan* p);

// Per-DOF coefficient arrays for mv_AN: (a, b) or (pre, a) for the adjoint.
// mode 0: a = Gram*Mr, b = Mc      mode 1: pre = Mc, a = Gram*conj(Mr)
int build_coefficients(marie_plan* p, const int64_t* idx_dev, long long n, const double2* Mr,
                       const double2* Mc, double Gram, int mode, double2* a, double2* b);

// Drops the cuFFT comparison state of a plan (cufft_compare.cu), if any.
void release_cufft_state(const marie_plan* p);

// Deterministic reductions and vector kernels (krylov.cu).
int dev_norm2(marie_plan* p, const double2* x, long long n, double* out_host);

// A linear operator on device vectors of length n.
using DevOp = std::function<int(const double2* x, double2* y)>;

// The plan's bound mv_AN as a DevOp on n DOFs (fails with MARIE_EINVAL when
// nothing is bound or n differs).
int bound_operator(marie_plan* p, long long n, DevOp* op);

struct GmresResult {
  int flag = 1;
  double relres = 0;
  int iter[2] = {0, 0};
  std::vector<double> resvec;
};

// A batched linear operator: out_s = Op(in_s) for the systems s whose stop[s]
// is not below step (in_s = in + s*is, out_s = out + s*os).
struct BatchOp {
  std::function<int(const double2* in, long long is, double2* out, long long os, int S, const int* stop, int step)>
      apply;
  // the same operator on FP32 vectors in FP32 arithmetic (set on plans with an
  // FP32 operator; used by GMRES with an FP32 Krylov basis)
  std::function<int(const float2* in, long long is, float2* out, long long os, int S, const int* stop, int step)>
      apply32;
};

// pgmres semantics for S systems sharing one operator, device-driven (one
// graph launch per restart cycle when use_graph).  x0 = 0.  active_in (may be
// null) selects the systems to solve (others return x = 0); true_residual
// adds the final ||b - A x|| / ||b|| (pgmres.m:175); tol_s (may be null)
// gives each system its own relative tolerance in place of tol.
// The FP64 side of mixed-precision refinement, on device vectors of S systems
// (stride n), for the systems whose flag is set: X += D, and R = B - A64 X.
struct RefineOps {
  std::function<int(const double2* D, double2* X, const int* flags)> add;
  std::function<int(const double2* X, double2* R, const int* flags)> residual;
};

// Mixed-precision refinement of S systems in ONE graph launch (nested
// conditional WHILE nodes: refinement steps around the restart cycles of the
// inner GMRES): per step, act = relres > tol; the inner FP32-operator GMRES
// (restart m, at most maxit_in cycles, FP64 or FP32 basis) solves A d = r to
// the system's own tolerance min(0.5, max(0.5 tol ||b|| / ||r||, 1e-5)); then
// x += d and r = b - A64 x with FP64 norms; at most max_refine steps.  The
// arithmetic and the results are those of the host-driven refinement; *ran =
// false (nothing done) when the graph cannot be built, e.g. on a driver
// without conditional nodes.  X: S x n solutions (stride n).
int refine_batch_graph(marie_plan* p, const BatchOp& A32, const BatchOp* L1, const BatchOp* R1, const RefineOps& ops,
                       const double2* Bv, long long n, int S, int m, double tol, int maxit_in, int max_refine,
                       bool fp32_basis, double2* X, std::vector<GmresResult>& out, bool* ran);
// The same in parts, so that the refinements of several plans (bodies) run in
// one graph launch: prepare (allocations and the eager start on the plan's
// stream; *ok = false when the graph form does not apply), then
// launch_refine_jobs (each job's loops as independent root nodes of one
// graph, launched once on st and waited for; *ran = false when the graph
// cannot be built), then finish (the results) -- or, when nothing ran, the
// host-driven refinement from scratch.  A job keeps copies of the operators.
class RefineJob {
 public:
  RefineJob();
  ~RefineJob();
  int prepare(marie_plan* p, const BatchOp& A32, const BatchOp* L1, const BatchOp* R1, const RefineOps& ops,
              const double2* Bv, long long n, int S, int m, double tol, int maxit_in, int max_refine, bool fp32_basis,
              double2* X, bool* ok);
  bool add_to(cudaGraph_t g);
  int finish(std::vector<GmresResult>& out);

 private:
  struct Impl;
  std::unique_ptr<Impl> d;
};
int launch_refine_jobs(const std::vector<RefineJob*>& jobs, cudaStream_t st, bool* ran);
// Batched FP64 norms of S vectors (stride xs) into out[S] on the device; with
// mask, only the systems whose mask[s] >= 1 (the others keep out[s]).  part:
// batch_norm_scratch(S) doubles of scratch.
size_t batch_norm_scratch(int S);
int batch_norms_dev(marie_plan* p, const double2* X, long long xs, long long n, int S, const int* mask, double* part,
                    double* out);

int gmres_batch(marie_plan* p, const BatchOp& A, const BatchOp* L1, const BatchOp* R1, const double2* B,
                long long bs, long long n, int S, int restart, double tol, int maxit, double2* X, long long xs,
                std::vector<GmresResult>& out, bool use_graph, const std::vector<int>* active_in,
                bool true_residual, bool fp32_basis = false, const std::vector<double>* tol_s = nullptr);

// MATLAB bicgstab semantics (the solver 'B' of JVIE_Solver.m:451-499) on
// device vectors: iter in half steps, resvec absolute (bicgstab.cu).
struct BicgResult {
  int flag = 1;
  double relres = 0;
  double iter = 0;
  std::vector<double> resvec;
};
int bicgstab(marie_plan* p, const DevOp& A, const DevOp* M1, const DevOp* M2, const double2* b, long long n,
             double tol, int maxit, const double2* x0, double2* x, BicgResult& out);

// pgmresDR semantics (pgmresDR.m, pgmresDR_iter.m: GMRES with deflated
// restarting by ritz harmonic Ritz vectors) on device vectors (gmres_dr.cu).
int gmres_dr(marie_plan* p, const DevOp& A, const DevOp* L1, const DevOp* L2, const DevOp* R1, const DevOp* R2,
             const double2* b, long long n, int restart, double tol, int maxit, int ritz, const double2* x0,
             double2* x, GmresResult& res);

// Gauss-Legendre rule of order n on [-1, 1], ascending nodes (assembly.cu).
void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w);

// DIRECTFN singular integrals {ST, EAc, EAo, VAc, VAo} for cubic voxels of
// edge dx at Np_1D = n (directfn.cu); one triangle-pair call of a DIRECTFN
// core with a MEX gateway's argument order (kind 'S', 'E' or 'V').
constexpr int kDirectfnMaxOrder = 64;
bool directfn_order_ok(int n);
int directfn_integrals(double ko, double dx, int n, double2 out[5], cudaStream_t st);
int directfn_single(char kind, const double* r, double ko, int n, double2* out, cudaStream_t st);

// pgmres semantics (pgmres.m:70-181) on device vectors.
int gmres(marie_plan* p, const DevOp& A, const DevOp* L1, const DevOp* L2, const DevOp* R1, const DevOp* R2,
          const double2* b, long long n, int restart, double tol, int maxit, const double2* x0, double2* x,
          GmresResult& res);

}  // namespace marie
