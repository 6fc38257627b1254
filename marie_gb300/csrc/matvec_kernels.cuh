// The circulant-embedded J-VIE matvec as five FFT passes over the 2L x 2M x 2N
// padded grid, with the gather of the local DOF vector fused into the first
// pass and the crop, diagonal (Gram*Mr, Mc) scaling and DOF scatter fused into
// the last one.  The zero half of the padded input is never loaded, and only the
// N retained z-planes / M retained y-rows are written back after the inverse
// transforms.
//
//   xfwd : rows (y<M, z<N, c)      gather J via inv map, FFT_x (L of 2L non-zero)
//   cols : columns (kx, z<N, c)    FFT_y forward (M of 2M non-zero)
//   zmul : columns (kx, ky)        FFT_z (N of 2N) x3, 3x3 symmetric fN multiply,
//                                  inverse FFT_z, keep z<N        (in place)
//   cols : columns (kx, z<N, c)    inverse FFT_y, keep y<M
//   xinv : rows (y<M, z<N, c)      inverse FFT_x, keep x<L, epilogue, scatter
//
// Spectra layout (column-major like the reference's arrays, kx fastest):
//   A[c][z][y][kx]  : 3 x N x M  x 2L   (after xfwd / before xinv)
//   B[c][z][ky][kx] : 3 x N x 2M x 2L   (after the y transform)
// fN layout: fN[q][kz][ky][kx], q in [xx,xy,xz,yy,yz,zz], pre-scaled by 1/(8LMN)
// so that the inverse transforms need no normalisation.
#pragma once
#include <cuda.h>  // CUtensorMap (the type only; no driver library is linked)

#include "fft.cuh"

namespace marie {

struct Dims {
  int L, M, N, Lp, Mp, Np;
  long long V;  // L*M*N
  // Batched solves: right-hand side r is skipped when stop[r] < step (a
  // system that has left the current GMRES cycle).  stop == nullptr: none.
  const int* stop = nullptr;
  int step = 0;
};

__device__ __forceinline__ bool rhs_skipped(const Dims& d, int rhs) { return d.stop && d.stop[rhs] < d.step; }

// Programmatic dependent launch: a pass launched with the
// programmatic-serialization attribute may start while the previous kernel
// finishes.  It loads only what that kernel cannot have written (the plan's
// operator tile and twiddles), then waits for it to complete (pdl_wait; a
// no-op when launched without the attribute) before reading anything else.
// The skip mask read at the top of the z and y+x passes is written by the
// Givens step at least two kernels earlier.  A pass signals with pdl_trigger,
// in its last phase, that the next one may start.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// A pointer to data that the previous kernel writes, taken again after
// pdl_wait through an opaque move.  A kernel parameter declared
// `const T* __restrict__` tells the compiler that its data is fixed for the
// kernel's lifetime, so it may schedule those loads before the wait or serve
// them from the non-coherent read-only path; under programmatic dependent
// launch the data changes during this kernel's lifetime.  Loads through the
// returned pointer depend on the move (they cannot start before the wait)
// and the pointer carries no __restrict__.
template <typename P> __device__ __forceinline__ P* after_wait(P* p) {
  unsigned long long v = reinterpret_cast<unsigned long long>(p);
  asm volatile("mov.b64 %0, %0;" : "+l"(v)::"memory");
  return reinterpret_cast<P*>(v);
}

// Epilogue: out[k] = A_k * J[k] - (conjout ? conj(v) : B_k * v)
struct Epilogue {
  const double2* a;  // per-DOF, or null -> a_s
  const double2* b;  // per-DOF, or null -> b_s
  double2 a_s, b_s;
  int conjout;
  // FP32 copies of a and b for matvecs on FP32 vectors (IO = float2)
  const float2* af;
  const float2* bf;
};
// Prologue: x_in[k] = (pre ? pre[k] : 1) * (conjin ? conj(J[k]) : J[k])
struct Prologue {
  const double2* pre;
  int conjin;
};

// The matvec's input and output vectors are FP64 (IO = double2) or, for the
// inner solves of mixed-precision refinement, FP32 (IO = float2); the
// epilogue then runs in that precision with the FP32 coefficient copies.
template <typename IO> struct EpiIO;
template <> struct EpiIO<double2> {
  __device__ __forceinline__ static double2 a(const Epilogue& ep, int k) { return ep.a ? ep.a[k] : ep.a_s; }
  __device__ __forceinline__ static double2 b(const Epilogue& ep, int k) { return ep.b ? ep.b[k] : ep.b_s; }
};
template <> struct EpiIO<float2> {
  __device__ __forceinline__ static float2 a(const Epilogue& ep, int k) {
    return ep.af ? ep.af[k] : cvt<float2>(ep.a_s);
  }
  __device__ __forceinline__ static float2 b(const Epilogue& ep, int k) {
    return ep.bf ? ep.bf[k] : cvt<float2>(ep.b_s);
  }
};
// J[k] with the prologue applied, in the precision of IO
template <typename IO>
__device__ __forceinline__ IO prologue_in(const IO* J, const Prologue& pro, int k) {
  IO jv = J[k];
  if (pro.conjin) jv.y = -jv.y;
  if (pro.pre) jv = cmul(cvt<IO>(pro.pre[k]), jv);
  return jv;
}

template <typename V, int N> struct RowCfg {
  static constexpr int T = FFT<V, N, false>::T;
  static constexpr int S = (256 / T) < 2 ? 2 : (256 / T);
  static constexpr int THREADS = S * T;
};

// Stage the twiddle table (N entries) into shared memory.
template <typename V>
__device__ __forceinline__ void stage_twiddles(V* tw_s, const V* __restrict__ tw, int n) {
  for (int i = threadIdx.x; i < n; i += blockDim.x) tw_s[i] = tw[i];
}

// ---------------------------------------------------------------------------
// xfwd: gather + forward x transform.  grid.x = ceil(rows / S), grid.y = rhs
// ---------------------------------------------------------------------------
template <typename T, int NL, typename IO>
__global__ void __launch_bounds__(RowCfg<cplx<T>, NL>::THREADS)
k_xfwd(const IO* __restrict__ J, long long j_stride, const int* __restrict__ inv, Prologue pro,
       cplx<T>* __restrict__ A, long long a_stride, Dims d, const cplx<T>* __restrict__ tw) {
  using V = cplx<T>;
  using F = FFT<V, NL, false>;
  constexpr int S = RowCfg<cplx<T>, NL>::S;
  constexpr int ES = S + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* tw_s = reinterpret_cast<V*>(smem_raw);
  V* buf = tw_s + NL;
  if (rhs_skipped(d, blockIdx.y)) return;
  const int rows = d.M * d.N * 3;
  const int row0 = blockIdx.x * S;
  const IO* Jr = J + blockIdx.y * j_stride;
  stage_twiddles(tw_s, tw, NL);
  // gather: x fastest across threads
  for (int i = threadIdx.x; i < S * d.L; i += blockDim.x) {
    const int s = i / d.L, x = i - s * d.L;
    const int row = row0 + s;
    V val = mk<V>(0, 0);
    if (row < rows) {
      const long long g3 = (long long)row * d.L + x;  // row = y + M*(z + N*c)
      const int k = inv[g3];
      if (k >= 0) val = cvt<V>(prologue_in(Jr, pro, k));
    }
    buf[x * ES + s] = val;
  }
  __syncthreads();
  const int s = threadIdx.x % S, t = threadIdx.x / S;
  V reg[F::E];
  F::load_half(reg, buf + s, ES, t, d.L);
  F::run_half(reg, buf + s, ES, t, tw_s);
  __syncthreads();
  F::store(reg, buf + s, ES, t);
  __syncthreads();
  V* Ar = A + blockIdx.y * a_stride;
  for (int i = threadIdx.x; i < S * NL; i += blockDim.x) {
    const int ss = i / NL, kx = i - ss * NL;
    const int row = row0 + ss;
    if (row < rows) Ar[(long long)row * NL + kx] = buf[kx * ES + ss];
  }
}

// ---------------------------------------------------------------------------
// xinv: inverse x transform + crop + epilogue + scatter to DOFs.
// ---------------------------------------------------------------------------
template <typename T, int NL, typename IO>
__global__ void __launch_bounds__(RowCfg<cplx<T>, NL>::THREADS)
k_xinv(const cplx<T>* __restrict__ A, long long a_stride, const IO* __restrict__ J, long long j_stride,
       const int* __restrict__ inv, Epilogue ep, IO* __restrict__ out, long long o_stride, Dims d,
       const cplx<T>* __restrict__ tw) {
  using V = cplx<T>;
  using F = FFT<V, NL, true>;
  constexpr int S = RowCfg<cplx<T>, NL>::S;
  constexpr int ES = S + 1;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* tw_s = reinterpret_cast<V*>(smem_raw);
  V* buf = tw_s + NL;
  if (rhs_skipped(d, blockIdx.y)) return;
  const int rows = d.M * d.N * 3;
  const int row0 = blockIdx.x * S;
  const V* Ar = A + blockIdx.y * a_stride;
  stage_twiddles(tw_s, tw, NL);
  for (int i = threadIdx.x; i < S * NL; i += blockDim.x) {
    const int s = i / NL, kx = i - s * NL;
    const int row = row0 + s;
    buf[kx * ES + s] = (row < rows) ? Ar[(long long)row * NL + kx] : mk<V>(0, 0);
  }
  __syncthreads();
  const int s = threadIdx.x % S, t = threadIdx.x / S;
  V reg[F::E];
  F::load(reg, buf + s, ES, t, NL);
  F::run(reg, buf + s, ES, t, tw_s);
  __syncthreads();
  F::store(reg, buf + s, ES, t);
  __syncthreads();
  const IO* Jr = J + blockIdx.y * j_stride;
  IO* outr = out + blockIdx.y * o_stride;
  for (int i = threadIdx.x; i < S * d.L; i += blockDim.x) {
    const int ss = i / d.L, x = i - ss * d.L;
    const int row = row0 + ss;
    if (row >= rows) continue;
    const long long g3 = (long long)row * d.L + x;
    const int k = inv[g3];
    if (k < 0) continue;
    const IO v = cvt<IO>(buf[x * ES + ss]);
    const IO jv = Jr[k];
    IO r = cmul(EpiIO<IO>::a(ep, k), jv);
    if (ep.conjout) {
      r.x -= v.x;
      r.y += v.y;
    } else {
      r = csub(r, cmul(EpiIO<IO>::b(ep, k), v));
    }
    outr[k] = r;
  }
}

// ---------------------------------------------------------------------------
// cols: transform along the middle (y) axis for S consecutive kx columns.
//   in [kx + Lp*y + in_w*w], y < n_in      out [kx + Lp*y + out_w*w], y < n_out
// grid.x = Lp / S, grid.y = number of w, grid.z = rhs
// ---------------------------------------------------------------------------
template <typename T> struct ColS { static constexpr int S = 128 / (int)sizeof(cplx<T>); };

// Columns are loaded straight into the first pass's registers and the last
// pass's registers are stored straight to global memory: lanes run over S
// consecutive kx (one 128-byte row segment per warp access), the FFT's
// exchanges go through shared memory only.
template <typename T, int NC, bool INV>
__global__ void __launch_bounds__(ColS<T>::S * FFT<cplx<T>, NC, INV>::T)
k_cols(const cplx<T>* __restrict__ in, long long in_w, long long in_rhs, int n_in,
       cplx<T>* __restrict__ out, long long out_w, long long out_rhs, int n_out, int Lp,
       const cplx<T>* __restrict__ tw, const int* __restrict__ stop, int step) {
  if (stop && stop[blockIdx.z] < step) return;
  using V = cplx<T>;
  using F = FFT<V, NC, INV>;
  constexpr int S = ColS<T>::S;
  constexpr int ES = S + 1;
  constexpr int E = F::E, R0 = F::R0, RL = F::RL;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* tw_s = reinterpret_cast<V*>(smem_raw);
  V* buf = tw_s + NC;
  const int kx0 = blockIdx.x * S;
  const long long w = blockIdx.y;
  const V* inp = in + blockIdx.z * in_rhs + w * in_w + kx0;
  V* outp = out + blockIdx.z * out_rhs + w * out_w + kx0;
  stage_twiddles(tw_s, tw, NC);
  const int s = threadIdx.x % S, t = threadIdx.x / S;
  const bool active = kx0 + s < Lp;
  const bool half = !INV && 2 * n_in <= NC;
  V reg[E];
#pragma unroll
  for (int b = 0; b < E / R0; ++b)
#pragma unroll
    for (int r = 0; r < R0; ++r) {
      const int p = F::in_pos(t, b, r);
      const bool ok = active && p < n_in && (!half || r < R0 / 2);
      reg[b * R0 + r] = ok ? inp[(long long)p * Lp + s] : mk<V>(0, 0);
    }
  __syncthreads();  // twiddles staged
  if constexpr (!INV && R0 % 2 == 0) {
    if (half)
      F::run_half(reg, buf + s, ES, t, tw_s);
    else
      F::run(reg, buf + s, ES, t, tw_s);
  } else {
    F::run(reg, buf + s, ES, t, tw_s);
  }
#pragma unroll
  for (int b = 0; b < E / RL; ++b)
#pragma unroll
    for (int r = 0; r < RL; ++r) {
      const int y = F::out_pos(t, b, r);
      if (active && y < n_out) outp[(long long)y * Lp + s] = reg[b * RL + r];
    }
}

// ---------------------------------------------------------------------------
// zmul: per (kx, ky) column: forward z transform of the three components,
// symmetric 3x3 multiply by fN, inverse z transform, keep z < N.  In place.
// B[c][z][ky][kx].  grid.x = Lp / S, grid.y = Mp, grid.z = rhs
//
// Operator storage (oct = 1): the circulant's per-axis parities make
// fN(2L-kx, ky, kz) = +-fN(kx, ky, kz) (sign = parity of the component along the
// reflected axis), so only the octant k <= (L, M, N) is kept:
// fNo[q][oz][oy][ox], (L+1) x (M+1) x (N+1) per component.  oct = 0: full
// fN[q][kz][ky][kx].
// ---------------------------------------------------------------------------
// The two circulant operators of the path: N, the symmetric 3x3 tensor of
// mv_AN / mv_L (6 components [xx xy xz yy yz zz], kind 0), and K, the
// curl-type kernel of mv_K (3 components [Kx Ky Kz], kind 1).  odd(q, a): the
// circulant component q is odd along axis a (gperiodic_coeff_nop.m,
// gperiodic_coeff_kop.m), so its transform changes sign under reflection.
template <int KIND> struct OpKind;
template <> struct OpKind<0> {
  static constexpr int NQ = 6;
  __host__ __device__ static constexpr bool odd(int q, int a) {
    return a == 0 ? (q == 1 || q == 2) : (a == 1 ? (q == 1 || q == 4) : (q == 2 || q == 4));
  }
};
template <> struct OpKind<1> {
  static constexpr int NQ = 3;
  __host__ __device__ static constexpr bool odd(int q, int a) { return q == a; }
};

// z-pass variants the autotuner chooses from (FP32, N operator): 0 the
// default (wide radix schedule where one exists, 8 columns per CTA), 1 the
// narrow radix schedule, 2 half the columns per CTA.
template <typename T, int NZ, int VAR> struct ZVar {
  static constexpr bool W = VAR == 1 ? false : (sizeof(cplx<T>) == 8 && HasWide<NZ>::value);
  static constexpr int S0 = (sizeof(T) == 4 ? 8 : 4) / (VAR == 2 ? 2 : 1);
};

template <typename T, int NZ, int KIND = 0, int VAR = 0> struct ZS {
  static constexpr bool W = ZVar<T, NZ, VAR>::W;             // radix schedule
  static constexpr int TT = FFT<cplx<T>, NZ, false, W>::T;   // threads per transform
  static constexpr int S0 = ZVar<T, NZ, VAR>::S0;            // columns per CTA
  static constexpr int S = (3 * S0 * TT <= 1024) ? S0 : ((3 * (S0 / 2) * TT <= 1024) ? S0 / 2 : S0 / 4);
  static constexpr int THREADS = 3 * S * TT;               // one thread group per component
  // rows of 64 B use the half-line swizzle, others one pad element per row
  static constexpr bool HALF = S * (int)sizeof(cplx<T>) == 64;
  static constexpr int ES = HALF ? S : S + 1;
  static constexpr int BUF = NZ * ES + (HALF ? (NZ / 16 + 1) * S : 0);  // one component's exchange buffer
  // octant operator tile of the CTA's columns: NQ components x (N+1) planes x S
  static constexpr int TILE = OpKind<KIND>::NQ * (NZ / 2 + 1) * S;
  // + 128 bytes so that the tile can start on a 128-byte boundary (bulk tensor copies)
  static constexpr long long bytes(int) { return (long long)(NZ + 3 * BUF + TILE) * sizeof(cplx<T>) + 128; }
  // The tile arrives by one bulk tensor copy (cp.async.bulk.tensor) from the
  // FP32 N operator stored full along x: needs FP32 values, the N operator, an
  // even column count (the box starts on a 16-byte boundary) and at most 256
  // octant planes (the box limit).
  static constexpr bool TMA = sizeof(T) == 4 && KIND == 0 && S % 2 == 0 && NZ / 2 + 1 <= 256;
  __device__ static SAddr addr() { return SAddr(ES, false, HALF ? S : 0); }
};

// asynchronous global -> shared copy of one complex value (no register staging)
template <typename V> __device__ __forceinline__ void cp_async_val(V* dst, const V* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  if constexpr (sizeof(V) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src));
  else
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src));
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\n" ::);
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// N components odd along z: xz (2), yz (4)
__host__ __device__ constexpr bool odd_z(int q) { return OpKind<0>::odd(q, 2); }

// Components of row c of the symmetric tensor [xx xy xz; xy yy yz; xz yz zz].
template <int C> struct ZRow {
  static constexpr int q0 = C == 0 ? 0 : (C == 1 ? 1 : 2);
  static constexpr int q1 = C == 0 ? 1 : (C == 1 ? 3 : 4);
  static constexpr int q2 = C == 0 ? 2 : (C == 1 ? 4 : 5);
};

template <typename V> __device__ __forceinline__ V neg_if(V v, bool f) { return f ? mk<V>(-v.x, -v.y) : v; }

// Row C of the product at this thread's output positions of the forward
// transform.  With the octant operator the tile already carries the x and y
// reflection signs; the z reflection (positions kz > NZ/2) flips the two
// z-odd components.  Without it the full operator is read from global memory.
template <int C, typename FF, typename V, int NZ, int S>
__device__ __forceinline__ void zrow(V* reg, int t, int s, bool active, int oct, const V* tile, const V* fp,
                                     long long fq, long long fplane, const V* b0, const V* b1, const V* b2,
                                     SAddr ad) {
  using RW = ZRow<C>;
  constexpr int NH = NZ / 2, NO = NH + 1, RL = FF::RL;
#pragma unroll
  for (int b = 0; b < FF::E / RL; ++b)
#pragma unroll
    for (int r = 0; r < RL; ++r) {
      const int kz = FF::out_pos(t, b, r);
      V y = mk<V>(0, 0);
      if (active) {
        V n0, n1, n2;
        if (oct) {
          const bool fz = kz > NH;
          const int oz = fz ? NZ - kz : kz;
          n0 = tile[(RW::q0 * NO + oz) * S + s];
          n1 = tile[(RW::q1 * NO + oz) * S + s];
          n2 = tile[(RW::q2 * NO + oz) * S + s];
          if constexpr (odd_z(RW::q0)) n0 = neg_if(n0, fz);
          if constexpr (odd_z(RW::q1)) n1 = neg_if(n1, fz);
          if constexpr (odd_z(RW::q2)) n2 = neg_if(n2, fz);
        } else {
          const long long o = (long long)kz * fplane;
          n0 = fp[RW::q0 * fq + o];
          n1 = fp[RW::q1 * fq + o];
          n2 = fp[RW::q2 * fq + o];
        }
        const int e = ad(kz);
        y = cadd(cadd(cmul(n0, b0[e]), cmul(n1, b1[e])), cmul(n2, b2[e]));
      }
      reg[b * RL + r] = y;
    }
}

// Row C of the K product out = K x J at this thread's output positions:
// out_x = Kz J_y - Ky J_z, out_y = Kx J_z - Kz J_x, out_z = Ky J_x - Kx J_y
// (mv_K.m:57-74).  Kz is odd along z, so the z reflection flips it.
template <int C> struct KRow {
  static constexpr int qa = C == 0 ? 2 : (C == 1 ? 0 : 1), ia = C == 0 ? 1 : (C == 1 ? 2 : 0);
  static constexpr int qb = C == 0 ? 1 : (C == 1 ? 2 : 0), ib = C == 0 ? 2 : (C == 1 ? 0 : 1);
};

template <int C, typename FF, typename V, int NZ, int S>
__device__ __forceinline__ void zrow_k(V* reg, int t, int s, bool active, int oct, const V* tile, const V* fp,
                                       long long fq, long long fplane, const V* const* bc, SAddr ad) {
  using RW = KRow<C>;
  constexpr int NH = NZ / 2, NO = NH + 1, RL = FF::RL;
#pragma unroll
  for (int b = 0; b < FF::E / RL; ++b)
#pragma unroll
    for (int r = 0; r < RL; ++r) {
      const int kz = FF::out_pos(t, b, r);
      V y = mk<V>(0, 0);
      if (active) {
        V na, nb;
        if (oct) {
          const bool fz = kz > NH;
          const int oz = fz ? NZ - kz : kz;
          na = tile[(RW::qa * NO + oz) * S + s];
          nb = tile[(RW::qb * NO + oz) * S + s];
          if constexpr (RW::qa == 2) na = neg_if(na, fz);
          if constexpr (RW::qb == 2) nb = neg_if(nb, fz);
        } else {
          const long long o = (long long)kz * fplane;
          na = fp[RW::qa * fq + o];
          nb = fp[RW::qb * fq + o];
        }
        const int e = ad(kz);
        y = csub(cmul(na, bc[RW::ia][e]), cmul(nb, bc[RW::ib][e]));
      }
      reg[b * RL + r] = y;
    }
}

// Thread group c (of three) transforms component c of the S columns.  After
// the forward transforms the three spectra meet in shared memory; group c
// forms row c of the symmetric product and runs its inverse transform from
// the registers (the inverse radix order starts where the forward ended).
//
// Operator tile (octant operators, oct = 1): with tma = 1 (FP32 N operator)
// one thread issues a single bulk tensor copy of the S columns x (N+1) planes
// x 6 components from the copy of the operator stored full along x (x
// reflections already carry their signs there) and every thread waits on the
// copy's mbarrier, with a time limit after which err is set and the pass goes
// on (tma = 2: a test of that path, the barrier armed for more bytes than the
// copy delivers); the y reflection is applied as N -> D N D with D = diag(1, -1, 1) on the
// y component's spectrum and product row (the symmetric tensor's xy and yz
// entries are the odd ones in y), the z reflection by the sign of the z-odd
// entries per position.  Otherwise every thread copies its share of the tile
// from the octant with cp.async and signs the x and y reflections in place.
template <typename T, int NZ, int KIND, int VAR>
__global__ void __launch_bounds__(ZS<T, NZ, KIND, VAR>::THREADS)
k_zmul(cplx<T>* __restrict__ B, long long b_rhs, const cplx<T>* __restrict__ fN, int oct, Dims d,
       const cplx<T>* __restrict__ tw, const __grid_constant__ CUtensorMap tmap, int tma, int* err) {
  if (rhs_skipped(d, blockIdx.z)) return;
  using V = cplx<T>;
  using ZC = ZS<T, NZ, KIND, VAR>;
  using FF = FFT<V, NZ, false, ZC::W>;
  using FI = FFT<V, NZ, true, ZC::W>;
  using OK = OpKind<KIND>;
  constexpr int S = ZC::S;
  constexpr int BUF = ZC::BUF;
  constexpr int NH = NZ / 2, NO = NH + 1;  // N non-zero planes; N+1 octant planes
  const SAddr ad = ZC::addr();
  constexpr int E = FF::E, R0 = FF::R0, RLI = FI::RL;
  static_assert(FI::R0 == FF::RL, "inverse must start where the forward transform ended");
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* tw_s = reinterpret_cast<V*>(smem_raw);
  V* buf = tw_s + NZ;  // 3 exchange buffers of BUF elements
  const int kx0 = blockIdx.x * S;
  // grid rows in the order 0, M, 1, 2M-1, 2, 2M-2, ...: the two rows that
  // read the same operator tile (ky and its y reflection 2M - ky) run one
  // grid row apart, so the second copy finds the tile in L2
  const int gy = blockIdx.y;
  const int ky = gy == 0 ? 0 : gy == 1 ? d.M : (gy & 1) ? d.Mp - (gy >> 1) : (gy >> 1);
  const long long plane = (long long)d.Lp * d.Mp;  // one z-plane of B
  const long long comp = plane * NH;                // one component of B
  const int c = threadIdx.x / (S * FF::T);
  const int rem = threadIdx.x - c * S * FF::T;
  const int s = rem % S, t = rem / S;
  V* Bp = B + blockIdx.z * b_rhs + c * comp + (long long)ky * d.Lp + kx0;
  V* tile = buf + 3 * BUF;  // operator tile of the CTA's columns, [q][oz][s], 128-byte aligned
  tile = reinterpret_cast<V*>(reinterpret_cast<char*>(tile) +
                              ((128u - ((unsigned)__cvta_generic_to_shared(tile) & 127u)) & 127u));
  const bool active = kx0 + s < d.Lp;
  const bool fy = oct && ky > d.M;
  const int oy = fy ? d.Mp - ky : ky;
  const long long fq = oct ? (long long)(d.L + 1) * (d.M + 1) * NO : (long long)d.Lp * d.Mp * d.Np;
  const long long fplane = oct ? (long long)(d.L + 1) * (d.M + 1) : plane;
  const long long frow = oct ? (long long)(d.L + 1) : d.Lp;
  // Tile rows (q, oz) of S columns: this thread copies column s of rows
  // row0, row0 + STEP, ... (THREADS is a multiple of S).
  constexpr int ROWS = OK::NQ * NO, STEP = ZC::THREADS / S;
  const int row0 = threadIdx.x / S;
  const bool bulk = ZC::TMA && tma && oct;
  __shared__ __align__(8) unsigned long long tile_bar;
  const unsigned bar = (unsigned)__cvta_generic_to_shared(&tile_bar);
  if (bulk) {
    if (threadIdx.x == 0) {
      // box origin (kx0, oy, 0, 0): kx0 is a multiple of the even S, so the
      // copy starts on a 16-byte boundary; the box (S x 1 x NO x 6) lies
      // inside the (Lp, M+1, N+1, 6) tensor
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar));
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      // tma == 2 (a test of the bounded wait): armed for 16 bytes more than
      // the copy delivers, so the barrier never completes
      const unsigned bytes = (unsigned)(OK::NQ * NO * S * sizeof(V)) + (tma == 2 ? 16u : 0u);
      asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
      asm volatile(
          "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
          "%5}], [%6];" ::"r"((unsigned)__cvta_generic_to_shared(tile)),
          "l"(reinterpret_cast<unsigned long long>(&tmap)), "r"(kx0), "r"(oy), "r"(0), "r"(0), "r"(bar)
          : "memory");
    }
  } else if (oct && active) {
    // the operator tile streams into shared memory while the forward
    // transforms run (its latency was the z pass's main stall)
    const int kx = kx0 + s;
    const int ox = kx > d.L ? d.Lp - kx : kx;
    int q = row0 / NO, oz = row0 - q * NO;
    const V* src = fN + q * fq + (long long)oz * fplane + (long long)oy * frow + ox;
    for (int row = row0; row < ROWS; row += STEP) {
      cp_async_val(tile + row * S + s, src);
      oz += STEP;
      src += STEP * fplane;
      while (oz >= NO) {
        oz -= NO;
        src += fq - NO * fplane;
      }
    }
  }
  stage_twiddles(tw_s, tw, NZ);
  pdl_wait();  // the spectrum B is the previous pass's output
  Bp = after_wait(Bp);
  V reg[E];
#pragma unroll
  for (int b = 0; b < E / R0; ++b)
#pragma unroll
    for (int r = 0; r < R0; ++r) {
      const int p = FF::in_pos(t, b, r);
      reg[b * R0 + r] = (active && r < R0 / 2 && p < NH) ? __ldcg(Bp + p * plane + s) : mk<V>(0, 0);
    }
  __syncthreads();  // twiddles staged
  V* my = buf + c * BUF + s;
  FF::run_half(reg, my, ad, t, tw_s);
  // D N D with D = diag(1, -1, 1) for a y-reflected column (bulk tile only)
  const bool neg_y = bulk && c == 1 && fy;
  if (neg_y) {
#pragma unroll
    for (int i = 0; i < E; ++i) reg[i] = mk<V>(-reg[i].x, -reg[i].y);
  }
  __syncthreads();
  FF::store(reg, my, ad, t);
  if (bulk) {
    // wait for the tile, at most ~2 s of global time (5 ms in the test of
    // this path); then flag it and go on (the values are wrong, the status
    // word tells the host)
    const unsigned long long limit = tma == 2 ? 5000000ull : 2000000000ull;
    unsigned long long t_start;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_start));
    for (;;) {
      unsigned done;
      asm volatile(
          "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\t"
          "selp.u32 %0, 1, 0, p;\n\t}"
          : "=r"(done)
          : "r"(bar)
          : "memory");
      if (done) break;
      unsigned long long t_now;
      asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t_now));
      if (t_now - t_start > limit) {
        if (err) atomicExch(err, 1);
        break;
      }
    }
  } else if (oct && active) {
    // each thread signs the tile entries it copied: reflections in x and y
    // flip the components odd along that axis
    cp_async_wait_all();
    const bool fx = kx0 + s > d.L;
    unsigned flip = 0;
#pragma unroll
    for (int q = 0; q < OK::NQ; ++q)
      if ((fx && OK::odd(q, 0)) != (fy && OK::odd(q, 1))) flip |= 1u << q;
    if (flip) {
      int q = row0 / NO, oz = row0 - q * NO;
      for (int row = row0; row < ROWS; row += STEP) {
        if ((flip >> q) & 1u) {
          V* e = tile + row * S + s;
          *e = mk<V>(-e->x, -e->y);
        }
        oz += STEP;
        while (oz >= NO) {
          oz -= NO;
          ++q;
        }
      }
    }
  }
  __syncthreads();

  const V* fp = fN + (long long)oy * frow + (kx0 + s);
  const V* b0 = buf + s;
  const V* b1 = buf + BUF + s;
  const V* b2 = buf + 2 * BUF + s;
  // c is uniform over whole warps (groups of S * T threads) for the long transforms
  if constexpr (KIND == 0) {
    if (c == 0)
      zrow<0, FF, V, NZ, S>(reg, t, s, active, oct, tile, fp, fq, fplane, b0, b1, b2, ad);
    else if (c == 1)
      zrow<1, FF, V, NZ, S>(reg, t, s, active, oct, tile, fp, fq, fplane, b0, b1, b2, ad);
    else
      zrow<2, FF, V, NZ, S>(reg, t, s, active, oct, tile, fp, fq, fplane, b0, b1, b2, ad);
  } else {
    const V* bc[3] = {b0, b1, b2};
    if (c == 0)
      zrow_k<0, FF, V, NZ, S>(reg, t, s, active, oct, tile, fp, fq, fplane, bc, ad);
    else if (c == 1)
      zrow_k<1, FF, V, NZ, S>(reg, t, s, active, oct, tile, fp, fq, fplane, bc, ad);
    else
      zrow_k<2, FF, V, NZ, S>(reg, t, s, active, oct, tile, fp, fq, fplane, bc, ad);
  }
  if (neg_y) {
#pragma unroll
    for (int i = 0; i < E; ++i) reg[i] = mk<V>(-reg[i].x, -reg[i].y);
  }
  pdl_trigger();
  FI::run(reg, my, ad, t, tw_s);
#pragma unroll
  for (int b = 0; b < E / RLI; ++b)
#pragma unroll
    for (int r = 0; r < RLI; ++r) {
      const int z = FI::out_pos(t, b, r);
      if (active && z < NH) Bp[z * plane + s] = reg[b * RLI + r];
    }
}

}  // namespace marie
