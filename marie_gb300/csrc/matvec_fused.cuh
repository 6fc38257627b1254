// Fused x+y passes of the matvec, one (z, component) plane per thread-block
// cluster, exchanging the x-transformed rows through distributed shared memory
// instead of a round trip of the A spectrum through HBM.
//
//   k_xyfwd:  gather J (inv map) -> FFT_x of the M non-zero rows (CTA q of the
//             cluster owns rows [q*M/CS, (q+1)*M/CS)) -> each output (kx, y) is
//             stored into the shared memory of the CTA that owns column kx ->
//             cluster barrier -> FFT_y of the owned 2L/CS columns -> B.
//   k_yxinv:  B -> inverse FFT_y of the owned columns, keep y < M -> rows sent
//             to their owners -> cluster barrier -> inverse FFT_x of the owned
//             rows, keep x < L -> Gram*Mr*J - Mc*(N J) epilogue -> scatter.
//
// Both kernels write/read the spectrum B[c][z][ky][kx] of the z pass, so the
// matvec is xyfwd -> zmul -> yxinv: 48V complex of spectrum traffic per RHS.
#pragma once
#include <cooperative_groups.h>

#include "matvec_kernels.cuh"

namespace marie {

namespace cg = cooperative_groups;

// Split cluster barrier: a CTA may store into another CTA's shared memory only
// once that CTA is running.  Arriving right after the kernel's set-up and
// waiting just before the first remote store lets the first gathers and
// transforms overlap the barrier (every thread arrives once, then waits once).
__device__ __forceinline__ void cluster_arrive_relaxed() {
  asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_arrive() { asm volatile("barrier.cluster.arrive.aligned;" ::: "memory"); }
__device__ __forceinline__ void cluster_wait() { asm volatile("barrier.cluster.wait.aligned;" ::: "memory"); }

// NARROW: the radix-8 schedules for the x and y transforms (twice the threads
// per transform, half the exchange buffer, one more CTA per SM for xyfwd); an
// autotuner variant for the lengths that have a wide schedule.
template <typename T, int NL, int NM, int CS, bool NARROW = false> struct XYCfg {
  using V = cplx<T>;
  static constexpr bool WX = !NARROW && (sizeof(V) == 8) && HasWide<NL>::value;
  static constexpr bool WY = !NARROW && (sizeof(V) == 8) && HasWide<NM>::value;
  using FX = FFT<V, NL, false, WX>;
  using FXI = FFT<V, NL, true, WX>;
  using FY = FFT<V, NM, false, WY>;
  using FYI = FFT<V, NM, true, WY>;
  static constexpr int THREADS = 256;
  static constexpr int L = NL / 2, M = NM / 2;
  static constexpr int RY = M / CS;                 // rows per CTA
  static constexpr int CW = NL / CS;                // columns per CTA
  static constexpr int SX = THREADS / FX::T;        // rows per x sweep
  static constexpr int SY = THREADS / FY::T;        // columns per y sweep
  static constexpr int ROWP = NL + NL / 16;         // swizzled row pitch
  static constexpr int RS = CW + 1;                 // pitch of the column receive buffer
  static constexpr int RYP = ((RY + SX - 1) / SX) * SX;
  static constexpr int XB = (SX * ROWP > NM * (SY + 1)) ? SX * ROWP : NM * (SY + 1);
  static constexpr size_t fwd_smem = (size_t)(NL + NM + M * RS + XB) * sizeof(V);
  static constexpr size_t inv_smem = (size_t)(NL + NM + RYP * ROWP + NM * (SY + 1)) * sizeof(V);
  static constexpr bool ok = (M % CS == 0) && (NL % CS == 0) && RY >= 1 && FX::T <= THREADS &&
                             FY::T <= THREADS;
};

template <typename T, int NL, int NM, int CS, bool NARROW, typename IO>
__global__ void __launch_bounds__(256, NARROW ? 4 : 0)
k_xyfwd(const IO* __restrict__ J, long long js, const int* __restrict__ inv, Prologue pro,
        cplx<T>* __restrict__ B, long long bs, Dims d, const cplx<T>* __restrict__ twx,
        const cplx<T>* __restrict__ twy) {
  using C = XYCfg<T, NL, NM, CS, NARROW>;
  using V = cplx<T>;
  using FX = typename C::FX;
  using FY = typename C::FY;
  constexpr int L = C::L, M = C::M;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* twx_s = reinterpret_cast<V*>(smem_raw);
  V* twy_s = twx_s + NL;
  V* recv = twy_s + NM;    // [y][col], M x RS
  V* xb = recv + M * C::RS;  // exchange buffer
  cg::cluster_group cluster = cg::this_cluster();
  const int q = (int)cluster.block_rank();
  const int plane = blockIdx.x / CS;  // z + N*c
  constexpr int EX = FX::E, R0X = FX::R0;
  const int tx = threadIdx.x % FX::T, sx = threadIdx.x / FX::T;
  // the twiddles are staged before the wait for the previous pass; the index
  // map, the skip mask, the prologue factors and J are read after it (the
  // kernel just before may have written any of them)
  for (int i = threadIdx.x; i < NL; i += blockDim.x) twx_s[i] = twx[i];
  pdl_wait();
  if (rhs_skipped(d, blockIdx.y)) return;  // uniform over the cluster, before any cluster barrier
  const int* invw = after_wait(inv);
  const IO* Jr = after_wait(J) + blockIdx.y * js;
  Prologue prw = pro;
  prw.pre = after_wait(pro.pre);
  // DOF indices of one sweep of rows (the zero half of each row is skipped)
  auto load_idx = [&](int* kk, int row0) {
    const int yl = row0 + sx;
    const bool valid = yl < C::RY;
    const int* invr = invw + (long long)L * (q * C::RY + yl + (long long)M * plane);
#pragma unroll
    for (int b = 0; b < EX / R0X; ++b)
#pragma unroll
      for (int r = 0; r < R0X; ++r) {
        const int p = FX::in_pos(tx, b, r);
        kk[b * R0X + r] = (valid && r < R0X / 2 && p < L) ? invr[p] : -1;
      }
  };
  int kk[EX];
  load_idx(kk, 0);
  __syncthreads();  // x twiddles staged
  cluster_arrive_relaxed();

  // ---- x transforms of the owned rows, results to the owners of their columns
  {
    constexpr int E = FX::E, RL = FX::RL;
    const int t = tx, s = sx;
    for (int row0 = 0; row0 < C::RY; row0 += C::SX) {
      const int yl = row0 + s;
      const bool valid = yl < C::RY;
      const int y = q * C::RY + yl;
      V reg[E];
      if (row0 > 0) load_idx(kk, row0);
#pragma unroll
      for (int i = 0; i < E; ++i) reg[i] = kk[i] >= 0 ? cvt<V>(prologue_in(Jr, prw, kk[i])) : mk<V>(0, 0);
      FX::run_half(reg, xb + s * C::ROWP, SAddr(1, true), t, twx_s);
      if (row0 == 0) cluster_wait();  // every CTA of the cluster runs before remote stores
      if (valid) {
#pragma unroll
        for (int b = 0; b < E / RL; ++b)
#pragma unroll
          for (int r = 0; r < RL; ++r) {
            const int kx = FX::out_pos(t, b, r);
            V* dst = cluster.map_shared_rank(recv, kx / C::CW);
            dst[y * C::RS + (kx % C::CW)] = reg[b * RL + r];
          }
      }
    }
  }
  // all rows delivered: arrive (release), stage the y twiddles while the
  // cluster meets, wait (acquire)
  cluster_arrive();
  for (int i = threadIdx.x; i < NM; i += blockDim.x) twy_s[i] = twy[i];
  cluster_wait();
  __syncthreads();  // y twiddles staged (written after this thread's arrive)

  pdl_trigger();

  // ---- y transforms of the owned columns, straight to B
  {
    constexpr int E = FY::E, R0 = FY::R0, RL = FY::RL;
    const int s = threadIdx.x % C::SY, t = threadIdx.x / C::SY;
    V* Bp = B + blockIdx.y * bs + (long long)plane * NM * NL + q * C::CW;
    for (int c0 = 0; c0 < C::CW; c0 += C::SY) {
      const int col = c0 + s;
      const bool valid = col < C::CW;
      V reg[E];
#pragma unroll
      for (int b = 0; b < E / R0; ++b)
#pragma unroll
        for (int r = 0; r < R0; ++r) {
          const int p = FY::in_pos(t, b, r);
          reg[b * R0 + r] = (valid && r < R0 / 2 && p < M) ? recv[p * C::RS + col] : mk<V>(0, 0);
        }
      FY::run_half(reg, xb + s, SAddr(C::SY + 1), t, twy_s);
      if (valid) {
#pragma unroll
        for (int b = 0; b < E / RL; ++b)
#pragma unroll
          for (int r = 0; r < RL; ++r) {
            const int ky = FY::out_pos(t, b, r);
            Bp[(long long)ky * NL + col] = reg[b * RL + r];
          }
      }
    }
  }
}

template <typename T, int NL, int NM, int CS, bool NARROW, typename IO>
__global__ void __launch_bounds__(256, (XYCfg<T, NL, NM, CS, NARROW>::FXI::E <= 16 &&
                                        XYCfg<T, NL, NM, CS, NARROW>::FYI::E <= 16) ? 3 : 1)
k_yxinv(const cplx<T>* __restrict__ B, long long bs, const IO* __restrict__ J, long long js,
        const int* __restrict__ inv, Epilogue ep, IO* __restrict__ out, long long os, Dims d,
        const cplx<T>* __restrict__ twx, const cplx<T>* __restrict__ twy) {
  if (rhs_skipped(d, blockIdx.y)) return;  // uniform over the cluster
  using C = XYCfg<T, NL, NM, CS, NARROW>;
  using V = cplx<T>;
  using FXI = typename C::FXI;
  using FYI = typename C::FYI;
  constexpr int L = C::L, M = C::M;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  V* twx_s = reinterpret_cast<V*>(smem_raw);
  V* twy_s = twx_s + NL;
  V* rows = twy_s + NM;             // [yl][swizzled kx], RYP x ROWP
  V* xb = rows + C::RYP * C::ROWP;  // column exchange buffer
  cg::cluster_group cluster = cg::this_cluster();
  const int q = (int)cluster.block_rank();
  const int plane = blockIdx.x / CS;
  const SAddr rowa(1, true);

  // ---- inverse y transforms of the owned columns, kept rows to their owners
  {
    constexpr int E = FYI::E, R0 = FYI::R0, RL = FYI::RL;
    const int s = threadIdx.x % C::SY, t = threadIdx.x / C::SY;
    // twiddles staged before the wait for the spectrum of the previous pass;
    // the spectrum is read after it, through L2 (the z pass writes it while
    // this kernel's first CTAs are already resident)
    for (int i = threadIdx.x; i < NL; i += blockDim.x) twx_s[i] = twx[i];
    for (int i = threadIdx.x; i < NM; i += blockDim.x) twy_s[i] = twy[i];
    pdl_wait();
    const V* Bp = after_wait(B) + blockIdx.y * bs + (long long)plane * NM * NL + q * C::CW;
    auto load_cols = [&](V* reg, int c0) {
      const int col = c0 + s;
      const bool valid = col < C::CW;
#pragma unroll
      for (int b = 0; b < E / R0; ++b)
#pragma unroll
        for (int r = 0; r < R0; ++r)
          reg[b * R0 + r] = valid ? __ldcg(Bp + (long long)FYI::in_pos(t, b, r) * NL + col) : mk<V>(0, 0);
    };
    V reg[E];
    load_cols(reg, 0);
    __syncthreads();  // twiddles staged
    cluster_arrive_relaxed();
    for (int c0 = 0; c0 < C::CW; c0 += C::SY) {
      const int col = c0 + s;
      const bool valid = col < C::CW;
      const int kx = q * C::CW + col;
      if (c0 > 0) load_cols(reg, c0);
      FYI::run(reg, xb + s, SAddr(C::SY + 1), t, twy_s);
      if (c0 == 0) cluster_wait();  // every CTA of the cluster runs before remote stores
#pragma unroll
      for (int b = 0; b < E / RL; ++b)
#pragma unroll
        for (int r = 0; r < RL; ++r) {
          const int y = FYI::out_pos(t, b, r);
          if (valid && y < M) {
            V* dst = cluster.map_shared_rank(rows, y / C::RY);
            dst[(y % C::RY) * C::ROWP + rowa(kx)] = reg[b * RL + r];
          }
        }
    }
  }

  // ---- inverse x transforms of the owned rows, epilogue, scatter
  {
    constexpr int E = FXI::E, RL = FXI::RL;
    const int t = threadIdx.x % FXI::T, s = threadIdx.x / FXI::T;
    const IO* Jr = J + blockIdx.y * js;
    IO* outr = out + blockIdx.y * os;
    // DOF indices of the epilogue of one sweep of rows
    auto load_epi_idx = [&](int* kk, int row0) {
      const int yl = row0 + s;
      const int* invr = inv + (long long)L * (q * C::RY + yl + (long long)M * plane);
#pragma unroll
      for (int b = 0; b < E / RL; ++b)
#pragma unroll
        for (int r = 0; r < RL; ++r) {
          const int x = FXI::out_pos(t, b, r);
          kk[b * RL + r] = (yl < C::RY && x < L) ? invr[x] : -1;
        }
    };
    // rows delivered: arrive (release) now and wait (acquire) once the first
    // sweep's epilogue indices are in flight
    cluster_arrive();
    int kk[E <= 16 ? E : 1];
    if constexpr (E <= 16) load_epi_idx(kk, 0);
    cluster_wait();
    for (int row0 = 0; row0 < C::RYP; row0 += C::SX) {
      const int yl = row0 + s;
      const bool valid = yl < C::RY;
      const int y = q * C::RY + yl;
      V* base = rows + yl * C::ROWP;
      V reg[E];
      FXI::load(reg, base, rowa, t, NL);
      FXI::run(reg, base, rowa, t, twx_s);
      if constexpr (E <= 16)
        if (row0 > 0) load_epi_idx(kk, row0);
      if (valid) {
        const int* invr = inv + (long long)L * (y + (long long)M * plane);
        if constexpr (E <= 16) {
          // index loads (above), then the per-DOF loads, then the epilogue arithmetic
          // per-DOF loads in groups of EPI (bounded registers)
          constexpr int EPI = 2;
          // FP64 vectors with FP32 coefficient copies (the matvec of the
          // mixed-precision inner solves): the whole epilogue in FP32, the
          // transforms' precision, with one conversion in and one out
          constexpr bool MIX = std::is_same<IO, double2>::value && std::is_same<V, float2>::value;
          const bool f32epi = MIX && ep.af != nullptr;
#pragma unroll
          for (int i0 = 0; i0 < E; i0 += EPI) {
            IO jv[EPI], ak[EPI], bk[EPI];
            float2 af[EPI], bf[EPI];
#pragma unroll
            for (int j = 0; j < EPI; ++j) {
              const int k = kk[i0 + j];
              if (k < 0) continue;
              jv[j] = Jr[k];
              if (f32epi) {
                af[j] = ep.af[k];
                bf[j] = ep.bf[k];
              } else {
                ak[j] = EpiIO<IO>::a(ep, k);
                bk[j] = EpiIO<IO>::b(ep, k);
              }
            }
#pragma unroll
            for (int j = 0; j < EPI; ++j) {
              const int k = kk[i0 + j];
              if (k < 0) continue;
              if constexpr (MIX) {
                if (f32epi) {
                  const float2 v = reg[i0 + j];
                  float2 r32 = cmul(af[j], cvt<float2>(jv[j]));
                  if (ep.conjout) {
                    r32.x -= v.x;
                    r32.y += v.y;
                  } else {
                    r32 = csub(r32, cmul(bf[j], v));
                  }
                  outr[k] = cvt<IO>(r32);
                  continue;
                }
              }
              // the diagonal Gram*Mr*J term in the vectors' precision; the
              // circulant term in the transform's precision
              IO res = cmul(ak[j], jv[j]);
              if (ep.conjout) {
                const IO v = cvt<IO>(reg[i0 + j]);
                res.x -= v.x;
                res.y += v.y;
              } else {
                res = csub(res, cvt<IO>(cmul(cvt<V>(bk[j]), reg[i0 + j])));
              }
              outr[k] = res;
            }
          }
        } else {
          // wide register sets (E = 20, 24): one DOF at a time
#pragma unroll
          for (int b = 0; b < E / RL; ++b)
#pragma unroll
            for (int r = 0; r < RL; ++r) {
              const int x = FXI::out_pos(t, b, r);
              if (x >= L) continue;
              const int k = invr[x];
              if (k < 0) continue;
              const IO jv = Jr[k];
              IO res = cmul(EpiIO<IO>::a(ep, k), jv);
              if (ep.conjout) {
                const IO v = cvt<IO>(reg[b * RL + r]);
                res.x -= v.x;
                res.y += v.y;
              } else {
                res = csub(res, cvt<IO>(cmul(cvt<V>(EpiIO<IO>::b(ep, k)), reg[b * RL + r])));
              }
              outr[k] = res;
            }
        }
      }
    }
  }
}

}  // namespace marie
