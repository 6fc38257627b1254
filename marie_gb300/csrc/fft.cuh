// Register-resident mixed-radix Stockham FFT for sequences staged in shared memory.
//
// A sequence of compile-time length N is processed by T = N/E threads; each
// thread keeps E complex values in registers.  A pass of radix R performs E/R
// butterflies per thread entirely in registers; between passes the values are
// exchanged through shared memory (one store + one load per element).  The
// Stockham autosort indexing (input j + r*N/R, output (j/Ns)*Ns*R + j%Ns + r*Ns)
// leaves the result in natural order, so no bit-reversal pass is needed.
//
// Shared-memory layout is described by an element pointer `base` (this thread's
// sequence) and an element stride `es`, so the same engine serves contiguous
// rows and strided columns (columns use es = S+1 with S sequences interleaved,
// which keeps every warp access to full 128-byte rows).
//
// Twiddles come from a per-length table exp(-2*pi*i*k/N), k < N, built on the
// host in double precision and staged into shared memory by the caller.
#pragma once
#include <type_traits>

#include "common.cuh"

namespace marie {

template <int... Rs> struct RList {};

// Shared-memory addressing of position p of a sequence: p*es, plus one pad
// element every 16 positions when swz is set (row layouts, where the first
// pass writes with stride R and would otherwise hit one bank).
// half: column layouts whose rows are half a bank line (S * sizeof(V) = 64 B)
// insert half a line after every block of 16 rows, so that rows 16 apart
// (written at once by neighbouring thread groups of a radix-16 pass) fall in
// alternate halves of the banks; consecutive rows stay contiguous.
struct SAddr {
  int es, m, half;
  __host__ __device__ SAddr(int e) : es(e), m(0), half(0) {}
  __host__ __device__ SAddr(int e, bool swz) : es(e), m(swz ? -1 : 0), half(0) {}
  __host__ __device__ SAddr(int e, bool swz, int h) : es(e), m(swz ? -1 : 0), half(h) {}
  __device__ __forceinline__ int operator()(int p) const { return p * es + ((p >> 4) & m) + (p >> 4) * half; }
};

// Reversed radix list: the inverse transform runs the forward schedule
// backwards, so its first pass consumes the registers exactly as the forward
// transform's last pass left them (no exchange between a forward transform, a
// pointwise product and the inverse transform).
template <typename A, typename B> struct RCat;
template <int... A, int... B> struct RCat<RList<A...>, RList<B...>> { using type = RList<A..., B...>; };
template <typename L> struct RRev;
template <> struct RRev<RList<>> { using type = RList<>; };
template <int R0, int... Rs> struct RRev<RList<R0, Rs...>> {
  using type = typename RCat<typename RRev<RList<Rs...>>::type, RList<R0>>::type;
};

// Radix schedule per FFT length for 4-byte reals (FP32): radix-16 passes keep
// 16 complex values per thread and halve the exchanges of the 256-point
// transform.  E = lcm of the radices (values per thread).
template <int N> struct FFTCfgWide;
template <> struct FFTCfgWide<16>  { using R = RList<16>;     static constexpr int E = 16; };
template <> struct FFTCfgWide<128> { using R = RList<16, 8>;  static constexpr int E = 16; };
template <> struct FFTCfgWide<256> { using R = RList<16, 16>; static constexpr int E = 16; };

// Radix schedule per FFT length (FP64, and FP32 lengths without a wide entry).
// The first radix is even so that a zero-padded input (only the first N/2
// values non-zero) skips the loads of the known-zero half in the first pass.
template <int N> struct FFTCfg;
template <> struct FFTCfg<8>   { using R = RList<8>;        static constexpr int E = 8; };
template <> struct FFTCfg<16>  { using R = RList<4, 4>;     static constexpr int E = 4; };
template <> struct FFTCfg<24>  { using R = RList<8, 3>;     static constexpr int E = 24; };
template <> struct FFTCfg<32>  { using R = RList<8, 4>;     static constexpr int E = 8; };
template <> struct FFTCfg<40>  { using R = RList<2, 4, 5>;  static constexpr int E = 20; };
template <> struct FFTCfg<48>  { using R = RList<4, 4, 3>;  static constexpr int E = 12; };
template <> struct FFTCfg<64>  { using R = RList<8, 8>;     static constexpr int E = 8; };
template <> struct FFTCfg<80>  { using R = RList<4, 4, 5>;  static constexpr int E = 20; };
template <> struct FFTCfg<96>  { using R = RList<8, 4, 3>;  static constexpr int E = 24; };
template <> struct FFTCfg<128> { using R = RList<8, 4, 4>;  static constexpr int E = 8; };
template <> struct FFTCfg<160> { using R = RList<4, 4, 2, 5>; static constexpr int E = 20; };
template <> struct FFTCfg<192> { using R = RList<8, 8, 3>;  static constexpr int E = 24; };
template <> struct FFTCfg<256> { using R = RList<8, 8, 4>;  static constexpr int E = 8; };
template <> struct FFTCfg<320> { using R = RList<4, 4, 4, 5>; static constexpr int E = 20; };
template <> struct FFTCfg<384> { using R = RList<8, 8, 2, 3>; static constexpr int E = 24; };
template <> struct FFTCfg<512> { using R = RList<8, 8, 8>;  static constexpr int E = 8; };

template <typename L> struct RFirst;
template <int R0, int... Rs> struct RFirst<RList<R0, Rs...>> { static constexpr int value = R0; };

// ---------------------------------------------------------------------------
// Butterfly additions.  An FP32 complex value is a pair of f32 registers, so a
// complex add or subtract is one packed f32x2 instruction (PTX add/sub.rn.f32x2,
// sm_100 and later) instead of two; results are bitwise those of two FADDs.
// Sums that involve a multiply stay scalar so that they contract into FMAs.
// ---------------------------------------------------------------------------
template <typename V> __device__ __forceinline__ V badd(V a, V b) { return cadd(a, b); }
template <typename V> __device__ __forceinline__ V bsub(V a, V b) { return csub(a, b); }
template <> __device__ __forceinline__ float2 badd<float2>(float2 a, float2 b) {
  float2 r;
  asm("{\n\t.reg .b64 pa, pb, pd;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
      "add.rn.f32x2 pd, pa, pb;\n\tmov.b64 {%0, %1}, pd;\n\t}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
template <> __device__ __forceinline__ float2 bsub<float2>(float2 a, float2 b) {
  float2 r;
  asm("{\n\t.reg .b64 pa, pb, pd;\n\tmov.b64 pa, {%2, %3};\n\tmov.b64 pb, {%4, %5};\n\t"
      "sub.rn.f32x2 pd, pa, pb;\n\tmov.b64 {%0, %1}, pd;\n\t}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}

// ---------------------------------------------------------------------------
// Small DFTs in registers.  Forward uses exp(-2*pi*i/R); INV uses exp(+2*pi*i/R).
// ---------------------------------------------------------------------------
template <int R, bool INV> struct DFT;

template <bool INV> struct DFT<2, INV> {
  template <typename V> __device__ __forceinline__ static void run(V* v) {
    V a = v[0], b = v[1];
    v[0] = badd(a, b);
    v[1] = bsub(a, b);
  }
};

template <bool INV> struct DFT<4, INV> {
  template <typename V> __device__ __forceinline__ static void run(V* v) {
    V t0 = badd(v[0], v[2]), t1 = bsub(v[0], v[2]);
    V t2 = badd(v[1], v[3]), t3 = rot90<INV>(bsub(v[1], v[3]));
    v[0] = badd(t0, t2);
    v[2] = bsub(t0, t2);
    v[1] = cadd(t1, t3);
    v[3] = csub(t1, t3);
  }
};

template <bool INV> struct DFT<8, INV> {
  template <typename V> __device__ __forceinline__ static void run(V* v) {
    using T = decltype(V::x);
    const T h = (T)0.70710678118654752440;  // cos(pi/4)
    V a[4], b[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      a[k] = badd(v[k], v[k + 4]);
      b[k] = bsub(v[k], v[k + 4]);
    }
    // b[k] *= exp(-+ i*pi*k/4)
    b[1] = INV ? mk<V>(h * (b[1].x - b[1].y), h * (b[1].x + b[1].y))
               : mk<V>(h * (b[1].x + b[1].y), h * (b[1].y - b[1].x));
    b[2] = rot90<INV>(b[2]);
    b[3] = INV ? mk<V>(-h * (b[3].x + b[3].y), h * (b[3].x - b[3].y))
               : mk<V>(h * (b[3].y - b[3].x), -h * (b[3].x + b[3].y));
    DFT<4, INV>::run(a);
    DFT<4, INV>::run(b);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      v[2 * q] = a[q];
      v[2 * q + 1] = b[q];
    }
  }
};

template <bool INV> struct DFT<3, INV> {
  template <typename V> __device__ __forceinline__ static void run(V* v) {
    using T = decltype(V::x);
    const T s = (T)0.86602540378443864676;  // sin(2*pi/3)
    V t1 = cadd(v[1], v[2]);
    V t2 = mk<V>(v[0].x - (T)0.5 * t1.x, v[0].y - (T)0.5 * t1.y);
    V d = csub(v[1], v[2]);
    V t3 = rot90<INV>(mk<V>(s * d.x, s * d.y));
    v[0] = cadd(v[0], t1);
    v[1] = cadd(t2, t3);
    v[2] = csub(t2, t3);
  }
};

template <bool INV> struct DFT<5, INV> {
  template <typename V> __device__ __forceinline__ static void run(V* v) {
    using T = decltype(V::x);
    const T c1 = (T)0.30901699437494742410;   // cos(2*pi/5)
    const T c2 = (T)-0.80901699437494742410;  // cos(4*pi/5)
    const T s1 = (T)0.95105651629515357212;   // sin(2*pi/5)
    const T s2 = (T)0.58778525229247312917;   // sin(4*pi/5)
    V t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
    V t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
    V a1 = mk<V>(v[0].x + c1 * t1.x + c2 * t2.x, v[0].y + c1 * t1.y + c2 * t2.y);
    V a2 = mk<V>(v[0].x + c2 * t1.x + c1 * t2.x, v[0].y + c2 * t1.y + c1 * t2.y);
    V b1 = mk<V>(s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y);
    V b2 = mk<V>(s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y);
    V rb1 = rot90<INV>(b1), rb2 = rot90<INV>(b2);
    v[0] = cadd(v[0], cadd(t1, t2));
    v[1] = cadd(a1, rb1);
    v[4] = csub(a1, rb1);
    v[2] = cadd(a2, rb2);
    v[3] = csub(a2, rb2);
  }
};

template <bool INV> struct DFT<16, INV> {
  template <typename V> __device__ __forceinline__ static void run(V* v) {
    V a[8], b[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      a[k] = badd(v[k], v[k + 8]);
      b[k] = bsub(v[k], v[k + 8]);
    }
    twiddle16(b);
    DFT<8, INV>::run(a);
    DFT<8, INV>::run(b);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      v[2 * q] = a[q];
      v[2 * q + 1] = b[q];
    }
  }
  // upper half of the inputs is zero (zero-padded transform)
  template <typename V> __device__ __forceinline__ static void run_half(V* v) {
    V a[8], b[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = b[k] = v[k];
    twiddle16(b);
    DFT<8, INV>::run(a);
    DFT<8, INV>::run(b);
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      v[2 * q] = a[q];
      v[2 * q + 1] = b[q];
    }
  }
  // b[k] *= exp(-+ 2 pi i k / 16), k = 1..7
  template <typename V> __device__ __forceinline__ static void twiddle16(V* b) {
    using T = decltype(V::x);
    const T c1 = (T)0.92387953251128675613;  // cos(pi/8)
    const T s1 = (T)0.38268343236508977173;  // sin(pi/8)
    const T h = (T)0.70710678118654752440;   // cos(pi/4)
    const T sg = INV ? (T)1 : (T)-1;         // sign of the imaginary part of the root
    const T wr[8] = {1, c1, h, s1, 0, -s1, -h, -c1};
    const T wi[8] = {0, s1, h, c1, 1, c1, h, s1};
#pragma unroll
    for (int k = 1; k < 8; ++k) {
      if (k == 4) {
        b[4] = rot90<INV>(b[4]);
      } else {
        const T ci = sg * wi[k];
        b[k] = mk<V>(b[k].x * wr[k] - b[k].y * ci, b[k].x * ci + b[k].y * wr[k]);
      }
    }
  }
};

// DFT of R values whose upper half is zero.  Radix 16 and 8 skip the first
// butterfly stage; other radices run the full transform on the zeros.
template <int R, bool INV> struct DFTHalf {
  template <typename V> __device__ __forceinline__ static void run(V* v) { DFT<R, INV>::run(v); }
};
template <bool INV> struct DFTHalf<16, INV> {
  template <typename V> __device__ __forceinline__ static void run(V* v) { DFT<16, INV>::run_half(v); }
};
template <bool INV> struct DFTHalf<8, INV> {
  template <typename V> __device__ __forceinline__ static void run(V* v) {
    using T = decltype(V::x);
    const T h = (T)0.70710678118654752440;
    V a[4], b[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) a[k] = b[k] = v[k];
    b[1] = INV ? mk<V>(h * (b[1].x - b[1].y), h * (b[1].x + b[1].y))
               : mk<V>(h * (b[1].x + b[1].y), h * (b[1].y - b[1].x));
    b[2] = rot90<INV>(b[2]);
    b[3] = INV ? mk<V>(-h * (b[3].x + b[3].y), h * (b[3].x - b[3].y))
               : mk<V>(h * (b[3].y - b[3].x), -h * (b[3].x + b[3].y));
    DFT<4, INV>::run(a);
    DFT<4, INV>::run(b);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      v[2 * q] = a[q];
      v[2 * q + 1] = b[q];
    }
  }
};

// ---------------------------------------------------------------------------
// Pass recursion.  reg[b*R + r] holds input r of butterfly j = t + b*T.
// HALF: the inputs of this (first) pass have a zero upper half.
// ---------------------------------------------------------------------------
template <typename V, int N, int E, bool INV, int NS, bool HALF, typename L> struct Passes;

template <typename V, int N, int E, bool INV, int NS, bool HALF, int R, int... Rest>
struct Passes<V, N, E, INV, NS, HALF, RList<R, Rest...>> {
  static constexpr int T = N / E;
  static constexpr int NB = E / R;
  static_assert(E % R == 0, "E must be a multiple of every radix");

  // Runs this pass and all following ones.  After return, reg[b*R_last + r]
  // holds output position out_pos(t, b, r) of the last pass.
  __device__ __forceinline__ static void run(V* reg, V* base, SAddr es, int t, const V* tw) {
#pragma unroll
    for (int b = 0; b < NB; ++b) {
      const int j = t + b * T;
      V* v = reg + b * R;
      if (NS > 1) {
        const int k = j % NS;
#pragma unroll
        for (int r = 1; r < R; ++r) {
          V w = tw[(r * k * (N / (NS * R))) % N];
          v[r] = INV ? cmulc(v[r], w) : cmul(v[r], w);
        }
      }
      if (HALF)
        DFTHalf<R, INV>::run(v);
      else
        DFT<R, INV>::run(v);
    }
    if constexpr (sizeof...(Rest) > 0) {
      constexpr int R2 = RFirst<RList<Rest...>>::value;
      __syncthreads();
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        const int j = t + b * T;
        const int d = (j / NS) * NS * R + (j % NS);
#pragma unroll
        for (int r = 0; r < R; ++r) base[es(d + r * NS)] = reg[b * R + r];
      }
      __syncthreads();
#pragma unroll
      for (int b = 0; b < E / R2; ++b) {
#pragma unroll
        for (int r = 0; r < R2; ++r) reg[b * R2 + r] = base[es(t + b * T + r * (N / R2))];
      }
      Passes<V, N, E, INV, NS * R, false, RList<Rest...>>::run(reg, base, es, t, tw);
    }
  }
};

// Output position bookkeeping for the last pass.
template <int N, int E, int NS, typename L> struct LastPass;
template <int N, int E, int NS, int R> struct LastPass<N, E, NS, RList<R>> {
  static constexpr int R_last = R;
  static constexpr int NS_last = NS;
};
template <int N, int E, int NS, int R, int R2, int... Rest>
struct LastPass<N, E, NS, RList<R, R2, Rest...>> : LastPass<N, E, NS * R, RList<R2, Rest...>> {};

template <int N> struct HasWide { static constexpr bool value = false; };
template <> struct HasWide<16> { static constexpr bool value = true; };
template <> struct HasWide<128> { static constexpr bool value = true; };
template <> struct HasWide<256> { static constexpr bool value = true; };

template <typename V, int N, bool W = (sizeof(V) == 8) && HasWide<N>::value> struct Sched {
  using R = typename FFTCfg<N>::R;
  static constexpr int E = FFTCfg<N>::E;
};
template <typename V, int N> struct Sched<V, N, true> {
  using R = typename FFTCfgWide<N>::R;
  static constexpr int E = FFTCfgWide<N>::E;
};

// Transform of length N on values of type V (float2 / double2).  The forward
// transform uses the schedule's radix list; the inverse uses it reversed, so
// reg after FFT<V,N,false>::run is directly the input of FFT<V,N,true>::run.
// W selects the radix schedule: the wide one (radix 16, FP32 lengths 16, 128,
// 256) or the narrow one (radix <= 8); the default is the wide one where it
// exists.  The matvec autotuner times both for the z pass.
template <typename V, int N, bool INV, bool W = (sizeof(V) == 8) && HasWide<N>::value> struct FFT {
  using RF = typename Sched<V, N, W>::R;
  using RL_ = typename std::conditional<INV, typename RRev<RF>::type, RF>::type;
  static constexpr int E = Sched<V, N, W>::E;
  static constexpr int T = N / E;
  static constexpr int R0 = RFirst<RL_>::value;
  using LP = LastPass<N, E, 1, RL_>;
  static constexpr int RL = LP::R_last;
  static constexpr int NSL = LP::NS_last;

  static_assert((T & (T - 1)) == 0, "threads per transform must be a power of two");
  // Every caller launches exactly T threads per transform, so t < T.  Masking
  // states that range to the compiler, which then folds the position
  // arithmetic (carries out of the low bits, the first/second-half tests of a
  // zero-padded input) into per-thread constants.
  __device__ __forceinline__ static int lane(int t) { return t & (T - 1); }

  // Input position of reg[b*R0 + r] for the first pass.
  __device__ __forceinline__ static int in_pos(int t, int b, int r) { return lane(t) + b * T + r * (N / R0); }

  // Load the first pass's inputs from shared memory.  Positions >= n_valid are
  // treated as zero without being read (zero padding).
  __device__ __forceinline__ static void load(V* reg, const V* base, SAddr es, int t, int n_valid) {
#pragma unroll
    for (int b = 0; b < E / R0; ++b) {
#pragma unroll
      for (int r = 0; r < R0; ++r) {
        const int p = in_pos(t, b, r);
        reg[b * R0 + r] = (p < n_valid) ? base[es(p)] : mk<V>(0, 0);
      }
    }
  }
  // Same, but the caller guarantees n_valid <= N/2: the upper half of every
  // first-pass butterfly is zero.  Pair with run_half().
  __device__ __forceinline__ static void load_half(V* reg, const V* base, SAddr es, int t, int n_valid) {
#pragma unroll
    for (int b = 0; b < E / R0; ++b) {
#pragma unroll
      for (int r = 0; r < R0; ++r) {
        const int p = in_pos(t, b, r);
        reg[b * R0 + r] = (r < R0 / 2 && p < n_valid) ? base[es(p)] : mk<V>(0, 0);
      }
    }
  }
  __device__ __forceinline__ static void run(V* reg, V* base, SAddr es, int t, const V* tw) {
    Passes<V, N, E, INV, 1, false, RL_>::run(reg, base, es, lane(t), tw);
  }
  // First pass on inputs with a zero upper half (R0 even).
  __device__ __forceinline__ static void run_half(V* reg, V* base, SAddr es, int t, const V* tw) {
    static_assert(R0 % 2 == 0, "zero-half skipping needs an even first radix");
    Passes<V, N, E, INV, 1, true, RL_>::run(reg, base, es, lane(t), tw);
  }
  // Output position of reg[b*RL + r] after run().
  __device__ __forceinline__ static int out_pos(int t, int b, int r) {
    const int j = lane(t) + b * T;
    return (j / NSL) * NSL * RL + (j % NSL) + r * NSL;
  }
  // Store all outputs (natural order) back to shared memory.  Caller syncs.
  __device__ __forceinline__ static void store(const V* reg, V* base, SAddr es, int t) {
#pragma unroll
    for (int b = 0; b < E / RL; ++b)
#pragma unroll
      for (int r = 0; r < RL; ++r) base[es(out_pos(t, b, r))] = reg[b * RL + r];
  }
};

}  // namespace marie
