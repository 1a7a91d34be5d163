// Device-side complex FP32 FFT building blocks for the scalar-propagation passes.
//
// One FFT of length N (a power of two) is computed by T = N/E threads, each holding
// E elements in registers.  The schedule is a Stockham auto-sort decomposition
// (Govindaraju et al., "High performance discrete Fourier transforms on graphics
// processors", SC'08): stage s with radix R and span Ns reads x[j + r*N/R], applies
// the twiddles w_{Ns*R}^{r*(j mod Ns)}, runs an R-point DFT in registers and writes
// to j/Ns*Ns*R + j mod Ns + r*Ns.  The first and the last stage use the same radix,
// so the last stage leaves a thread holding exactly the positions that the first
// stage of another transform reads: an inverse transform, a pointwise operation and
// a forward transform chain in registers without touching shared memory in between.
// Intermediate stages exchange through shared memory with one pad slot per 16
// elements, which keeps both the strided writes and the unit-stride reads free of
// bank conflicts for the radices used here.
//
// Only the forward (negative exponent) transform is written out; inverse
// transforms use IFFT(x) = conj(FFT(conj(x))), with the 1/N factors folded into
// the transfer functions by the host.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fo {

__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n >> 1); }

// Stage schedule for N = 2^nb with E = 2^e elements per thread: first and last
// stage have radix E, the middle bits are split into chunks of at most e bits.
template <int N, int E>
struct Sched {
  static constexpr int nb = ilog2c(N);
  static constexpr int e = ilog2c(E);
  static_assert((1 << nb) == N, "N must be a power of two");
  static_assert((1 << e) == E, "E must be a power of two");
  static_assert(nb == e || nb >= 2 * e, "N must be E or at least E*E");
  static constexpr int rem = (nb == e) ? 0 : nb - 2 * e;
  static constexpr int nmid = (rem + e - 1) / e;
  static constexpr int S = (nb == e) ? 1 : 2 + nmid;
  static constexpr int T = N / E;
  __host__ __device__ static constexpr int bits(int s) {
    return (S == 1) ? e
           : (s == 0 || s == S - 1) ? e
           : ((s - 1) < rem / e ? e : rem - (rem / e) * e);
  }
  __host__ __device__ static constexpr int span(int s) {  // Ns = product of radices before s
    return s == 0 ? 1 : span(s - 1) << bits(s - 1);
  }
  // Offset of stage s's twiddle table (stages >= 1; table s holds R*Ns entries,
  // entry r*Ns + k = exp(-2 pi i r k / (Ns R))).
  __host__ __device__ static constexpr int twoff(int s) {
    return s <= 1 ? 0 : twoff(s - 1) + (1 << bits(s - 1)) * span(s - 1);
  }
  static constexpr int twsize = twoff(S);
};

// Host-side copy of the schedule for runtime (N, E): fills the stage-major
// twiddle tables of every stage s >= 1 (see Sched::twoff).  Returns the entry count.
inline int stage_twiddle_count(int N, int E) {
  int nb = ilog2c(N), e = ilog2c(E);
  if (nb == e) return 0;
  const int rem = nb - 2 * e, nmid = (rem + e - 1) / e, S = 2 + nmid;
  int total = 0, span = 1;
  for (int s = 0; s < S; ++s) {
    const int b = (s == 0 || s == S - 1) ? e : ((s - 1) < rem / e ? e : rem - (rem / e) * e);
    if (s >= 1) total += (1 << b) * span;
    span <<= b;
  }
  return total;
}

template <typename F>
inline void for_each_stage_twiddle(int N, int E, F f) {  // f(index, numerator, denominator)
  int nb = ilog2c(N), e = ilog2c(E);
  if (nb == e) return;
  const int rem = nb - 2 * e, nmid = (rem + e - 1) / e, S = 2 + nmid;
  int off = 0, span = 1;
  for (int s = 0; s < S; ++s) {
    const int b = (s == 0 || s == S - 1) ? e : ((s - 1) < rem / e ? e : rem - (rem / e) * e);
    const int R = 1 << b;
    if (s >= 1) {
      for (int r = 0; r < R; ++r)
        for (int k = 0; k < span; ++k) f(off + r * span + k, (long long)r * k, (long long)span * R);
      off += R * span;
    }
    span <<= b;
  }
}

// Complex add / subtract as one paired-FP32 instruction each (sm_100 and later):
// the (re, im) pair of a float2 is exactly the operand pair of FADD2 / FFMA2, and
// each lane rounds like the scalar operation, so results are unchanged.  a - b is
// formed as fma(b, -1, a), which is exact before its single rounding.
#ifndef FO_F32X2
#define FO_F32X2 1
#endif
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
#if FO_F32X2
  return __fadd2_rn(a, b);
#else
  return make_float2(a.x + b.x, a.y + b.y);
#endif
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
#if FO_F32X2
  return __ffma2_rn(b, make_float2(-1.f, -1.f), a);
#else
  return make_float2(a.x - b.x, a.y - b.y);
#endif
}
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
// a * (-i)
__device__ __forceinline__ float2 cmul_mi(float2 a) { return make_float2(a.y, -a.x); }
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }

// Two independent complex values carried by one thread (two adjacent columns of
// the column pass, or two rows of the row pass).  Every operation below applies
// to both halves, so a thread runs two transforms with the same twiddles and
// moves them through shared memory as one 16-byte access.
struct __align__(16) cf2 {
  float2 a, b;
};
__device__ __forceinline__ cf2 cadd(cf2 x, cf2 y) { return cf2{cadd(x.a, y.a), cadd(x.b, y.b)}; }
__device__ __forceinline__ cf2 csub(cf2 x, cf2 y) { return cf2{csub(x.a, y.a), csub(x.b, y.b)}; }
__device__ __forceinline__ cf2 cmul(cf2 x, float2 w) { return cf2{cmul(x.a, w), cmul(x.b, w)}; }
__device__ __forceinline__ cf2 cmul_mi(cf2 x) { return cf2{cmul_mi(x.a), cmul_mi(x.b)}; }
__device__ __forceinline__ cf2 cconj(cf2 x) { return cf2{cconj(x.a), cconj(x.b)}; }
template <typename V>
__device__ __forceinline__ V vzero();
template <>
__device__ __forceinline__ float2 vzero<float2>() { return make_float2(0.f, 0.f); }
template <>
__device__ __forceinline__ cf2 vzero<cf2>() { return cf2{make_float2(0.f, 0.f), make_float2(0.f, 0.f)}; }
// w8 multiplications used by the radix-8 butterfly
__device__ __forceinline__ float2 mul_w8_1(float2 d) { return make_float2(0.70710678118654752440f * (d.x + d.y), 0.70710678118654752440f * (d.y - d.x)); }
__device__ __forceinline__ float2 mul_w8_3(float2 d) { return make_float2(0.70710678118654752440f * (d.y - d.x), -0.70710678118654752440f * (d.x + d.y)); }
__device__ __forceinline__ cf2 mul_w8_1(cf2 d) { return cf2{mul_w8_1(d.a), mul_w8_1(d.b)}; }
__device__ __forceinline__ cf2 mul_w8_3(cf2 d) { return cf2{mul_w8_3(d.a), mul_w8_3(d.b)}; }

// cos/sin of 2*pi*k/16, k = 1..3 (exact decimal expansions of the algebraic values)
#define FO_C16_1 0.92387953251128675613f
#define FO_S16_1 0.38268343236508977173f
#define FO_SQRT1_2 0.70710678118654752440f

// In-place DFTs on a[o], a[o+1], ... (forward sign).  Outputs in natural order.
template <int R>
struct Dft;

template <>
struct Dft<1> {
  __host__ __device__ static constexpr int out(int r) { return r; }
  template <typename V, int E>
  __device__ __forceinline__ static void run(V (&)[E], int) {}
};

template <>
struct Dft<2> {
  __host__ __device__ static constexpr int out(int r) { return r; }
  template <typename V, int E>
  __device__ __forceinline__ static void run(V (&a)[E], int o) {
    V t = a[o];
    a[o] = cadd(t, a[o + 1]);
    a[o + 1] = csub(t, a[o + 1]);
  }
};

template <typename V>
__device__ __forceinline__ void dft4(V& a0, V& a1, V& a2, V& a3) {
  V t0 = cadd(a0, a2), t1 = csub(a0, a2);
  V t2 = cadd(a1, a3), t3 = cmul_mi(csub(a1, a3));
  a0 = cadd(t0, t2);
  a2 = csub(t0, t2);
  a1 = cadd(t1, t3);
  a3 = csub(t1, t3);
}

template <>
struct Dft<4> {
  __host__ __device__ static constexpr int out(int r) { return r; }
  template <typename V, int E>
  __device__ __forceinline__ static void run(V (&a)[E], int o) {
    dft4(a[o], a[o + 1], a[o + 2], a[o + 3]);
  }
};

template <>
struct Dft<8> {
  __host__ __device__ static constexpr int out(int r) { return r; }
  template <typename V, int E>
  __device__ __forceinline__ static void run(V (&a)[E], int o) {
    // even/odd split: E = DFT4(a0,a2,a4,a6), O = DFT4(a1,a3,a5,a7)
    V e0 = a[o], e1 = a[o + 2], e2 = a[o + 4], e3 = a[o + 6];
    V d0 = a[o + 1], d1 = a[o + 3], d2 = a[o + 5], d3 = a[o + 7];
    dft4(e0, e1, e2, e3);
    dft4(d0, d1, d2, d3);
    // w8^k * O[k]
    d1 = mul_w8_1(d1);
    d2 = cmul_mi(d2);
    d3 = mul_w8_3(d3);
    a[o] = cadd(e0, d0);
    a[o + 4] = csub(e0, d0);
    a[o + 1] = cadd(e1, d1);
    a[o + 5] = csub(e1, d1);
    a[o + 2] = cadd(e2, d2);
    a[o + 6] = csub(e2, d2);
    a[o + 3] = cadd(e3, d3);
    a[o + 7] = csub(e3, d3);
  }
};

// 16 = 4 x 4 in place: n = 4*n1 + n2, k = k1 + 4*k2.  Output X[r] is left in
// register out(r) = 4*(r%4) + r/4 (a compile-time renaming, no data movement).
template <>
struct Dft<16> {
  __host__ __device__ static constexpr int out(int r) { return 4 * (r % 4) + r / 4; }
  template <typename V, int E>
  __device__ __forceinline__ static void run(V (&a)[E], int o) {
#pragma unroll
    for (int n2 = 0; n2 < 4; ++n2) dft4(a[o + n2], a[o + 4 + n2], a[o + 8 + n2], a[o + 12 + n2]);
    // a[o + n2 + 4*k1] = Y[k1][n2]; twiddles w16^(n2*k1)
    const float2 w1 = make_float2(FO_C16_1, -FO_S16_1);
    const float2 w2 = make_float2(FO_SQRT1_2, -FO_SQRT1_2);
    const float2 w3 = make_float2(FO_S16_1, -FO_C16_1);
    const float2 w6 = make_float2(-FO_SQRT1_2, -FO_SQRT1_2);
    const float2 w9 = make_float2(-FO_C16_1, FO_S16_1);
    a[o + 1 + 4] = cmul(a[o + 1 + 4], w1);
    a[o + 2 + 4] = cmul(a[o + 2 + 4], w2);
    a[o + 3 + 4] = cmul(a[o + 3 + 4], w3);
    a[o + 1 + 8] = cmul(a[o + 1 + 8], w2);
    a[o + 2 + 8] = cmul_mi(a[o + 2 + 8]);
    a[o + 3 + 8] = cmul(a[o + 3 + 8], w6);
    a[o + 1 + 12] = cmul(a[o + 1 + 12], w3);
    a[o + 2 + 12] = cmul(a[o + 2 + 12], w6);
    a[o + 3 + 12] = cmul(a[o + 3 + 12], w9);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) dft4(a[o + 4 * k1], a[o + 4 * k1 + 1], a[o + 4 * k1 + 2], a[o + 4 * k1 + 3]);
    // X[k1 + 4*k2] is now in a[o + 4*k1 + k2]
  }
};

// Shared-memory slot of element `pos` (one pad slot per 16 elements).
__host__ __device__ __forceinline__ constexpr int spad(int pos) { return pos + (pos >> 4); }

// For powers of two Ns, R and a Stockham destination d of span Ns (or a source
// position j < M with M a power of two), the padded slot of d + r*Ns is
// spad(d) + padoff(r*Ns): the low four bits of d never carry into the offset.
// Addresses are then one padded base per butterfly plus compile-time offsets.
__host__ __device__ constexpr int padoff(int k) { return k + k / 16; }

template <int N>
struct SmemSize {
  static constexpr int value = N + N / 16;  // float2 slots per transform
};

// Register i of thread t holds position t + i*(N/E) on entry to the first stage
// and on exit from the last stage.
template <int N, int E>
__device__ __forceinline__ int reg_pos(int t, int i) { return t + i * (N / E); }

// One Stockham stage s >= 1: registers <- smem, twiddle, DFT.
template <int N, int E, int s, int PS, typename V>
__device__ __forceinline__ void stage_from_smem(V (&v)[E], int t, const float2* __restrict__ tw,
                                                const V* sm) {
  using SC = Sched<N, E>;
  constexpr int R = 1 << SC::bits(s);
  constexpr int Ns = SC::span(s);
  constexpr int T = SC::T;
  constexpr int NB = E / R;  // butterflies per thread
#pragma unroll
  for (int m = 0; m < NB; ++m) {
    const int j = t + m * T;
    const V* base = sm + spad(j) * PS;
#pragma unroll
    for (int r = 0; r < R; ++r) v[m * R + r] = base[padoff(r * (N / R)) * PS];
    if constexpr (Ns > 1) {
      const int k = j & (Ns - 1);
#pragma unroll
      for (int r = 1; r < R; ++r) {
        const float2 w = tw[SC::twoff(s) + r * Ns + k];
        v[m * R + r] = cmul(v[m * R + r], w);
      }
    }
    Dft<R>::run(v, m * R);
  }
}

// Write the outputs of stage s (s < S-1) to smem at their Stockham destinations.
template <int N, int E, int s, int PS, typename V>
__device__ __forceinline__ void stage_to_smem(const V (&v)[E], int t, V* sm) {
  using SC = Sched<N, E>;
  constexpr int R = 1 << SC::bits(s);
  constexpr int Ns = SC::span(s);
  constexpr int T = SC::T;
  constexpr int NB = E / R;
#pragma unroll
  for (int m = 0; m < NB; ++m) {
    const int j = t + m * T;
    const int d = (j / Ns) * Ns * R + (j & (Ns - 1));
    V* base = sm + spad(d) * PS;
#pragma unroll
    for (int r = 0; r < R; ++r) base[padoff(r * Ns) * PS] = v[m * R + Dft<R>::out(r)];
  }
}

// Barrier among the threads of one transform: the whole CTA (bar_id 0) or the
// bar_n threads of a named barrier (bar_id 1..15, bar_n a multiple of 32).
__device__ __forceinline__ void fft_sync(int bar_id, int bar_n) {
  if (bar_id == 0)
    __syncthreads();
  else
    asm volatile("bar.sync %0, %1;\n" ::"r"(bar_id), "r"(bar_n) : "memory");
}

template <int N, int E, int s, int PS, typename V>
__device__ __forceinline__ void stages_from(V (&v)[E], int t, const float2* __restrict__ tw, V* sm, int bar_id,
                                            int bar_n) {
  using SC = Sched<N, E>;
  if constexpr (s < SC::S) {
    fft_sync(bar_id, bar_n);  // earlier readers of this smem region are done
    stage_to_smem<N, E, s - 1, PS>(v, t, sm);
    fft_sync(bar_id, bar_n);
    stage_from_smem<N, E, s, PS>(v, t, tw, sm);
    stages_from<N, E, s + 1, PS>(v, t, tw, sm, bar_id, bar_n);
  }
}

// Forward FFT of the N elements spread over the T = N/E threads of one lane.  On
// entry register i of thread t holds x[t + i*T]; on exit it holds X[t + i*T].
// `sm` points at this lane's first smem slot and PS is the slot stride between
// consecutive positions.  Every thread of the block must make the call (it holds
// __syncthreads when the schedule has more than one stage).
template <int N, int E, int PS, typename V>
__device__ __forceinline__ void fft_forward(V (&v)[E], int t, const float2* __restrict__ tw, V* sm,
                                            int bar_id = 0, int bar_n = 0) {
  Dft<E>::run(v, 0);  // stage 0: radix E, span 1, no twiddles
  stages_from<N, E, 1, PS>(v, t, tw, sm, bar_id, bar_n);
  // the last stage has one butterfly of radix E per thread: register out(r) holds X[t + r*T]
  if constexpr (Dft<E>::out(1) != 1) {
    V w[E];
#pragma unroll
    for (int r = 0; r < E; ++r) w[r] = v[Dft<E>::out(r)];
#pragma unroll
    for (int r = 0; r < E; ++r) v[r] = w[r];
  }
}

// Twiddles of one thread held in registers.  Stage s >= 1 needs w^{r k} for
// r = 1..R-1 and k = j mod Ns of each of its E/R butterflies j = t + m*T; when T
// is a multiple of Ns every butterfly has the same k and one set serves all.
// The values do not depend on the data, so a kernel that transforms many
// tiles loads them once.
template <int N, int E>
struct TwRegs {
  using SC = Sched<N, E>;
  __host__ __device__ static constexpr int radix(int s) { return 1 << SC::bits(s); }
  __host__ __device__ static constexpr bool shared(int s) { return SC::T % SC::span(s) == 0; }
  __host__ __device__ static constexpr int count(int s) {
    return (s < 1 || s >= SC::S) ? 0 : (shared(s) ? radix(s) - 1 : (E / radix(s)) * (radix(s) - 1));
  }
  __host__ __device__ static constexpr int off(int s) { return s <= 1 ? 0 : off(s - 1) + count(s - 1); }
  static constexpr int total = off(SC::S);
  static constexpr int size = total > 0 ? total : 1;
};

template <int N, int E, int s>
__device__ __forceinline__ void load_twiddles_from(float2 (&w)[TwRegs<N, E>::size], int t,
                                                   const float2* __restrict__ tw) {
  using SC = Sched<N, E>;
  using TR = TwRegs<N, E>;
  if constexpr (s < SC::S) {
    constexpr int R = TR::radix(s);
    constexpr int Ns = SC::span(s);
    constexpr int NB = TR::shared(s) ? 1 : E / R;
#pragma unroll
    for (int m = 0; m < NB; ++m) {
      const int k = (t + m * SC::T) & (Ns - 1);
#pragma unroll
      for (int r = 1; r < R; ++r) w[TR::off(s) + m * (R - 1) + r - 1] = tw[SC::twoff(s) + r * Ns + k];
    }
    load_twiddles_from<N, E, s + 1>(w, t, tw);
  }
}
template <int N, int E>
__device__ __forceinline__ void load_twiddles(float2 (&w)[TwRegs<N, E>::size], int t, const float2* __restrict__ tw) {
  load_twiddles_from<N, E, 1>(w, t, tw);
}

// stage_from_smem with the twiddles taken from registers
template <int N, int E, int s, int PS, typename V>
__device__ __forceinline__ void stage_from_smem_r(V (&v)[E], int t, const float2 (&w)[TwRegs<N, E>::size],
                                                  const V* sm) {
  using SC = Sched<N, E>;
  using TR = TwRegs<N, E>;
  constexpr int R = TR::radix(s);
  constexpr int T = SC::T;
  constexpr int NB = E / R;
#pragma unroll
  for (int m = 0; m < NB; ++m) {
    const int j = t + m * T;
    const V* base = sm + spad(j) * PS;
#pragma unroll
    for (int r = 0; r < R; ++r) v[m * R + r] = base[padoff(r * (N / R)) * PS];
#pragma unroll
    for (int r = 1; r < R; ++r) {
      const int wi = TR::off(s) + (TR::shared(s) ? 0 : m * (R - 1)) + r - 1;
      v[m * R + r] = cmul(v[m * R + r], w[wi]);
    }
    Dft<R>::run(v, m * R);
  }
}

template <int N, int E, int s, int PS, typename V>
__device__ __forceinline__ void stages_from_r(V (&v)[E], int t, const float2 (&w)[TwRegs<N, E>::size], V* sm,
                                              int bar_id, int bar_n) {
  using SC = Sched<N, E>;
  if constexpr (s < SC::S) {
    fft_sync(bar_id, bar_n);
    stage_to_smem<N, E, s - 1, PS>(v, t, sm);
    fft_sync(bar_id, bar_n);
    stage_from_smem_r<N, E, s, PS>(v, t, w, sm);
    stages_from_r<N, E, s + 1, PS>(v, t, w, sm, bar_id, bar_n);
  }
}

// The last stage leaves X[t + r*T] in register out(r): rename into natural order.
template <int E, typename V>
__device__ __forceinline__ void fft_last_stage_order(V (&v)[E]) {
  if constexpr (Dft<E>::out(1) != 1) {
    V x[E];
#pragma unroll
    for (int r = 0; r < E; ++r) x[r] = v[Dft<E>::out(r)];
#pragma unroll
    for (int r = 0; r < E; ++r) v[r] = x[r];
  }
}

// fft_forward with register-resident twiddles (see TwRegs / load_twiddles).
template <int N, int E, int PS, typename V>
__device__ __forceinline__ void fft_forward_r(V (&v)[E], int t, const float2 (&w)[TwRegs<N, E>::size], V* sm,
                                              int bar_id = 0, int bar_n = 0) {
  Dft<E>::run(v, 0);
  stages_from_r<N, E, 1, PS>(v, t, w, sm, bar_id, bar_n);
  fft_last_stage_order<E>(v);
}

}  // namespace fo
