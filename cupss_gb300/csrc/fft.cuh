// Register/shared-memory FFT building blocks for the GB300 pseudospectral engine.
//
// A line of length L (a power of two 1..1024, or 3 * 2^a up to 384) is split as
// L = R * M: M threads cooperate on one line and each holds R complex values in
// registers.  The four-step form uses M = 2^floor(a/2) for L = 2^a or 3 * 2^a (R is M or
// 2M, or 3M or 6M).  Lines of 512 and 1024 points can instead take the split form below
// (template flag SP): R = 16 and M = L/16 threads, so that a pass over few long lines (a
// 2D grid) still gives the GPU enough threads.
//
//   step-1 layout: thread m holds positions  n = m + M*r,            r in [0,R)
//   step-2 layout: thread m holds positions  k = s + R*k',  s = m + M*j,
//                  j in [0, R/M), k' in [0,M)   (register index j*M + k')
//                  split form: k = m + M*f      (register index f)
//
// Forward transform (unnormalised, exp(-2 pi i n k / L)):
//   fwd_step1 (radix-R DFT over r, twiddle W_L^{m s}), store to the transpose
//   buffer at position s*M + m, sync, fwd_load_step2 (load, radix-M).
// Inverse transform (unnormalised, exp(+2 pi i n k / L)) runs the same steps
// backwards: inv_step2 in step-2 layout, inv_store_t, sync, inv_load_step1.
//
// The four-step split X[s + R k'] = sum_m W_M^{m k'} W_L^{m s} sum_r x[m + M r] W_R^{r s}
// is the standard Cooley-Tukey factorisation; the register DFTs are recursive
// radix-2 decimation in time with compile-time twiddles, ending in a radix-3 butterfly
// for orders 3 * 2^b.
//
// Split form (M = G*R threads, G = 2 or 4): the radix-M DFT of step 2 is itself split
// with m = a + R b, k' = e + G f (a, f in [0,R); b, e in [0,G)):
//   X[s + R (e + G f)] = sum_a W_R^{a f} W_M^{a e} sum_b W_G^{b e} Y_{a + R b}[s],
// Y_m[s] the step-1 output of thread m.  Thread m' = s + R e loads the G values of each
// a from row s of the transpose buffer and sums them with the roots W_G^{b e} (+-1, +-i,
// exact), twiddles and runs a radix-R DFT over a; its outputs k = m' + M f are cyclic like
// the step-1 inputs.  The inverse runs the same steps backwards: radix-R over f, twiddle,
// store at s*M + e*R + a, sync, thread m = a + R b sums the G values of each s.
#pragma once
#if !defined(__CUDACC_RTC__)
#include <cuda_runtime.h>
#endif
#include "twiddle32.h"

#if defined(__CUDACC__)
#define CG_HD __host__ __device__ __forceinline__
#else
#define CG_HD inline
#endif

namespace cupssgb {

// compile-time index sequence (no <utility> under NVRTC)
template <int... K>
struct iseq {};
template <int N, int... K>
struct make_iseq_t : make_iseq_t<N - 1, N - 1, K...> {};
template <int... K>
struct make_iseq_t<0, K...> {
  using type = iseq<K...>;
};
template <int N>
using make_iseq = typename make_iseq_t<N>::type;

CG_HD float2 c_add(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
CG_HD float2 c_sub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
CG_HD float2 c_mul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
CG_HD float2 c_mulc(float2 a, float2 b) {
  return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
CG_HD float2 c_conj(float2 a) { return make_float2(a.x, -a.y); }

// Programmatic dependent launch.  A step kernel launched with programmatic stream
// serialization may become resident while its predecessor in the stream drains.  At its
// top it lets its own successor launch (all of its CTAs are running by the time that
// fires) and then waits until the predecessor grid has completed and its memory is
// visible, before touching global memory.  Both are no-ops for a kernel launched without
// the attribute.
#if defined(__CUDACC__)
__device__ __forceinline__ void grid_dep_sync() {
#if defined(__CUDA_ARCH__)
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
}
#endif

#if defined(__CUDACC__)
// 32-bit shared-window address of a shared-memory pointer.
__device__ __forceinline__ unsigned smem_u32(const void* p) {
  unsigned sa;
  asm("{ .reg .u64 t; cvta.to.shared.u64 t, %1; cvt.u32.u64 %0, t; }" : "=r"(sa) : "l"(p));
  return sa;
}
// 8-byte asynchronous global -> shared copy to shared address sa (zero-filled when
// src_bytes is 0, in which case nothing is read).
__device__ __forceinline__ void cp_async8(unsigned sa, const float2* gsrc, int src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(sa), "l"(gsrc), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
#endif

// Butterfly sums on the paired FP32 pipe of sm_100+ (one f32x2 instruction per complex
// add or subtract; a - b is fma(b, -1, a), exact like the scalar subtraction).
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 1000)
__device__ __forceinline__ float2 p_add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 p_sub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
#else
CG_HD float2 p_add(float2 a, float2 b) { return c_add(a, b); }
CG_HD float2 p_sub(float2 a, float2 b) { return c_sub(a, b); }
#endif
CG_HD float2 c_scale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
CG_HD float2 c_muli(float2 a) { return make_float2(-a.y, a.x); }    // i * a
CG_HD float2 c_mulmi(float2 a) { return make_float2(a.y, -a.x); }   // -i * a

// Multiply by W_N^K (forward, W = exp(-2 pi i/N)) or its conjugate (INV), N dividing 64
// or 192.
template <int N, int K, bool INV>
CG_HD float2 tw_const(float2 a) {
  constexpr int k = K % N;
  static_assert(64 % N == 0 || 192 % N == 0, "compile-time twiddles of orders dividing 64 or 192");
  if constexpr (k == 0) {
    return a;
  } else if constexpr (4 * k == N) {
    return INV ? c_muli(a) : c_mulmi(a);
  } else if constexpr (2 * k == N) {
    return make_float2(-a.x, -a.y);
  } else if constexpr (4 * k == 3 * N) {
    return INV ? c_mulmi(a) : c_muli(a);
  } else if constexpr (64 % N == 0) {
    constexpr int j = k * (64 / N);
    constexpr float wr = kTw64Re[j];
    constexpr float wi = INV ? -kTw64Im[j] : kTw64Im[j];
    return c_mul(a, make_float2(wr, wi));
  } else {
    constexpr int j = k * (192 / N);
    constexpr float wr = kTw192Re[j];
    constexpr float wi = INV ? -kTw192Im[j] : kTw192Im[j];
    return c_mul(a, make_float2(wr, wi));
  }
}

// sqrt(3)/2 rounded to float (the imaginary part of W_3 = exp(-2 pi i/3))
constexpr float kSqrt3Half = 0x1.bb67aep-1f;

// In-place DFT of the N values v[O + S*i], i in [0,N), natural-order output.
template <int N, bool INV, int S>
struct Dft {
  // lo = e + W_N^K o, hi = e - W_N^K o.  Twiddles +-i stay on the scalar pipe, where the
  // swap and sign fold into the additions; every other sum uses the paired pipe.
  template <int K>
  CG_HD static void bfly(float2& lo, float2& hi, float2 e, float2 o) {
    constexpr int k = K % N;
    if constexpr (k == 0) {
      lo = p_add(e, o);
      hi = p_sub(e, o);
    } else if constexpr (2 * k == N) {
      lo = p_sub(e, o);
      hi = p_add(e, o);
    } else if constexpr (4 * k == N || 4 * k == 3 * N) {
      const float2 t = tw_const<N, K, INV>(o);
      lo = c_add(e, t);
      hi = c_sub(e, t);
    } else {
      const float2 t = tw_const<N, K, INV>(o);
      lo = p_add(e, t);
      hi = p_sub(e, t);
    }
  }
  template <int O, int... K>
  CG_HD static void combine(float2* v, iseq<K...>) {
    constexpr int H = N / 2;
    float2 ev[H], od[H];
#pragma unroll
    for (int q = 0; q < H; ++q) {
      ev[q] = v[O + 2 * S * q];
      od[q] = v[O + S + 2 * S * q];
    }
    (bfly<K>(v[O + S * K], v[O + S * (K + H)], ev[K], od[K]), ...);
  }
  template <int O>
  CG_HD static void run(float2* v) {
    if constexpr (N == 1) {
      return;
    } else if constexpr (N == 2) {
      float2 a = v[O], b = v[O + S];
      v[O] = p_add(a, b);
      v[O + S] = p_sub(a, b);
    } else if constexpr (N == 3) {
      // X0 = a + (b + c), X1,2 = a - (b + c)/2 -+ i sqrt(3)/2 (b - c) (forward; + for INV)
      const float2 a = v[O], b = v[O + S], c = v[O + 2 * S];
      const float2 t = p_add(b, c);
      const float2 u = make_float2(a.x - 0.5f * t.x, a.y - 0.5f * t.y);
      const float2 d = p_sub(b, c);
      const float2 w = INV ? make_float2(-kSqrt3Half * d.y, kSqrt3Half * d.x)
                           : make_float2(kSqrt3Half * d.y, -kSqrt3Half * d.x);
      v[O] = p_add(a, t);
      v[O + S] = p_add(u, w);
      v[O + 2 * S] = p_sub(u, w);
    } else {
      Dft<N / 2, INV, 2 * S>::template run<O>(v);
      Dft<N / 2, INV, 2 * S>::template run<O + S>(v);
      combine<O>(v, make_iseq<N / 2>{});
    }
  }
};

// log2 of the power-of-two part of a supported line length (L = 2^a or 3 * 2^a), -1 else
CG_HD constexpr int line_log2(int L) {
  int n = (L % 3 == 0) ? L / 3 : L;
  int a = 0;
  while (n > 1 && n % 2 == 0) {
    n /= 2;
    ++a;
  }
  return n == 1 ? a : -1;
}
CG_HD constexpr bool line_pow2(int L) { return L >= 1 && (L & (L - 1)) == 0; }

template <int L, bool SP = false>
struct LineCfg {
  static constexpr int lg = line_log2(L);
  static_assert(lg >= 0 && (line_pow2(L) ? L <= 1024 : L <= 384),
                "line length must be 2^a in [1, 1024] or 3 * 2^a up to 384");
  static constexpr bool kSplit = SP && (L >= 512) && line_pow2(L);
  static constexpr int M = kSplit ? L / 16 : (1 << (lg / 2));   // threads per line
  static constexpr int R = L / M;                               // values per thread
  static constexpr int J = kSplit ? 1 : R / M;   // s-values per thread in step 2 (1, 2, 3 or 6)
  static constexpr int G = kSplit ? M / R : 1;   // split form: threads per s-value in step 2
};

// Host-side threads per line (equals LineCfg<L, split>::M for every supported L).
CG_HD int line_m_of(int L, bool split) {
  if (split && L >= 512 && line_pow2(L)) return L / 16;
  return 1 << (line_log2(L) / 2);
}

// Twiddle super-table: the table for length L holds exp(-2 pi i j / L) for j in [0, L)
// and starts at tw + L for powers of two (L <= 2048) and at tw + kTwOdd + L for lengths
// 3 * 2^a (L <= 1536).
// The device load is a volatile read-only load: a kernel that runs a forward and an
// inverse transform of the same length reads the same twiddles twice, and letting the
// compiler merge those loads keeps every twiddle live in registers between the two
// transforms (spills and lower occupancy); an L1 hit is cheaper than that.
constexpr int kTwOdd = 4096;
constexpr int kTwLen = kTwOdd + 2 * 1536;   // float2 entries of the whole table
CG_HD int tw_base(int L) { return line_pow2(L) ? L : kTwOdd + L; }
#if !defined(__CUDACC_RTC__)
// Host: fills the kTwLen entries (double-precision angles rounded once to float).
inline void fill_twiddle_table(float2* h) {
  for (int i = 0; i < kTwLen; ++i) h[i] = make_float2(0.f, 0.f);
  for (int L = 1; L <= 2048; L *= 2)
    for (int j = 0; j < L; ++j) {
      const double a = -2.0 * 3.14159265358979323846 * (double)j / (double)L;
      h[tw_base(L) + j] = make_float2((float)__builtin_cos(a), (float)__builtin_sin(a));
    }
  for (int L = 3; L <= 1536; L *= 2)
    for (int j = 0; j < L; ++j) {
      const double a = -2.0 * 3.14159265358979323846 * (double)j / (double)L;
      h[tw_base(L) + j] = make_float2((float)__builtin_cos(a), (float)__builtin_sin(a));
    }
}
#endif
CG_HD float2 tw_load(const float2* tw, int L, int j) {
#if defined(__CUDA_ARCH__)
  float2 w;
  asm volatile("ld.global.nc.v2.f32 {%0, %1}, [%2];" : "=f"(w.x), "=f"(w.y) : "l"(tw + tw_base(L) + j));
  return w;
#else
  return tw[tw_base(L) + j];
#endif
}

template <int L, bool INV, bool SP = false>
CG_HD void step_r(float2 (&v)[LineCfg<L, SP>::R]) {
  Dft<LineCfg<L, SP>::R, INV, 1>::template run<0>(v);
}

// Forward step 1: v[r] = x[m + M r] in, v[s] = W_L^{m s} * DFT_R(x[m + M .])[s] out.
template <int L, bool SP = false>
CG_HD void fwd_step1(float2 (&v)[LineCfg<L, SP>::R], int m, const float2* tw) {
  constexpr int R = LineCfg<L, SP>::R;
  Dft<R, false, 1>::template run<0>(v);
#pragma unroll
  for (int s = 1; s < R; ++s) v[s] = c_mul(v[s], tw_load(tw, L, m * s));
}

// Step-2 DFTs of the four-step form: register index j*M + k holds position s*M + k
// (s = m + M j) of the transposed data; output register j*M + k' holds X[s + R k'].
template <int L, bool SP, bool INV, int... Js>
CG_HD void dft2_each(float2* v, iseq<Js...>) {
  (Dft<LineCfg<L, SP>::M, INV, 1>::template run<Js * LineCfg<L, SP>::M>(v), ...);
}
template <int L, bool SP = false>
CG_HD void fwd_dft2(float2 (&v)[LineCfg<L, SP>::R]) {
  dft2_each<L, SP, false>(v, make_iseq<LineCfg<L, SP>::J>{});
}
// register j*M + k' holds X[s + R k']; out register j*M + m' holds
// y_{m'}[s] = sum_k' X[s + R k'] W_M^{-m' k'}  (to be stored at position s*M + m').
template <int L, bool SP = false>
CG_HD void inv_dft2(float2 (&v)[LineCfg<L, SP>::R]) {
  dft2_each<L, SP, true>(v, make_iseq<LineCfg<L, SP>::J>{});
}

// W_G^q = exp(-2 pi i q / G) for G = 2 or 4: one of +-1, +-i, exact.
template <int G>
CG_HD float2 root_g(int q) {
  const int qq = (q * (4 / G)) & 3;
  return make_float2(qq == 0 ? 1.f : (qq == 2 ? -1.f : 0.f), qq == 1 ? -1.f : (qq == 3 ? 1.f : 0.f));
}

// Inverse step 1: v[s] = y_m[s] (loaded from positions s*M + m) in,
// v[r] = x[m + M r] out.
template <int L, bool SP = false>
CG_HD void inv_step1(float2 (&v)[LineCfg<L, SP>::R], int m, const float2* tw) {
  constexpr int R = LineCfg<L, SP>::R;
#pragma unroll
  for (int s = 1; s < R; ++s) v[s] = c_mulc(v[s], tw_load(tw, L, m * s));
  Dft<R, true, 1>::template run<0>(v);
}

// Transpose-buffer position written after fwd_step1 for value s.
template <int L, bool SP = false>
CG_HD int pos_t1(int m, int s) { return s * LineCfg<L, SP>::M + m; }
// Four-step form: position read before step 2 for register index idx (= j*M + k).
template <int L, bool SP = false>
CG_HD int pos_t2(int m, int idx) {
  constexpr int M = LineCfg<L, SP>::M;
  const int j = idx / M, k = idx % M;
  return (m + M * j) * M + k;
}

// Forward step 2 after the transpose (the buffer holds every thread's fwd_step1 output
// at pos_t1; ld(pos) reads the buffer at position pos): v[i] = X[pos_step2(m, i)] out.
template <int L, bool SP = false, class Ld>
CG_HD void fwd_load_step2(float2 (&v)[LineCfg<L, SP>::R], int m, const float2* tw, Ld&& ld) {
  using C = LineCfg<L, SP>;
  constexpr int M = C::M, R = C::R;
  if constexpr (!C::kSplit) {
#pragma unroll
    for (int i = 0; i < R; ++i) v[i] = ld(pos_t2<L, SP>(m, i));
    fwd_dft2<L, SP>(v);
  } else {
    constexpr int G = C::G;
    const int s = m % R, e = m / R;
    float2 w[G];
#pragma unroll
    for (int b = 0; b < G; ++b) w[b] = root_g<G>(b * e);
#pragma unroll
    for (int a = 0; a < R; ++a) {
      float2 acc = ld(s * M + a);
#pragma unroll
      for (int b = 1; b < G; ++b) acc = c_add(acc, c_mul(ld(s * M + a + R * b), w[b]));
      v[a] = acc;
    }
#pragma unroll
    for (int a = 1; a < R; ++a) v[a] = c_mul(v[a], tw_load(tw, M, a * e));
    Dft<R, false, 1>::template run<0>(v);
  }
}

// Inverse step 2 in registers: v[i] = X[pos_step2(m, i)] in; out the values that
// inv_store_t writes to the transpose buffer.
template <int L, bool SP = false>
CG_HD void inv_step2(float2 (&v)[LineCfg<L, SP>::R], int m, const float2* tw) {
  using C = LineCfg<L, SP>;
  constexpr int M = C::M, R = C::R;
  if constexpr (!C::kSplit) {
    inv_dft2<L, SP>(v);
  } else {
    Dft<R, true, 1>::template run<0>(v);
    const int e = m / R;
#pragma unroll
    for (int a = 1; a < R; ++a) v[a] = c_mulc(v[a], tw_load(tw, M, a * e));
  }
}
// Store of the inv_step2 output: st(pos, value) writes the transpose buffer.
template <int L, bool SP = false, class St>
CG_HD void inv_store_t(const float2 (&v)[LineCfg<L, SP>::R], int m, St&& st) {
  using C = LineCfg<L, SP>;
  constexpr int M = C::M, R = C::R;
  if constexpr (!C::kSplit) {
#pragma unroll
    for (int i = 0; i < R; ++i) st(pos_t2<L, SP>(m, i), v[i]);
  } else {
    const int s = m % R, e = m / R;
#pragma unroll
    for (int a = 0; a < R; ++a) st(s * M + e * R + a, v[a]);
  }
}
// After the transpose: loads and inverse step 1; v[r] = x[m + M r] out.
template <int L, bool SP = false, class Ld>
CG_HD void inv_load_step1(float2 (&v)[LineCfg<L, SP>::R], int m, const float2* tw, Ld&& ld) {
  using C = LineCfg<L, SP>;
  constexpr int M = C::M, R = C::R;
  if constexpr (!C::kSplit) {
#pragma unroll
    for (int s = 0; s < R; ++s) v[s] = ld(pos_t1<L, SP>(m, s));
  } else {
    constexpr int G = C::G;
    const int a = m % R, b = m / R;
    float2 w[G];
#pragma unroll
    for (int e = 0; e < G; ++e) w[e] = root_g<G>(b * e);
#pragma unroll
    for (int s = 0; s < R; ++s) {
      float2 acc = ld(s * M + a);
#pragma unroll
      for (int e = 1; e < G; ++e) acc = c_add(acc, c_mulc(ld(s * M + e * R + a), w[e]));
      v[s] = acc;
    }
  }
  inv_step1<L, SP>(v, m, tw);
}

// Index of the partner -k of k (mod n), k in [0, n).
CG_HD int neg_mod(int k, int n) { return k == 0 ? 0 : n - k; }

// Position of register index idx in the step-1 / step-2 layouts.  Both are cyclic:
// pos = m + step2_off(idx) with the offset a multiple of M.
template <int L, bool SP = false>
CG_HD int pos_step1(int m, int r) { return m + LineCfg<L, SP>::M * r; }
template <int L, bool SP = false>
CG_HD constexpr int step2_off(int idx) {
  constexpr int M = LineCfg<L, SP>::M;
  constexpr int R = LineCfg<L, SP>::R;
  return LineCfg<L, SP>::kSplit ? M * idx : M * (idx / M) + R * (idx % M);
}
template <int L, bool SP = false>
CG_HD int pos_step2(int m, int idx) { return m + step2_off<L, SP>(idx); }

// Padded shared-memory index of position n: one pad slot every M positions keeps
// the strided step-2 accesses free of bank conflicts.
template <int L, bool SP = false>
CG_HD int pad_pos(int n) { return n + n / LineCfg<L, SP>::M; }
template <int L, bool SP = false>
CG_HD constexpr int padded_len() { return L + L / LineCfg<L, SP>::M; }

}  // namespace cupssgb
