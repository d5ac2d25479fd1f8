// Per-mode Fourier-space math of the update: q-grid, term multipliers, implicit
// factors, noise amplitude and Fourier-space noise, dealias mask, packed-column
// unpacking.  Shared by the interpreted and the generated (NVRTC) update programs.
#pragma once
#include "engine_types.h"
#include "fft.cuh"
#include "philox.cuh"

namespace cupssgb {

struct VPoint {
  int kx, ky, kz;
  bool origin, nyx, nyy, nyz;
  float qx, qy, qz, q2;
};

// Grid sizes as the per-mode math sees them.  Kernels generated for one system fill
// them with compile-time constants, so that every index expression below folds.
struct Dims {
  int sx, sy, sz;
};
__device__ __forceinline__ Dims dims_of(const LineParams& P) { return Dims{P.sx, P.sy, P.sz}; }

__device__ __forceinline__ float q_of(int k, int n, float step) {
  return (float)(k < (n + 1) / 2 ? k : k - n) * step;   // src/field_init.cpp:248-250
}

__device__ __forceinline__ VPoint make_vpoint(const LineParams& P, const Dims& d, int kx, int ky, int kz) {
  VPoint vp;
  vp.kx = kx;
  vp.ky = ky;
  vp.kz = kz;
  vp.origin = (kx == 0 && ky == 0 && kz == 0);
  vp.nyx = (d.sx > 1) && (2 * kx == d.sx);
  vp.nyy = (d.sy > 1) && (2 * ky == d.sy);
  vp.nyz = (d.sz > 1) && (2 * kz == d.sz);
  vp.qx = q_of(kx, d.sx, P.stepqx);
  vp.qy = q_of(ky, d.sy, P.stepqy);
  vp.qz = q_of(kz, d.sz, P.stepqz);
  vp.q2 = vp.qx * vp.qx + vp.qy * vp.qy + vp.qz * vp.qz;
  return vp;
}

// Noise counter inputs of the system a CTA works on: the solver's (single system) or
// the batch member's (blockIdx.z).
struct NoiseKey {
  uint32_t key0, key1, step;
};

// Numerical value of prefactor k / noise base of phase field fi for this CTA's system.
__device__ __forceinline__ float pre_val(const LineParams& P, int k) {
  return P.mvals ? __ldg(P.mvals + (size_t)blockIdx.z * kMemberVals + k) : P.pres[k].pre;
}
__device__ __forceinline__ float noise_base_val(const LineParams& P, int fi) {
  return P.mvals ? __ldg(P.mvals + (size_t)blockIdx.z * kMemberVals + kMaxPres + fi) : P.f[fi].noise_base;
}

__device__ __forceinline__ float ipow(float x, int n) {
  float r = 1.f;
  for (int i = 0; i < n; ++i) r *= x;
  return r;
}

// Effective Fourier multiplier of one explicit term.  The reference multiplies the
// full C2C spectrum by i^s * P(q) (term_init.cpp:135-200) and then projects onto real
// fields each step (field.cpp:63-89).  On the half spectrum that projection keeps a
// monomial only when s + sum of its iq exponents over the axes that are NOT at their
// Nyquist index is even (at a Nyquist index q_a(-k) = q_a(k) under the reference's
// q convention, so odd powers there do not survive the projection).
__device__ __forceinline__ float term_mult(const LineParams& P, const TermK& T, const VPoint& vp) {
  float acc = 0.f;
  for (int j = 0; j < T.npres; ++j) {
    const PresK pr = P.pres[T.pres0 + j];
    const int e = T.s + (vp.nyx ? 0 : pr.iqx) + (vp.nyy ? 0 : pr.iqy) + (vp.nyz ? 0 : pr.iqz);
    if (e & 1) continue;
    float v = pre_val(P, T.pres0 + j);
    v *= ipow(vp.q2, pr.q2n);
    v *= ipow(vp.qx, pr.iqx);
    v *= ipow(vp.qy, pr.iqy);
    v *= ipow(vp.qz, pr.iqz);
    if (pr.invq > 0) {
      const float iq = vp.origin ? 0.f : 1.0f / sqrtf(vp.q2);
      v *= ipow(iq, pr.invq);
    }
    acc += v;
  }
  return acc;
}

// 1 - dt*sum implicit (dynamic, precalculateImplicit, field_init.cpp:242-267) or
// sum implicit (non-dynamic, setNotDynamic_k, field_kernels.cu:167-188).
__device__ __forceinline__ float implicit_factor(const LineParams& P, const FieldK& F, const VPoint& vp) {
  float acc = F.dynamic ? 1.f : 0.f;
  for (int j = 0; j < F.nimp; ++j) {
    const PresK pr = P.pres[F.imp0 + j];
    float v = pre_val(P, F.imp0 + j);
    if (pr.q2n != 0) v *= ipow(vp.q2, pr.q2n);
    if (pr.invq != 0) {
      bool nz = F.dynamic ? (vp.kx > 0 || vp.ky > 0) : !vp.origin;
      const float iq = nz ? 1.0f / sqrtf(vp.q2) : 0.f;
      v *= ipow(iq, pr.invq);
    }
    if (F.dynamic) acc -= P.dt * v;
    else acc += v;
  }
  return acc;
}

__device__ __forceinline__ float noise_amp(const LineParams& P, int fi, const VPoint& vp) {
  const FieldK& F = P.f[fi];
  float a = noise_base_val(P, fi);
  if (F.noise_q2n != 0) a *= sqrtf(ipow(vp.q2, F.noise_q2n));
  if (F.noise_invq != 0) {
    const float iq = vp.origin ? 0.f : 1.0f / sqrtf(vp.q2);
    a *= sqrtf(ipow(iq, F.noise_invq));
  }
  return a;
}

// Fourier-space white noise: the DFT of i.i.d. N(0,1) real noise, i.e. a Hermitian
// complex Gaussian field with Re, Im ~ N(0, N/2) per independent pair and N(0, N) on
// self-conjugate modes.  Counters (Philox4x32-10 key = seed, counter = (c, step, fid, 0)):
//  * modes 0 < kx < sx/2 (their partner has kx > sx/2): the line axis coordinate t
//    (z in 3D, y in 2D; none in 1D) is folded to t mod Lt/2; c = linear index
//    ((kz*sy + ky)*sx + kx) with t folded; words 0,1 serve t < Lt/2, words 2,3 the
//    mode at t + Lt/2 -- one generator call for two modes of the same thread;
//  * modes on the kx = 0 and kx = sx/2 planes: c = the smaller linear index of the
//    Hermitian pair (k, -k), words 0,1; the other member takes the conjugate.
__device__ __forceinline__ int line_axis_len(const Dims& d) {
  return d.sz > 1 ? d.sz : (d.sy > 1 ? d.sy : 1);
}

// Both modes (t, t + Lt/2) of a folded pair from its counter lin (see noise_pair).
__device__ __forceinline__ void noise_pair_lin(const LineParams& P, const NoiseKey& nk, int fid, uint32_t lin,
                                               float2& lo, float2& hi) {
  float g1, g2, g3, g4;
  philox_normal4(lin, nk.step, (uint32_t)fid, nk.key0, nk.key1, g1, g2, g3, g4);
  lo = make_float2(P.sqrtHalfN * g1, P.sqrtHalfN * g2);
  hi = make_float2(P.sqrtHalfN * g3, P.sqrtHalfN * g4);
}

// Both modes (t, t + Lt/2) of a folded pair, t < Lt/2, 0 < kx < sx/2.
__device__ __forceinline__ void noise_pair(const LineParams& P, const Dims& d, const NoiseKey& nk, int fid, int kx,
                                           int ky, int kz, float2& lo, float2& hi) {
  const uint32_t lin = ((uint32_t)kz * d.sy + ky) * d.sx + kx;
  float g1, g2, g3, g4;
  philox_normal4(lin, nk.step, (uint32_t)fid, nk.key0, nk.key1, g1, g2, g3, g4);
  lo = make_float2(P.sqrtHalfN * g1, P.sqrtHalfN * g2);
  hi = make_float2(P.sqrtHalfN * g3, P.sqrtHalfN * g4);
}

// Any mode with kx <= sx/2.
__device__ __forceinline__ float2 noise_at(const LineParams& P, const Dims& d, const NoiseKey& nk, int fid, int kx,
                                           int ky, int kz) {
  if (kx != 0 && 2 * kx != d.sx) {
    const int Lt = line_axis_len(d);
    if (Lt == 1) {
      float2 lo, hi;
      noise_pair(P, d, nk, fid, kx, ky, kz, lo, hi);
      return lo;
    }
    const int h = Lt / 2;
    int& t = (d.sz > 1) ? kz : ky;
    const bool upper = t >= h;
    if (upper) t -= h;
    float2 lo, hi;
    noise_pair(P, d, nk, fid, kx, ky, kz, lo, hi);
    return upper ? hi : lo;
  }
  const uint32_t lin = ((uint32_t)kz * d.sy + ky) * d.sx + kx;
  const int pky = neg_mod(ky, d.sy);
  const int pkz = neg_mod(kz, d.sz);
  const uint32_t plin = ((uint32_t)pkz * d.sy + pky) * d.sx + kx;
  uint32_t ctr = lin;
  bool conj = false;
  float g1, g2;
  if (plin < lin) {
    ctr = plin;
    conj = true;
  }
  philox_normal2(ctr, nk.step, (uint32_t)fid, nk.key0, nk.key1, g1, g2);
  if (plin == lin) return make_float2(P.sqrtN * g1, 0.f);
  return make_float2(P.sqrtHalfN * g1, conj ? -P.sqrtHalfN * g2 : P.sqrtHalfN * g2);
}

// Per-thread constants of the plain modes (kx' > 0) of one line along the last axis (z
// in 3D, y in 2D): every coordinate of the mode but the one along the line, which is
// m + C for register index i of thread m (C = pos_step2<L>(0, i) becomes a compile-time
// constant once the register loop unrolls, so the wrap, Nyquist and mask tests along the
// line reduce to one comparison of m with a constant).
struct LinePre {
  VPoint base;        // the fixed axes; the line axis is filled in per mode
  float fm;           // (float)m
  uint32_t lin0;      // noise counter of line position m
  uint32_t lin_step;  // noise counter increment per line position
};

template <bool Z3>
__device__ __forceinline__ LinePre line_pre(const LineParams& P, const Dims& d, int kx, int ky, int m) {
  LinePre lp;
  lp.base = make_vpoint(P, d, kx, Z3 ? ky : 0, 0);
  lp.fm = (float)m;
  if (Z3) {
    lp.lin0 = ((uint32_t)m * d.sy + ky) * d.sx + kx;
    lp.lin_step = (uint32_t)d.sy * d.sx;
  } else {
    lp.lin0 = (uint32_t)m * d.sx + kx;
    lp.lin_step = (uint32_t)d.sx;
  }
  return lp;
}

// The mode at line position m + C; the same values as make_vpoint (q is the exact
// float of the wrapped integer index times the step, as in q_of).
template <int L, bool Z3>
__device__ __forceinline__ VPoint line_vpoint(const LineParams& P, const LinePre& lp, int m, int C) {
  VPoint vp = lp.base;
  const bool wrap = (L > 1) && (C >= L / 2);
  const float q = (lp.fm + (float)(C - (wrap ? L : 0))) * (Z3 ? P.stepqz : P.stepqy);
  const bool ny = (L > 1) && (m == L / 2 - C);
  if (Z3) {
    vp.kz = m + C;
    vp.qz = q;
    vp.nyz = ny;
  } else {
    vp.ky = m + C;
    vp.qy = q;
    vp.nyy = ny;
  }
  vp.origin = (vp.kx == 0 && vp.ky == 0 && vp.kz == 0);
  vp.q2 = vp.qx * vp.qx + vp.qy * vp.qy + vp.qz * vp.qz;
  return vp;
}

// dealias_k mask (src/field_kernels.cu:229-256): keep a mode iff |n| <= N/(order+1)
// on every axis, n = k or k - N for k > N/2.  The three limits are per-field
// constants (FieldK::chan_xlimit / chan_ylimit / chan_zlimit).
__device__ __forceinline__ bool keep_axis(int k, int n, int lim) {
  const int nk = (k > (n >> 1)) ? n - k : k;
  return nk <= lim;
}
__device__ __forceinline__ bool keep_point(const Dims& d, const VPoint& vp, const FieldK& F) {
  return keep_axis(vp.kx, d.sx, F.chan_xlimit) && keep_axis(vp.ky, d.sy, F.chan_ylimit) &&
         keep_axis(vp.kz, d.sz, F.chan_zlimit);
}
// keep_axis along a line of length L at position m + C (see LinePre): positions below
// L/2 are m + C, the others L - m - C.
template <int L>
__device__ __forceinline__ bool keep_line(int m, int C, int lim) {
  if (L == 1) return true;
  return (C < L / 2) ? (m <= lim - C) : (m >= L - C - lim);
}

// Unpacks component `which` (0: kx = 0 plane, 1: kx = sx/2 plane) of a packed value.
__device__ __forceinline__ float2 unpack(float2 z, float2 zp, int which) {
  const float2 zc = c_conj(zp);
  if (which == 0) return c_scale(c_add(z, zc), 0.5f);
  return c_scale(c_mulmi(c_sub(z, zc)), 0.5f);
}

}  // namespace cupssgb
