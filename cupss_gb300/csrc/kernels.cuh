// CUDA kernels of the pseudospectral step (sm_103a).
//
//  row_pass<Lx>   : per x-row, packed inverse real FFT of every real-space input,
//                   pointwise products, packed forward real FFT of every product.
//                   (the fused form of computeProduct_k + the product term FFT,
//                   src/term_kernels.cu:48-70, src/term.cpp:48-64, and the x part of
//                   the C2C transforms of src/field.cpp:247-273)
//  line_pass<L,NL>: along the last (y in 1D/2D, z in 3D) or middle axis; in turnaround
//                   mode it does the forward FFT of the product channels, the
//                   Fourier-space update of every field of the phase (setDynamic_k /
//                   setNotDynamic_k, src/field_kernels.cu:130-227, with the term
//                   prefactors of applyPres_vector_pre_k, src/term_kernels.cu:221-240,
//                   evaluated in registers), Fourier-space Philox noise, the dealias
//                   mask (dealias_k, :229-256) and 1/N normalisation (normalize_k,
//                   :115-128), and the inverse FFT of the dealiased copies.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "engine_types.h"
#include "fft.cuh"
#include "philox.cuh"

namespace cupssgb {

// ------------------------------------------------------------------------------------
// row pass (x axis, contiguous rows)
// ------------------------------------------------------------------------------------
// C2R pre-processing: packed P -> Z = E' + i O' with E' = X[k] + conj X[Lx-k],
// O' = (X[k] - conj X[Lx-k]) W_sx^{-k};  z = IDFT_Lx(Z) gives z[n] = r[2n] + i r[2n+1]
// of the unnormalised inverse real DFT.
__device__ __forceinline__ float2 c2r_pre(float2 a, float2 bm, int k, int sx, const float2* tw) {
  if (k == 0) {
    return make_float2(a.x + a.y, a.x - a.y);
  }
  float2 b = c_conj(bm);
  float2 e = c_add(a, b);
  float2 o = c_mulc(c_sub(a, b), tw_load(tw, sx, k));
  return c_add(e, c_muli(o));
}
// R2C post-processing: Z = DFT_Lx(z) -> packed P.
__device__ __forceinline__ float2 r2c_post(float2 zk, float2 zm, int k, int sx, const float2* tw) {
  if (k == 0) {
    return make_float2(zk.x + zk.y, zk.x - zk.y);
  }
  float2 zc = c_conj(zm);
  float2 e = c_scale(c_add(zk, zc), 0.5f);
  float2 o = c_scale(c_mulmi(c_sub(zk, zc)), 0.5f);
  return c_add(e, c_mul(tw_load(tw, sx, k), o));
}

template <int LX>
struct RowCfg {
  static constexpr int M = LineCfg<LX>::M;
  static constexpr int R = LineCfg<LX>::R;
  static constexpr int PL = padded_len<LX>() + 1;   // padded row length in smem
  static constexpr int RW = (M >= 128) ? 1 : (128 / M > 32 ? 32 : 128 / M);   // rows per CTA
};

// smem: (1 + n_in) slots of RW*PL float2.  Slot 0 is the transpose buffer.
template <int LX>
__global__ void __launch_bounds__(RowCfg<LX>::M * RowCfg<LX>::RW)
row_pass(const XParams p) {
  using C = RowCfg<LX>;
  constexpr int M = C::M, R = C::R, PL = C::PL, RW = C::RW;
  extern __shared__ float2 smem[];
  const int m = threadIdx.x;
  const int rl = threadIdx.y;
  const int row = blockIdx.x * RW + rl;
  const bool live = row < p.rows;
  const int sx = 2 * LX;
  float2* T = smem + rl * PL;
  auto slot = [&](int i) { return smem + (size_t)(1 + i) * RW * PL + rl * PL; };
  const size_t rowoff = (size_t)(live ? row : 0) * LX;
  float2 v[R];

  for (int c = 0; c < p.n_in; ++c) {
    float2* V = slot(c);
    if (p.in_mode == kXInReal) {
      const float2* in = p.in[c] + rowoff;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int n = pos_step1<LX>(m, r);
        V[pad_pos<LX>(n)] = live ? in[n] : make_float2(0.f, 0.f);
      }
      continue;
    }
    const float2* in = p.in[c] + rowoff;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int k = pos_step2<LX>(m, i);
      float2 a = live ? in[k] : make_float2(0.f, 0.f);
      float2 b = live ? in[(LX - k) & (LX - 1)] : make_float2(0.f, 0.f);
      v[i] = c2r_pre(a, b, k, sx, p.tw);
    }
    inv_step2<LX>(v);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < R; ++i) T[pad_pos<LX>(pos_t2<LX>(m, i))] = v[i];
    __syncthreads();
#pragma unroll
    for (int s = 0; s < R; ++s) v[s] = T[pad_pos<LX>(pos_t1<LX>(m, s))];
    inv_step1<LX>(v, m, p.tw);
#pragma unroll
    for (int r = 0; r < R; ++r) V[pad_pos<LX>(pos_step1<LX>(m, r))] = v[r];
  }

  for (int q = 0; q < p.n_prod; ++q) {
    // pointwise product of the real values (packed as pairs r[2n], r[2n+1])
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int a = pad_pos<LX>(pos_step1<LX>(m, r));
      float2 acc = make_float2(1.f, 1.f);
      for (int t = 0; t < p.prod_n[q]; ++t) {
        float2 x = slot(p.prod_f[q][t])[a];
        acc.x *= x.x;
        acc.y *= x.y;
      }
      v[r] = acc;
    }
    if (p.out_mode != kXOutSpectral) {
      if (live) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const int n = pos_step1<LX>(m, r);
          const float2 z = c_scale(v[r], p.out_scale);
          if (p.out_mode == kXOutReal) {
            reinterpret_cast<float2*>(p.out[q])[rowoff + n] = z;
          } else {
            reinterpret_cast<float4*>(p.out[q])[rowoff + n] = make_float4(z.x, 0.f, z.y, 0.f);
          }
        }
      }
      continue;
    }
    fwd_step1<LX>(v, m, p.tw);
    __syncthreads();
#pragma unroll
    for (int s = 0; s < R; ++s) T[pad_pos<LX>(pos_t1<LX>(m, s))] = v[s];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < R; ++i) v[i] = T[pad_pos<LX>(pos_t2<LX>(m, i))];
    fwd_step2<LX>(v);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < R; ++i) T[pad_pos<LX>(pos_step2<LX>(m, i))] = v[i];
    __syncthreads();
    float2* out = reinterpret_cast<float2*>(p.out[q]) + rowoff;
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int k = pos_step2<LX>(m, i);
      const float2 zm = T[pad_pos<LX>((LX - k) & (LX - 1))];
      const float2 x = r2c_post(v[i], zm, k, sx, p.tw);
      if (live) out[k] = x;
    }
  }
}

// ------------------------------------------------------------------------------------
// line pass (strided axis)
// ------------------------------------------------------------------------------------
struct VPoint {
  int kx, ky, kz;
  bool origin, nyx, nyy, nyz;
  float qx, qy, qz, q2;
};

__device__ __forceinline__ float q_of(int k, int n, float step) {
  return (float)(k < (n + 1) / 2 ? k : k - n) * step;   // src/field_init.cpp:248-250
}

__device__ __forceinline__ VPoint make_vpoint(const LineParams& P, int kx, int ky, int kz) {
  VPoint vp;
  vp.kx = kx;
  vp.ky = ky;
  vp.kz = kz;
  vp.origin = (kx == 0 && ky == 0 && kz == 0);
  vp.nyx = (P.sx > 1) && (2 * kx == P.sx);
  vp.nyy = (P.sy > 1) && (2 * ky == P.sy);
  vp.nyz = (P.sz > 1) && (2 * kz == P.sz);
  vp.qx = q_of(kx, P.sx, P.stepqx);
  vp.qy = q_of(ky, P.sy, P.stepqy);
  vp.qz = q_of(kz, P.sz, P.stepqz);
  vp.q2 = vp.qx * vp.qx + vp.qy * vp.qy + vp.qz * vp.qz;
  return vp;
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
    float v = pr.pre;
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
    float v = pr.pre;
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

__device__ __forceinline__ float noise_amp(const FieldK& F, const VPoint& vp) {
  float a = F.noise_base;
  if (F.noise_q2n != 0) a *= sqrtf(ipow(vp.q2, F.noise_q2n));
  if (F.noise_invq != 0) {
    const float iq = vp.origin ? 0.f : 1.0f / sqrtf(vp.q2);
    a *= sqrtf(ipow(iq, F.noise_invq));
  }
  return a;
}

// Fourier-space white noise at full-grid point (kx <= sx/2, ky, kz): the DFT of
// i.i.d. N(0,1) real noise, generated per Hermitian pair from a Philox counter.
__device__ __forceinline__ float2 noise_at(const LineParams& P, int fid, int kx, int ky, int kz) {
  const uint32_t lin = ((uint32_t)kz * P.sy + ky) * P.sx + kx;
  uint32_t ctr = lin;
  bool conj = false, real_only = false;
  if (kx == 0 || 2 * kx == P.sx) {
    const int pky = (P.sy - ky) & (P.sy - 1);
    const int pkz = (P.sz - kz) & (P.sz - 1);
    const uint32_t plin = ((uint32_t)pkz * P.sy + pky) * P.sx + kx;
    if (plin == lin) real_only = true;
    else if (plin < lin) { ctr = plin; conj = true; }
  }
  float g1, g2;
  philox_normal2(ctr, P.step, (uint32_t)fid, P.key0, P.key1, g1, g2);
  if (real_only) return make_float2(P.sqrtN * g1, 0.f);
  return make_float2(P.sqrtHalfN * g1, conj ? -P.sqrtHalfN * g2 : P.sqrtHalfN * g2);
}

__device__ __forceinline__ bool keep_mode(int k, int n, int order) {
  int nk = (k > n / 2) ? k - n : k;
  if (nk < 0) nk = -nk;
  return nk <= n / (order + 1);
}
__device__ __forceinline__ bool keep_point(const LineParams& P, const VPoint& vp, int order) {
  return keep_mode(vp.kx, P.sx, order) && keep_mode(vp.ky, P.sy, order) && keep_mode(vp.kz, P.sz, order);
}

// Unpacks component `which` (0: kx = 0 plane, 1: kx = sx/2 plane) of a packed value.
__device__ __forceinline__ float2 unpack(float2 z, float2 zp, int which) {
  const float2 zc = c_conj(zp);
  if (which == 0) return c_scale(c_add(z, zc), 0.5f);
  return c_scale(c_mulmi(c_sub(z, zc)), 0.5f);
}

template <int L>
struct LineShape {
  static constexpr int M = LineCfg<L>::M;
  static constexpr int R = LineCfg<L>::R;
  static constexpr int PL = padded_len<L>();
};

// Grid: x = kx' tile (W columns), y = z (kGeoY3) / ky or ky-pair (kGeoZ3).
// Block: (W, M, NL).  smem: nslots * NL * PL * W float2.
template <int L, int NL>
__global__ void __launch_bounds__(512)
line_pass(const LineParams P) {
  using S = LineShape<L>;
  constexpr int M = S::M, R = S::R, PL = S::PL;
  extern __shared__ float2 smem[];
  const int W = P.W;
  const int w = threadIdx.x;
  const int m = threadIdx.y;
  const int l = threadIdx.z;
  const int kx0 = blockIdx.x * W;
  const int kxp = kx0 + w;
  const bool colok = kxp < P.Lx;
  const int Lx = P.Lx;

  // line geometry
  int lineky = 0, linez = 0;
  bool lineok = true;
  size_t lbase;
  size_t pstride;
  if (P.geo == kGeoCol) {
    lbase = kxp;
    pstride = Lx;
  } else if (P.geo == kGeoY3) {
    linez = blockIdx.y;
    lbase = (size_t)linez * P.sy * Lx + kxp;
    pstride = Lx;
  } else {
    if (NL == 2) {
      const int pr = blockIdx.y;
      if (l == 0) lineky = pr;
      else lineky = (pr == 0) ? P.sy / 2 : P.sy - pr;
      lineok = !(l == 1 && P.sy == 1);
    } else {
      lineky = blockIdx.y;
    }
    lbase = (size_t)lineky * Lx + kxp;
    pstride = (size_t)P.sy * Lx;
  }
  const bool ok = colok && lineok;
  auto elem = [&](int pos) { return lbase + (size_t)pos * pstride; };
  auto sidx = [&](int line, int pos) { return (size_t)(line * PL + pad_pos<L>(pos)) * W + w; };
  const size_t slot_sz = (size_t)NL * PL * W;
  float2 v[R];

  if (P.mode == kModeFwd || P.mode == kModeInv) {
    for (int c = 0; c < P.n_prod; ++c) {
      if (P.mode == kModeInv && kx0 > P.inv_xlimit[c]) continue;   // CTA-uniform
      float2* T = smem;
      const float2* in = P.prod_in[c];
      float2* out = P.prod_out[c];
      if (P.mode == kModeFwd) {
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = ok ? in[elem(pos_step1<L>(m, r))] : make_float2(0.f, 0.f);
        fwd_step1<L>(v, m, P.tw);
        __syncthreads();
#pragma unroll
        for (int s = 0; s < R; ++s) T[sidx(l, pos_t1<L>(m, s))] = v[s];
        __syncthreads();
#pragma unroll
        for (int i = 0; i < R; ++i) v[i] = T[sidx(l, pos_t2<L>(m, i))];
        fwd_step2<L>(v);
        if (ok) {
#pragma unroll
          for (int i = 0; i < R; ++i) out[elem(pos_step2<L>(m, i))] = v[i];
        }
      } else {
#pragma unroll
        for (int i = 0; i < R; ++i) v[i] = ok ? in[elem(pos_step2<L>(m, i))] : make_float2(0.f, 0.f);
        inv_step2<L>(v);
        __syncthreads();
#pragma unroll
        for (int i = 0; i < R; ++i) T[sidx(l, pos_t2<L>(m, i))] = v[i];
        __syncthreads();
#pragma unroll
        for (int s = 0; s < R; ++s) v[s] = T[sidx(l, pos_t1<L>(m, s))];
        inv_step1<L>(v, m, P.tw);
        if (ok) {
#pragma unroll
          for (int r = 0; r < R; ++r) out[elem(pos_step1<L>(m, r))] = v[r];
        }
      }
    }
    return;
  }

  // ---------------- turnaround ----------------
  // 1) forward transform of every product channel into its slot (step-2 positions)
  for (int c = 0; c < P.n_prod; ++c) {
    float2* Sl = smem + (size_t)c * slot_sz;
    const float2* in = P.prod_in[c];
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = ok ? in[elem(pos_step1<L>(m, r))] : make_float2(0.f, 0.f);
    fwd_step1<L>(v, m, P.tw);
#pragma unroll
    for (int s = 0; s < R; ++s) Sl[sidx(l, pos_t1<L>(m, s))] = v[s];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < R; ++i) v[i] = Sl[sidx(l, pos_t2<L>(m, i))];
    fwd_step2<L>(v);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < R; ++i) Sl[sidx(l, pos_step2<L>(m, i))] = v[i];
  }
  __syncthreads();

  // 2) per field: pointwise update (state -> next, dealiased copy -> channel slot),
  //    then the inverse transform of the dealiased copy.  The update reads only the
  //    phase-start states (ping-pong buffers) and the product slots, so the order of
  //    fields is immaterial.
  const int sy = P.sy;
  float2* Cs = smem + (size_t)P.n_prod * slot_sz;
  for (int fi = 0; fi < P.nf; ++fi) {
    const FieldK& F = P.f[fi];
    const bool has_chan = (F.chan != nullptr);
#pragma unroll 1
    for (int i = 0; i < R; ++i) {
      if (!ok) break;
      const int pos = pos_step2<L>(m, i);
      int ky, kz;
      if (P.geo == kGeoZ3) { ky = lineky; kz = pos; } else { ky = pos; kz = 0; }
      const int ppos = (L - pos) & (L - 1);
      // partner line in smem: pair p >= 1 holds {p, sy-p}; pair 0 holds {0, sy/2},
      // each of which is its own partner under ky -> -ky
      const int pl = (NL == 2 && sy > 1 && blockIdx.y != 0) ? (l ^ 1) : l;
      const size_t es = elem(pos);
      size_t ep;   // partner element, used on the packed column kx' = 0 only
      if (P.geo == kGeoZ3) {
        const int pky = (sy - ky) & (sy - 1);
        ep = (size_t)pky * Lx + kxp + (size_t)ppos * pstride;
      } else {
        ep = elem(ppos);
      }
      const size_t as = sidx(l, pos), ap = sidx(pl, ppos);
      const bool packed = (kxp == 0);
      const int nvp = packed ? 2 : 1;
      float2 outv0 = make_float2(0.f, 0.f), outv1 = make_float2(0.f, 0.f);
      bool keep0 = false, keep1 = false;
      for (int which = 0; which < nvp; ++which) {
        const int kx = packed ? (which == 0 ? 0 : P.sx / 2) : kxp;
        const VPoint vp = make_vpoint(P, kx, ky, kz);
        const int wsel = packed ? which : -1;
        auto fetch_state = [&](const float2* st) {
          const float2 z = st[es];
          if (wsel < 0) return z;
          return unpack(z, st[ep], wsel);
        };
        float2 acc = make_float2(0.f, 0.f);
        for (int t = 0; t < F.nterms; ++t) {
          const TermK T = P.term[F.term0 + t];
          float2 src;
          if (T.kind == kTermProduct) {
            const float2* Sl = smem + (size_t)T.src * slot_sz;
            src = (wsel < 0) ? Sl[as] : unpack(Sl[as], Sl[ap], wsel);
          } else if (T.kind == kTermSingle) {
            src = fetch_state(P.state[T.src]);
          } else {
            // empty product: FFT of the all-ones field is N at q = 0
            src = (vp.origin) ? make_float2((float)P.sx * (float)P.sy * (float)P.sz, 0.f)
                              : make_float2(0.f, 0.f);
          }
          const float mlt = term_mult(P, T, vp);
          float2 c = c_scale(src, mlt);
          if (T.s) c = c_muli(c);
          acc = c_add(acc, c);
        }
        float2 nv;
        if (F.dynamic) {
          nv = fetch_state(F.cur);
          nv = c_add(nv, c_scale(acc, P.dt));
          if (F.noisy) nv = c_add(nv, c_scale(noise_at(P, F.fid, kx, ky, kz), noise_amp(F, vp)));
          if (F.nimp > 0) {
            const float d = implicit_factor(P, F, vp);
            nv = make_float2(nv.x / d, nv.y / d);
          }
        } else {
          nv = (F.nterms > 0) ? acc : fetch_state(F.cur);
          if (F.noisy) {
            const float2 nz = c_scale(noise_at(P, F.fid, kx, ky, kz), noise_amp(F, vp));
            nv = (F.nterms > 0) ? c_add(nv, nz) : nz;
          }
          if (F.nimp > 0 && !vp.origin) {
            const float d = implicit_factor(P, F, vp);
            nv = make_float2(nv.x / d, nv.y / d);
          }
        }
        const bool kp = has_chan && keep_point(P, vp, F.order);
        if (which == 0) { outv0 = nv; keep0 = kp; } else { outv1 = nv; keep1 = kp; }
      }
      float2 z, zc;
      if (packed) {
        z = c_add(outv0, c_muli(outv1));
        const float2 a = keep0 ? c_scale(outv0, P.invN) : make_float2(0.f, 0.f);
        const float2 b = keep1 ? c_scale(outv1, P.invN) : make_float2(0.f, 0.f);
        zc = c_add(a, c_muli(b));
      } else {
        z = outv0;
        zc = keep0 ? c_scale(outv0, P.invN) : make_float2(0.f, 0.f);
      }
      F.next[es] = z;
      if (has_chan) Cs[as] = zc;
    }
    if (!has_chan) continue;
    bool skip = kx0 > F.chan_xlimit;
    if (P.geo == kGeoZ3 && NL == 2) {
      // both lines of pair p >= 1 have |n_y| = p; pair 0 holds n_y = 0
      const int pr = (int)blockIdx.y;
      if (pr > 0 && pr > F.chan_ylimit) skip = true;
    }
    if (skip) continue;   // CTA-uniform: masked tile, the channel stays zero
    __syncthreads();      // all own-position writes of Cs done (and previous readers)
#pragma unroll
    for (int i = 0; i < R; ++i) v[i] = Cs[sidx(l, pos_step2<L>(m, i))];
    inv_step2<L>(v);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < R; ++i) Cs[sidx(l, pos_t2<L>(m, i))] = v[i];
    __syncthreads();
#pragma unroll
    for (int s = 0; s < R; ++s) v[s] = Cs[sidx(l, pos_t1<L>(m, s))];
    inv_step1<L>(v, m, P.tw);
    if (ok) {
#pragma unroll
      for (int r = 0; r < R; ++r) F.chan[elem(pos_step1<L>(m, r))] = v[r];
    }
    __syncthreads();      // Cs free for the next field
  }
}

// Packed half spectrum -> reference-layout full complex spectrum.
__global__ void expand_spectrum(const ExpandParams p);

}  // namespace cupssgb
