// Turnaround kernel of one phase: forward FFT of the product channels along the line
// axis, Fourier-space update of every field of the phase, inverse FFT of the
// dealiased copies.  Fused form of, per field, the reference's term product FFT +
// applyPres_vector_pre_k + setDynamic_k / setNotDynamic_k + dealias_k + normalize_k +
// the line-axis part of the inverse transforms (src/term.cpp:12-25,
// src/field.cpp:25-92, src/field_kernels.cu:115-256, src/term_kernels.cu:221-240).
//
// The per-point arithmetic is a policy `Prog`:
//   template <class Fetch> static float2 eval(const LineParams&, int fi, const VPoint&,
//                                              const Fetch&)
// returns the new value of phase field fi at one (virtual) mode.  InterpProg walks
// the term / prefactor tables of the parameter block; the engine can instead compile
// a program generated for the system's equations (straight-line code, same tables
// for the numerical values).
//
// Shared-memory slots (each NL * PL * W float2):
//   [0, n_prod)                 forward-transformed products (step-2 positions)
//   [n_prod, n_prod+src_slots)  prefetched states read by the field being updated
//   [n_prod+src_slots]          dealiased copy being inverse-transformed
#pragma once
#include "engine_types.h"
#include "fft.cuh"
#include "line_geom.cuh"
#include "point_math.cuh"

namespace cupssgb {

// Source access at one mode: self and Hermitian-partner shared-memory addresses;
// wsel >= 0 selects the unpacked component on the packed column.
// States come either from prefetch slots (src_direct == false) or straight from the
// phase-start state arrays at global elements es / ep.  xi is the Fourier-space noise
// sample of the mode (used by noisy fields).
struct Fetch {
  const float2* smem;
  size_t slot_sz, as, ap;
  int n_prod, wsel;
  bool src_direct;
  const float2* const* states;   // P.state
  const int* srcs;               // F.src
  size_t es, ep;
  float2 xi;
  __device__ __forceinline__ float2 get(int slot) const {
    const float2* S = smem + (size_t)slot * slot_sz;
    if (wsel < 0) return S[as];
    return unpack(S[as], S[ap], wsel);
  }
  __device__ __forceinline__ float2 prod(int c) const { return get(c); }
  __device__ __forceinline__ float2 src(int j) const {
    if (!src_direct) return get(n_prod + j);
    const float2* st = states[srcs[j]];
    if (wsel < 0) return st[es];
    return unpack(st[es], st[ep], wsel);
  }
};

struct InterpProg {
  static constexpr bool kUnroll = false;
  template <class F>
  __device__ __forceinline__ static float2 eval(const LineParams& P, int fi, const VPoint& vp, const F& fx) {
    const FieldK& K = P.f[fi];
    float2 acc = make_float2(0.f, 0.f);
    for (int t = 0; t < K.nterms; ++t) {
      const TermK T = P.term[K.term0 + t];
      float2 src;
      if (T.kind == kTermProduct) {
        src = fx.prod(T.src);
      } else if (T.kind == kTermSingle) {
        src = fx.src(T.src);
      } else {
        // empty product: FFT of the all-ones field is N at q = 0
        src = vp.origin ? make_float2((float)P.sx * (float)P.sy * (float)P.sz, 0.f) : make_float2(0.f, 0.f);
      }
      float2 c = c_scale(src, term_mult(P, T, vp));
      if (T.s) c = c_muli(c);
      acc = c_add(acc, c);
    }
    float2 nv;
    if (K.dynamic) {
      nv = c_add(fx.src(K.self_src), c_scale(acc, P.dt));
      if (K.noisy) nv = c_add(nv, c_scale(fx.xi, noise_amp(P, fi, vp)));
      if (K.nimp > 0) {
        const float rd = 1.0f / implicit_factor(P, K, vp);
        nv = make_float2(nv.x * rd, nv.y * rd);
      }
    } else {
      nv = (K.nterms > 0) ? acc : fx.src(K.self_src);
      if (K.noisy) {
        const float2 nz = c_scale(fx.xi, noise_amp(P, fi, vp));
        nv = (K.nterms > 0) ? c_add(nv, nz) : nz;
      }
      if (K.nimp > 0 && !vp.origin) {
        const float rd = 1.0f / implicit_factor(P, K, vp);
        nv = make_float2(nv.x * rd, nv.y * rd);
      }
    }
    return nv;
  }
};

// One plain (kx' > 0) mode: register index i of the thread's step-2 positions.
template <int L, class Prog, class G>
__device__ __forceinline__ void update_mode(const LineParams& P, const FieldK& F, int fi, const G& g, int i,
                                            bool z3, const float2* smem, size_t slot_sz, float2* Cs,
                                            bool has_chan, float2 xi) {
  const int pos = pos_step2<L>(g.m, i);
  Fetch fx;
  fx.smem = smem;
  fx.slot_sz = slot_sz;
  fx.as = g.sidx(g.l, pos);
  fx.ap = fx.as;
  fx.n_prod = P.n_prod;
  fx.wsel = -1;
  fx.src_direct = false;
  fx.states = P.state;
  fx.srcs = F.src;
  fx.es = g.mbase + g.elem(pos);
  fx.ep = fx.es;
  fx.xi = xi;
  const VPoint vp = make_vpoint(P, g.kxp, z3 ? g.lineky : pos, z3 ? pos : 0);
  const float2 z = Prog::eval(P, fi, vp, fx);
  g.at(F.next)[g.elem(pos)] = z;
  if (has_chan) Cs[fx.as] = keep_point(P, vp, F) ? c_scale(z, P.invN) : make_float2(0.f, 0.f);
}

template <int L, int NL, class Prog>
__device__ __forceinline__ void turn_body(const LineParams& P) {
  constexpr int R = LineCfg<L>::R;
  extern __shared__ float2 smem[];
  NoiseKey nk{P.key0, P.key1, P.step};
  if (P.members) {
    const MemberK mk = P.members[blockIdx.z];
    if (!mk.active) return;   // CTA-uniform, before any barrier
    nk = NoiseKey{mk.key0, mk.key1, mk.step + P.step_off};
  }
  const LineGeom<L, NL> g(P);
  const int m = g.m, l = g.l;
  const size_t slot_sz = g.slot_sz;
  const int sy = P.sy;
  const bool z3 = (P.geo == kGeoZ3);
  float2 v[R];

  // 1) forward transform of every product channel into its slot (step-2 positions)
  for (int c = 0; c < P.n_prod; ++c) {
    float2* Sl = smem + (size_t)c * slot_sz;
    const float2* in = g.at(P.prod_in[c]);
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = g.ok ? in[g.elem(pos_step1<L>(m, r))] : make_float2(0.f, 0.f);
    fwd_step1<L>(v, m, P.tw);
#pragma unroll
    for (int s = 0; s < R; ++s) Sl[g.sidx(l, pos_t1<L>(m, s))] = v[s];
    __syncthreads();
#pragma unroll
    for (int i = 0; i < R; ++i) v[i] = Sl[g.sidx(l, pos_t2<L>(m, i))];
    fwd_step2<L>(v);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < R; ++i) Sl[g.sidx(l, pos_step2<L>(m, i))] = v[i];
  }

  float2* Cs = smem + (size_t)(P.n_prod + P.src_slots) * slot_sz;
  for (int fi = 0; fi < P.nf; ++fi) {
    const FieldK& F = P.f[fi];
    const bool has_chan = (F.chan != nullptr);
    // 2a) table-driven program: prefetch every state the update reads, all R points of
    //     the thread at once (generated programs load them directly, unrolled)
    for (int j = 0; j < F.nsrc; ++j) {
      float2* Sj = smem + (size_t)(P.n_prod + j) * slot_sz;
      const float2* st = g.at(P.state[F.src[j]]);
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const int pos = pos_step2<L>(m, i);
        Sj[g.sidx(l, pos)] = g.ok ? st[g.elem(pos)] : make_float2(0.f, 0.f);
      }
    }
    __syncthreads();
    // 2b) pointwise update.  Columns kx' > 0: plain half-spectrum modes; with a
    // generated program (Prog::kUnroll) the R points are unrolled so that their
    // independent arithmetic (noise draws included) overlaps.
    const int pl = (NL == 2 && sy > 1 && blockIdx.y != 0) ? (l ^ 1) : l;
    if (g.ok && g.kxp != 0) {
      if constexpr (Prog::kUnroll) {
        // Fourier noise of the thread's R modes, drawn in (t, t + Lt/2) pairs
        float2 xi[R];
#pragma unroll
        for (int i = 0; i < R; ++i) xi[i] = make_float2(0.f, 0.f);
        if (F.noisy) {
          constexpr int Mx = LineCfg<L>::M;
          constexpr int HALF = (Mx >= 2) ? Mx / 2 : R / 2;   // register offset of t + L/2
#pragma unroll
          for (int i = 0; i < R; ++i) {
            const int kp = (Mx >= 2) ? (i % Mx) : (i / Mx);
            const bool lower = (L == 1) || ((Mx >= 2) ? (kp < Mx / 2) : (kp < R / 2));
            if (lower) {
              const int pos = pos_step2<L>(m, i);
              float2 lo, hi;
              if (z3) noise_pair(P, nk, F.fid, g.kxp, g.lineky, pos, lo, hi);
              else noise_pair(P, nk, F.fid, g.kxp, pos, 0, lo, hi);
              xi[i] = lo;
              if (L > 1) xi[i + HALF] = hi;
            }
          }
        }
#pragma unroll
        for (int i = 0; i < R; ++i)
          update_mode<L, Prog>(P, F, fi, g, i, z3, smem, slot_sz, Cs, has_chan, xi[i]);
      } else {
#pragma unroll 1
        for (int i = 0; i < R; ++i) {
          float2 xi = make_float2(0.f, 0.f);
          if (F.noisy) {
            const int pos = pos_step2<L>(m, i);
            xi = z3 ? noise_at(P, nk, F.fid, g.kxp, g.lineky, pos) : noise_at(P, nk, F.fid, g.kxp, pos, 0);
          }
          update_mode<L, Prog>(P, F, fi, g, i, z3, smem, slot_sz, Cs, has_chan, xi);
        }
      }
    } else if (g.ok) {
      // packed column kx' = 0: the kx = 0 and kx = sx/2 planes, unpacked with the
      // Hermitian partner (-ky, -kz)
#pragma unroll 1
      for (int i = 0; i < R; ++i) {
        const int pos = pos_step2<L>(m, i);
        const int ky = z3 ? g.lineky : pos;
        const int kz = z3 ? pos : 0;
        const int ppos = (L - pos) & (L - 1);
        Fetch fx;
        fx.smem = smem;
        fx.slot_sz = slot_sz;
        fx.as = g.sidx(l, pos);
        fx.ap = g.sidx(pl, ppos);
        fx.n_prod = P.n_prod;
        fx.src_direct = false;
        fx.states = P.state;
        fx.srcs = F.src;
        fx.es = g.mbase + g.elem(pos);
        if (z3) fx.ep = g.mbase + (size_t)((sy - ky) & (sy - 1)) * P.Lx + (size_t)ppos * g.pstride;
        else fx.ep = g.mbase + g.elem(ppos);
        fx.wsel = 0;
        const VPoint v0 = make_vpoint(P, 0, ky, kz);
        fx.xi = F.noisy ? noise_at(P, nk, F.fid, 0, ky, kz) : make_float2(0.f, 0.f);
        const float2 o0 = Prog::eval(P, fi, v0, fx);
        fx.wsel = 1;
        const VPoint v1 = make_vpoint(P, P.sx / 2, ky, kz);
        fx.xi = F.noisy ? noise_at(P, nk, F.fid, P.sx / 2, ky, kz) : make_float2(0.f, 0.f);
        const float2 o1 = Prog::eval(P, fi, v1, fx);
        const float2 z = c_add(o0, c_muli(o1));
        const float2 a = (has_chan && keep_point(P, v0, F)) ? c_scale(o0, P.invN) : make_float2(0.f, 0.f);
        const float2 b = (has_chan && keep_point(P, v1, F)) ? c_scale(o1, P.invN) : make_float2(0.f, 0.f);
        g.at(F.next)[g.elem(pos)] = z;
        if (has_chan) Cs[g.sidx(l, pos)] = c_add(a, c_muli(b));
      }
    }
    // 2c) inverse transform of the dealiased copy
    bool skip = !has_chan || g.kx0 > F.chan_xlimit;
    if (z3 && NL == 2) {
      // both lines of pair p >= 1 have |n_y| = p; pair 0 holds n_y = 0
      const int pr = (int)blockIdx.y;
      if (pr > 0 && pr > F.chan_ylimit) skip = true;
    }
    __syncthreads();   // Cs written; prefetch slots free for the next field
    if (skip) continue;   // CTA-uniform: masked tile, the channel stays zero
#pragma unroll
    for (int i = 0; i < R; ++i) v[i] = Cs[g.sidx(l, pos_step2<L>(m, i))];
    inv_step2<L>(v);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < R; ++i) Cs[g.sidx(l, pos_t2<L>(m, i))] = v[i];
    __syncthreads();
#pragma unroll
    for (int s = 0; s < R; ++s) v[s] = Cs[g.sidx(l, pos_t1<L>(m, s))];
    inv_step1<L>(v, m, P.tw);
    if (g.ok) {
#pragma unroll
      for (int r = 0; r < R; ++r) g.at(F.chan)[g.elem(pos_step1<L>(m, r))] = v[r];
    }
    __syncthreads();   // Cs free for the next field
  }
}

template <int L, int NL>
__global__ void __launch_bounds__(256, 2) turn_pass(const LineParams P) {
  turn_body<L, NL, InterpProg>(P);
}

}  // namespace cupssgb
