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
//   [n_prod, n_prod+src_slots)  states read by the field being updated, copied in
//                               asynchronously (cp.async) while earlier work runs
//   tslot                       transpose buffer of the inverse transform of the dealiased
//                               copy: slot 0 when the phase has one field (every read of
//                               the other slots is done by then), else a slot of its own
//                               so that the next field's states can be copied in meanwhile.
// The dealiased copy itself stays in registers between the update and its inverse
// transform.
#pragma once
#include "engine_types.h"
#include "fft.cuh"
#include "line_geom.cuh"
#include "point_math.cuh"

namespace cupssgb {

// Issues the copies of every state field F reads into its prefetch slots, at the
// thread's step-2 positions (zeros outside the grid).
template <int L, bool SP, class G>
__device__ __forceinline__ void prefetch_states(const LineParams& P, const FieldK& F, const G& g, float2* smem,
                                                int n_prod, int slot_sz) {
  constexpr int R = LineCfg<L, SP>::R;
  const unsigned sbase = smem_u32(smem) + 8u * (unsigned)g.sidx(g.l, 0);
  for (int j = 0; j < F.nsrc; ++j) {
    const unsigned sj = sbase + 8u * (unsigned)((n_prod + j) * slot_sz);
    const float2* st = g.at(P.state[F.src[j]]);
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int pos = pos_step2<L, SP>(g.m, i);
      const unsigned off = 8u * (unsigned)(g.sidx(g.l, pos) - g.sidx(g.l, 0));
      cp_async8(sj + off, g.ok ? st + g.elem(pos) : st, g.ok ? 8 : 0);
    }
  }
  cp_async_commit();
}

// Source access at one mode: self and Hermitian-partner shared-memory indices; wsel >= 0
// selects the unpacked component on the packed column.  xi is the Fourier-space noise
// sample of the mode (used by noisy fields).
struct Fetch {
  const float2* smem;
  int slot_sz, as, ap;
  int n_prod, wsel;
  float2 xi;
  bool p0_reg;   // product 0 of this mode is p0 (kept in registers), not in its slot
  float2 p0;
  __device__ __forceinline__ float2 get(int slot) const {
    const float2* S = smem + slot * slot_sz;
    if (wsel < 0) return S[as];
    return unpack(S[as], S[ap], wsel);
  }
  __device__ __forceinline__ float2 prod(int c) const { return (p0_reg && c == 0) ? p0 : get(c); }
  __device__ __forceinline__ float2 src(int j) const { return get(n_prod + j); }
};

struct InterpProg {
  static constexpr bool kUnroll = false;
  template <class F>
  __device__ __forceinline__ static float2 eval(const LineParams& P, int fi, const VPoint& vp, const F& fx) {
    const FieldK& K = P.f[fi];
    float2 acc = make_float2(0.f, 0.f);
    for (int t = 0; t < K.nterms; ++t) {
      const TermK T = P.term[K.term0 + t];
      if (T.kind == kTermMerged) continue;   // in another term's product channel
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

// Structure of the phase a kernel is compiled for.  The table-driven kernel reads it
// from the parameter block (zeros here); a generated program fixes the number of fields
// of the phase and the grid sizes at compile time, so the field loop unrolls (static
// parameter offsets) and every index expression of the per-mode math folds.
struct RtSpec {
  static constexpr int kNF = 0;
  static constexpr int kNProd = -1;   // product channels (-1: P.n_prod)
  static constexpr int kSX = 0, kSY = 0, kSZ = 0;
  static constexpr int kW = 0;   // tile width (0: P.W)
  // lines of 512 and 1024 points in the split FFT form (more threads per line)
  static constexpr bool kSplit = false;
  // draw the first field's noise while the first product's loads are in flight (pays off
  // when those loads come from HBM; for grids whose arrays stay in L2 it only delays the
  // transform)
  static constexpr bool kEarlyNoise = false;
};

// One plain (kx' > 0) mode: register index i of the thread's step-2 positions.  Writes
// the new state and returns the dealiased, 1/N-scaled copy of the mode (zero when masked
// or when the field has no dealiased copy).
// Fourier noise of a thread's R plain modes of one line, drawn in (t, t + Lt/2) pairs
// (one generator call per pair).
// The lower registers (positions t < L/2) in order: register of pair p.
template <int L, bool SP>
__host__ __device__ constexpr int lower_reg(int p) {
  constexpr int Mx = LineCfg<L, SP>::M;
  if (L == 1) return 0;
  if (LineCfg<L, SP>::kSplit || Mx < 2) return p;
  return (p / (Mx / 2)) * Mx + p % (Mx / 2);
}
// Register offset of position t + L/2 from the register of position t.
template <int L, bool SP>
__host__ __device__ constexpr int upper_half_reg() {
  constexpr int Mx = LineCfg<L, SP>::M;
  return (LineCfg<L, SP>::kSplit || Mx < 2) ? LineCfg<L, SP>::R / 2 : Mx / 2;
}

template <int L, bool SP>
__device__ __forceinline__ void draw_line_noise(const LineParams& P, const NoiseKey& nk, int fid, const LinePre& lp,
                                                float2 (&xi)[LineCfg<L, SP>::R]) {
  constexpr int R = LineCfg<L, SP>::R;
  constexpr int HALF = upper_half_reg<L, SP>();   // register offset of t + L/2
  constexpr int NP = (L == 1) ? 1 : R / 2;            // generator calls: one per pair
  uint32_t c[NP][4];
#pragma unroll
  for (int q = 0; q < NP; ++q) {
    c[q][0] = lp.lin0 + (uint32_t)pos_step2<L, SP>(0, lower_reg<L, SP>(q)) * lp.lin_step;
    c[q][1] = nk.step;
    c[q][2] = (uint32_t)fid;
    c[q][3] = 0u;
  }
  philox4x32_10_batch<NP>(c, nk.key0, nk.key1);
#pragma unroll
  for (int q = 0; q < NP; ++q) {
    const int i = lower_reg<L, SP>(q);
    float g1, g2, g3, g4;
    box_muller(c[q][0], c[q][1], g1, g2);
    box_muller(c[q][2], c[q][3], g3, g4);
    xi[i] = make_float2(P.sqrtHalfN * g1, P.sqrtHalfN * g2);
    if (L > 1) xi[i + HALF] = make_float2(P.sqrtHalfN * g3, P.sqrtHalfN * g4);
  }
}

// keep_fixed: the dealias test of the axes other than the line axis (per thread and field).
template <int L, bool SP, bool Z3, class Prog, class G>
__device__ __forceinline__ float2 update_mode(const LineParams& P, const LinePre& lp, const FieldK& F, int fi,
                                              const G& g, int i, const float2* smem, int n_prod, bool has_chan,
                                              bool keep_fixed, float2 xi, bool p0_reg = false,
                                              float2 p0 = float2{0.f, 0.f}) {
  const int C = pos_step2<L, SP>(0, i);
  const int pos = g.m + C;
  Fetch fx;
  fx.smem = smem;
  fx.slot_sz = g.slot_sz;
  fx.as = g.sidx(g.l, pos);
  fx.ap = fx.as;
  fx.n_prod = n_prod;
  fx.wsel = -1;
  fx.xi = xi;
  fx.p0_reg = p0_reg;
  fx.p0 = p0;
  const VPoint vp = line_vpoint<L, Z3>(P, lp, g.m, C);
  const float2 z = Prog::eval(P, fi, vp, fx);
  g.at(F.next)[g.elem(pos)] = z;
  const bool keep = keep_fixed && keep_line<L>(g.m, C, Z3 ? F.chan_zlimit : F.chan_ylimit);
  return (has_chan && keep) ? c_scale(z, P.invN) : make_float2(0.f, 0.f);
}

// The turnaround of the CTA at tile (tx, ty), thread (tw, tm, tl) -- blockIdx.x/y and
// threadIdx in a plain launch (turn_body); the batch member is blockIdx.z either way.
template <int L, int NL, class Prog, class Spec = RtSpec>
__device__ __forceinline__ void turn_body_at(const LineParams& P, int tx, int ty, int tw, int tm, int tl) {
  constexpr bool SP = Spec::kSplit;
  constexpr int R = LineCfg<L, SP>::R;
  constexpr bool Z3 = (NL == 2);   // the paired z-line form is the 3D turnaround
  extern __shared__ float2 smem[];
  grid_dep_sync();
  NoiseKey nk{P.key0, P.key1, P.step};
  if (P.members) {
    const MemberK mk = P.members[blockIdx.z];
    if (!mk.active) return;   // CTA-uniform, before any barrier
    nk = NoiseKey{mk.key0, mk.key1, mk.step + P.step_off};
  }
  const Dims d = Spec::kSX ? Dims{Spec::kSX, Spec::kSY, Spec::kSZ} : dims_of(P);
  const LineGeom<L, NL, Spec::kW, SP> g(P, d.sy, d.sx / 2, tx, ty, tw, tm, tl);
  if (g.idle) return;   // CTA-uniform, before any barrier
  const int m = g.m, l = g.l;
  const int slot_sz = g.slot_sz;
  const int sy = d.sy;
  const int nf = Spec::kNF ? Spec::kNF : P.nf;
  const int n_prod = Spec::kNProd >= 0 ? Spec::kNProd : P.n_prod;
  float2 v[R];

  // 0) the states the first field reads start on their way to shared memory now, and
  //    arrive while the products are transformed
  if (nf > 0) prefetch_states<L, SP>(P, P.f[0], g, smem, n_prod, slot_sz);

  // 1) forward transform of every product channel into its slot (step-2 positions).
  //    The first field's Fourier noise depends on no data: with a generated program it is
  //    drawn while the first product's loads are in flight.
  const bool plain = g.ok && g.kxp != 0;
  float2 xi0[R];
#pragma unroll
  for (int i = 0; i < R; ++i) xi0[i] = make_float2(0.f, 0.f);
  auto load_product = [&](int c) {
    const float2* in = g.at(P.prod_in[c]);
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = g.ok ? in[g.elem(pos_step1<L, SP>(m, r))] : make_float2(0.f, 0.f);
  };
  if (n_prod > 0) load_product(0);
  if constexpr (Prog::kUnroll && Spec::kEarlyNoise) {
    if (nf > 0 && plain && P.f[0].noisy)
      draw_line_noise<L, SP>(P, nk, P.f[0].fid, line_pre<Z3>(P, d, g.kxp, g.lineky, m), xi0);
  }
  // One field and one product (the Cahn-Hilliard form): the transformed product stays in
  // v, at the modes the thread updates, unless a thread of the CTA reads a Hermitian
  // partner's value (the packed column: its own tiles in 3D, tile 0 in 2D).  CTA-uniform.
  const bool p0_reg = Prog::kUnroll && Spec::kNF == 1 && Spec::kNProd == 1 && (Z3 ? !g.packed_tile : g.kx0 > 0);
  for (int c = 0; c < n_prod; ++c) {
    float2* Sl = smem + c * slot_sz;
    if (c > 0) load_product(c);
    fwd_step1<L, SP>(v, m, P.tw);
#pragma unroll
    for (int s = 0; s < R; ++s) Sl[g.sidx(l, pos_t1<L, SP>(m, s))] = v[s];
    __syncthreads();
    fwd_load_step2<L, SP>(v, m, P.tw, [&](int n) { return Sl[g.sidx(l, n)]; });
    if (p0_reg) break;   // the only product: kept in v
    __syncthreads();
#pragma unroll
    for (int i = 0; i < R; ++i) Sl[g.sidx(l, pos_step2<L, SP>(m, i))] = v[i];
  }

  auto field_step = [&](const int fi) {
    const FieldK& F = P.f[fi];
    const bool has_chan = (F.chan != nullptr);
    cp_async_wait_all();
    // this field's states and every product slot are in place for the whole CTA (with the
    // product in registers every thread reads only its own copies: its wait suffices; the
    // barrier before the inverse transform keeps slot 0's transposes apart)
    if (!p0_reg) __syncthreads();
    // 2) pointwise update.  Columns kx' > 0: plain half-spectrum modes; with a
    // generated program (Prog::kUnroll) the R points are unrolled so that their
    // independent arithmetic overlaps, the noise draws first (independent generator
    // calls side by side).
    float2 ch[R];
#pragma unroll
    for (int i = 0; i < R; ++i) ch[i] = make_float2(0.f, 0.f);
    const int pl = (NL == 2 && sy > 1 && g.pr != 0) ? (l ^ 1) : l;
    if (g.ok && g.kxp != 0) {
      const LinePre lp = line_pre<Z3>(P, d, g.kxp, g.lineky, m);
      const bool keep_fixed = keep_axis(g.kxp, d.sx, F.chan_xlimit) &&
                              (Z3 ? keep_axis(g.lineky, d.sy, F.chan_ylimit) : keep_axis(0, d.sz, F.chan_zlimit));
      if constexpr (Prog::kUnroll) {
        // Fourier noise of the thread's R modes; ch holds the noise until the update of
        // its mode replaces it (the first field's was drawn during the product loads)
        if (Spec::kEarlyNoise && fi == 0) {
#pragma unroll
          for (int i = 0; i < R; ++i) ch[i] = xi0[i];
        } else if (F.noisy) {
          draw_line_noise<L, SP>(P, nk, F.fid, lp, ch);
        }
#pragma unroll
        for (int i = 0; i < R; ++i)
          ch[i] = update_mode<L, SP, Z3, Prog>(P, lp, F, fi, g, i, smem, n_prod, has_chan, keep_fixed, ch[i], p0_reg,
                                           v[i]);
      } else {
        // table-driven program: a rolled loop (its unrolled code would be very large);
        // the results go through a thread-local array into the registers
        float2 chl[R];
#pragma unroll 1
        for (int i = 0; i < R; ++i) {
          float2 xi = make_float2(0.f, 0.f);
          if (F.noisy) {
            const int pos = pos_step2<L, SP>(m, i);
            xi = Z3 ? noise_at(P, d, nk, F.fid, g.kxp, g.lineky, pos) : noise_at(P, d, nk, F.fid, g.kxp, pos, 0);
          }
          chl[i] = update_mode<L, SP, Z3, Prog>(P, lp, F, fi, g, i, smem, n_prod, has_chan, keep_fixed, xi);
        }
#pragma unroll
        for (int i = 0; i < R; ++i) ch[i] = chl[i];
      }
    } else if (g.ok) {
      // packed column kx' = 0: the kx = 0 and kx = sx/2 planes, unpacked with the
      // Hermitian partner (-ky, -kz).  One thread in W of the first tile only: a rolled
      // loop through a thread-local array keeps the common path's code small.
      float2 chl[R];
#pragma unroll 1
      for (int i = 0; i < R; ++i) {
        const int pos = pos_step2<L, SP>(m, i);
        const int ky = Z3 ? g.lineky : pos;
        const int kz = Z3 ? pos : 0;
        const int ppos = neg_mod(pos, L);
        Fetch fx;
        fx.smem = smem;
        fx.slot_sz = slot_sz;
        fx.as = g.sidx(l, pos);
        fx.ap = g.sidx(pl, ppos);
        fx.n_prod = n_prod;
        fx.p0_reg = false;
        fx.wsel = 0;
        const VPoint v0 = make_vpoint(P, d, 0, ky, kz);
        fx.xi = F.noisy ? noise_at(P, d, nk, F.fid, 0, ky, kz) : make_float2(0.f, 0.f);
        const float2 o0 = Prog::eval(P, fi, v0, fx);
        fx.wsel = 1;
        const VPoint v1 = make_vpoint(P, d, d.sx / 2, ky, kz);
        fx.xi = F.noisy ? noise_at(P, d, nk, F.fid, d.sx / 2, ky, kz) : make_float2(0.f, 0.f);
        const float2 o1 = Prog::eval(P, fi, v1, fx);
        const float2 z = c_add(o0, c_muli(o1));
        const float2 a = (has_chan && keep_point(d, v0, F)) ? c_scale(o0, P.invN) : make_float2(0.f, 0.f);
        const float2 b = (has_chan && keep_point(d, v1, F)) ? c_scale(o1, P.invN) : make_float2(0.f, 0.f);
        g.at(F.next)[g.elem(pos)] = z;
        chl[i] = c_add(a, c_muli(b));
      }
#pragma unroll
      for (int i = 0; i < R; ++i) ch[i] = chl[i];
    }
    // 3) inverse transform of the dealiased copy
    bool skip = !has_chan || g.kx0 > F.chan_xlimit;
    if (Z3 && !g.packed_tile) {
      // both lines of pair p >= 1 have |n_y| = p; pair 0 holds n_y = 0 (the packed-column
      // tiles hold several pairs and are never skipped: masked modes come out zero)
      if (g.pr > 0 && g.pr > F.chan_ylimit) skip = true;
    }
    __syncthreads();   // every read of the slots is done
    if (fi + 1 < nf) prefetch_states<L, SP>(P, P.f[fi + 1], g, smem, n_prod, slot_sz);
    if (skip) return;   // CTA-uniform: masked tile, the channel stays zero
    float2* Ts = smem + P.tslot * slot_sz;
    inv_step2<L, SP>(ch, m, P.tw);
    inv_store_t<L, SP>(ch, m, [&](int n, float2 x) { Ts[g.sidx(l, n)] = x; });
    __syncthreads();
    inv_load_step1<L, SP>(ch, m, P.tw, [&](int n) { return Ts[g.sidx(l, n)]; });
    if (g.ok) {
#pragma unroll
      for (int r = 0; r < R; ++r) g.at(F.chan)[g.elem(pos_step1<L, SP>(m, r))] = ch[r];
    }
    // the next field writes Ts only after its update and the barrier that follows it,
    // which every thread reaches after its reads of Ts above
  };
  if constexpr (Spec::kNF > 0) {
#pragma unroll
    for (int fi = 0; fi < Spec::kNF; ++fi) field_step(fi);
  } else {
    for (int fi = 0; fi < nf; ++fi) field_step(fi);
  }
}

template <int L, int NL, class Prog, class Spec = RtSpec>
__device__ __forceinline__ void turn_body(const LineParams& P) {
  turn_body_at<L, NL, Prog, Spec>(P, blockIdx.x, blockIdx.y, threadIdx.x, threadIdx.y, threadIdx.z);
}

template <int L, int NL>
__global__ void __launch_bounds__(256, 2) turn_pass(const LineParams P) {
  turn_body<L, NL, InterpProg>(P);
}

}  // namespace cupssgb
