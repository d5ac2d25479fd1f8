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
#if !defined(__CUDACC_RTC__)
#include <cuda_runtime.h>
#include <cstdint>
#endif
#include "engine_types.h"
#include "fft.cuh"
#include "philox.cuh"
#include "point_math.cuh"
#include "line_geom.cuh"

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

// The same two steps with the twiddle w = W_sx^k given.
__device__ __forceinline__ float2 c2r_pre_w(float2 a, float2 bm, int k, float2 w) {
  if (k == 0) return make_float2(a.x + a.y, a.x - a.y);
  const float2 b = c_conj(bm);
  return c_add(c_add(a, b), c_muli(c_mulc(c_sub(a, b), w)));
}
__device__ __forceinline__ float2 r2c_post_w(float2 zk, float2 zm, int k, float2 w) {
  if (k == 0) return make_float2(zk.x + zk.y, zk.x - zk.y);
  const float2 zc = c_conj(zm);
  const float2 e = c_scale(c_add(zk, zc), 0.5f);
  const float2 o = c_scale(c_mulmi(c_sub(zk, zc)), 0.5f);
  return c_add(e, c_mul(w, o));
}

// Compile-time loop: f(ic<0>{}), ..., f(ic<N-1>{}) (each index usable as a template argument).
template <int N>
struct ic {
  static constexpr int value = N;
};
template <class F, int... I>
__device__ __forceinline__ void static_for(iseq<I...>, F&& f) {
  (f(ic<I>{}), ...);
}

// Twiddle W_sx^k of register I of thread m in the step-2 layout of a packed row
// (k = m + M c, c = step2_off(I) / M), from W_sx^m: W_sx^k = W_sx^m W_{2R}^c, the second
// factor a compile-time constant (sx = 2 R M).  One table load per thread instead of one
// per register; usable while 2R <= 64 (the compile-time twiddle table).
template <int LX, bool SP>
struct RowTwSplit {
  static constexpr int N = 2 * LineCfg<LX, SP>::R;
  static constexpr bool value = (64 % N == 0 || 192 % N == 0) && (LineCfg<LX, SP>::M > 1);
};
template <int LX, bool SP, int I>
__device__ __forceinline__ float2 row_twiddle(float2 wm) {
  constexpr int M = LineCfg<LX, SP>::M, R = LineCfg<LX, SP>::R;
  return tw_const<2 * R, step2_off<LX, SP>(I) / M, false>(wm);
}

// Register i of the two loops below, i a compile-time index (a functor rather than a
// lambda: the generated kernels that include this header are compiled by NVRTC, which
// treats lambdas without an execution-space annotation as host code).
template <int LX, bool SP>
struct RowC2rAt {
  float2 (&v)[LineCfg<LX, SP>::R];
  const float2* T;
  int m;
  float2 wm;
  template <int i>
  __device__ __forceinline__ void operator()(ic<i>) const {
    const int k = pos_step2<LX, SP>(m, i);
    v[i] = c2r_pre_w(v[i], T[pad_pos<LX, SP>(neg_mod(k, LX))], k, row_twiddle<LX, SP, i>(wm));
  }
};
template <int LX, bool SP>
struct RowR2cAt {
  const float2 (&v)[LineCfg<LX, SP>::R];
  const float2* T;
  int m;
  float2 wm;
  float2* out;
  bool live;
  template <int i>
  __device__ __forceinline__ void operator()(ic<i>) const {
    const int k = pos_step2<LX, SP>(m, i);
    const float2 x = r2c_post_w(v[i], T[pad_pos<LX, SP>(neg_mod(k, LX))], k, row_twiddle<LX, SP, i>(wm));
    if (live) out[k] = x;
  }
};

// C2R pre-processing of a packed row held in step-2 layout (v) and also stored in T
// (padded positions): v[i] <- Z at k = pos_step2(m, i), the mirror X[Lx - k] from T.
template <int LX, bool SP>
__device__ __forceinline__ void row_c2r(float2 (&v)[LineCfg<LX, SP>::R], const float2* T, int m, const float2* tw) {
  constexpr int R = LineCfg<LX, SP>::R, sx = 2 * LX;
  if constexpr (RowTwSplit<LX, SP>::value) {
    const float2 wm = tw_load(tw, sx, m);
    static_for(make_iseq<R>{}, RowC2rAt<LX, SP>{v, T, m, wm});
  } else {
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int k = pos_step2<LX, SP>(m, i);
      v[i] = c2r_pre(v[i], T[pad_pos<LX, SP>(neg_mod(k, LX))], k, sx, tw);
    }
  }
}

// R2C post-processing of a transformed row (v in step-2 layout, also stored in T) and
// its store to out (packed row).
template <int LX, bool SP>
__device__ __forceinline__ void row_r2c_store(const float2 (&v)[LineCfg<LX, SP>::R], const float2* T, int m,
                                              const float2* tw, float2* out, bool live) {
  constexpr int R = LineCfg<LX, SP>::R, sx = 2 * LX;
  if constexpr (RowTwSplit<LX, SP>::value) {
    const float2 wm = tw_load(tw, sx, m);
    static_for(make_iseq<R>{}, RowR2cAt<LX, SP>{v, T, m, wm, out, live});
  } else {
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int k = pos_step2<LX, SP>(m, i);
      const float2 x = r2c_post(v[i], T[pad_pos<LX, SP>(neg_mod(k, LX))], k, sx, tw);
      if (live) out[k] = x;
    }
  }
}

template <int LX, bool SP>
struct RowCfg {
  static constexpr int M = LineCfg<LX, SP>::M;
  static constexpr int R = LineCfg<LX, SP>::R;
  // Padded row length in smem.  A half-warp covers 16/M rows of M threads each
  // (2M banks per row for 8-byte accesses); a pitch = M (mod 16) float2 puts those
  // rows on disjoint banks.
  static constexpr int PL0 = padded_len<LX, SP>();
  static constexpr int PL = (M >= 16) ? PL0 + 1 : PL0 + ((M - PL0 % 16) % 16 + 16) % 16;
  static constexpr int RW = (M >= 128) ? 1 : (128 / M > 32 ? 32 : 128 / M);   // rows per CTA
};

// smem: (1 + n_in) slots of RW*PL float2.  Slot 0 is the transpose buffer.
// Row block bx, thread (m, rl): blockIdx.x and threadIdx in a plain launch; a fused launch
// over several grids maps its flat indices to them.  The batch member is blockIdx.z.
template <int LX, bool SP>
__device__ __forceinline__ void row_pass_body(const XParams& p, int bx, int m, int rl) {
  using C = RowCfg<LX, SP>;
  constexpr int M = C::M, R = C::R, PL = C::PL, RW = C::RW;
  extern __shared__ float2 smem[];
  grid_dep_sync();
  if (p.members && !p.members[blockIdx.z].active) return;   // CTA-uniform
  const int row = bx * RW + rl;
  const bool live = row < p.rows;
  const int sx = 2 * LX;
  float2* T = smem + rl * PL;
  auto slot = [&](int i) { return smem + (size_t)(1 + i) * RW * PL + rl * PL; };
  const size_t rowoff = (size_t)blockIdx.z * p.mstride + (size_t)(live ? row : 0) * LX;
  float2 v[R];

  // Spectral inputs: every channel's row is copied into its slot asynchronously at once,
  // so that the loads of all channels are in flight together; each channel's inverse
  // transform then reads its row, and the Hermitian mirror X[Lx - k] of the C2R step,
  // from the slot, and finally overwrites the slot with its real-space values.
  const bool spectral = p.in_mode == kXInSpectral;
  if (spectral) {
#pragma unroll 1
    for (int c = 0; c < p.n_in; ++c) {
      const float2* in = p.in[c] + rowoff;
      const int xcols = p.in_xcols[c] > 0 ? p.in_xcols[c] : LX;
      const unsigned sv = smem_u32(slot(c));
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const int k = pos_step2<LX, SP>(m, i);
        const bool ld = live && k < xcols;   // columns at or beyond xcols are known zero
        cp_async8(sv + 8u * (unsigned)pad_pos<LX, SP>(k), ld ? in + k : in, ld ? 8 : 0);
      }
    }
    cp_async_commit();
    cp_async_wait_all();
    __syncthreads();
  }

  for (int c = 0; c < p.n_in; ++c) {
    float2* V = slot(c);
    if (p.in_mode == kXInReal) {
      const float2* in = p.in[c] + rowoff;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int n = pos_step1<LX, SP>(m, r);
        V[pad_pos<LX, SP>(n)] = live ? in[n] : make_float2(0.f, 0.f);
      }
      continue;
    }
    if (p.in_mode == kXInRealPair) {
      // reference float2 layout: point 2n at (.x of) element 2n, point 2n+1 at 2n+1
      const float4* in = reinterpret_cast<const float4*>(p.in[c]) + rowoff;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int n = pos_step1<LX, SP>(m, r);
        const float4 q = live ? in[n] : make_float4(0.f, 0.f, 0.f, 0.f);
        V[pad_pos<LX, SP>(n)] = make_float2(q.x, q.z);
      }
      continue;
    }
    // the staged spectral row (every thread's copies are complete and visible: wait and
    // barrier above); the slot is overwritten only after the two barriers below, which
    // follow every thread's reads of it
#pragma unroll
    for (int i = 0; i < R; ++i) v[i] = V[pad_pos<LX, SP>(pos_step2<LX, SP>(m, i))];
    row_c2r<LX, SP>(v, V, m, p.tw);
    inv_step2<LX, SP>(v, m, p.tw);
    __syncthreads();   // CTA-uniform: the previous channel's last reads of T
    inv_store_t<LX, SP>(v, m, [&](int n, float2 x) { T[pad_pos<LX, SP>(n)] = x; });
    __syncthreads();
    inv_load_step1<LX, SP>(v, m, p.tw, [&](int n) { return T[pad_pos<LX, SP>(n)]; });
#pragma unroll
    for (int r = 0; r < R; ++r) V[pad_pos<LX, SP>(pos_step1<LX, SP>(m, r))] = v[r];
  }

  for (int q = 0; q < p.n_prod; ++q) {
    // pointwise product of the real values (packed as pairs r[2n], r[2n+1]), added to the
    // channel's earlier products when prod_add[q] is set
    const bool add = p.prod_add[q] != 0;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int a = pad_pos<LX, SP>(pos_step1<LX, SP>(m, r));
      float2 acc = make_float2(p.out_scale, p.out_scale);   // output scale folded into the product
      for (int t = 0; t < p.prod_n[q]; ++t) {
        float2 x = slot(p.prod_f[q][t])[a];
        acc.x *= x.x;
        acc.y *= x.y;
      }
      v[r] = add ? make_float2(v[r].x + acc.x, v[r].y + acc.y) : acc;
    }
    if (q + 1 < p.n_prod && p.prod_add[q + 1]) continue;   // CTA-uniform: the channel goes on
    if (p.out_mode != kXOutSpectral) {
      if (live) {
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const int n = pos_step1<LX, SP>(m, r);
          const float2 z = v[r];
          if (p.out_mode == kXOutReal) {
            reinterpret_cast<float2*>(p.out[q])[rowoff + n] = z;
          } else {
            reinterpret_cast<float4*>(p.out[q])[rowoff + n] = make_float4(z.x, 0.f, z.y, 0.f);
          }
        }
      }
      continue;
    }
    fwd_step1<LX, SP>(v, m, p.tw);
    __syncthreads();
#pragma unroll
    for (int s = 0; s < R; ++s) T[pad_pos<LX, SP>(pos_t1<LX, SP>(m, s))] = v[s];
    __syncthreads();
    fwd_load_step2<LX, SP>(v, m, p.tw, [&](int n) { return T[pad_pos<LX, SP>(n)]; });
    __syncthreads();
#pragma unroll
    for (int i = 0; i < R; ++i) T[pad_pos<LX, SP>(pos_step2<LX, SP>(m, i))] = v[i];
    __syncthreads();
    row_r2c_store<LX, SP>(v, T, m, p.tw, reinterpret_cast<float2*>(p.out[q]) + rowoff, live);
  }
}

// The four-step form and the split form (register budget of two resident CTAs per SM:
// without it the register allocation of the split form spills).
template <int LX>
__global__ void __launch_bounds__(RowCfg<LX, false>::M * RowCfg<LX, false>::RW) row_pass(const XParams p) {
  row_pass_body<LX, false>(p, blockIdx.x, threadIdx.x, threadIdx.y);
}
template <int LX>
__global__ void __launch_bounds__(RowCfg<LX, true>::M * RowCfg<LX, true>::RW, 2) row_pass_split(const XParams p) {
  row_pass_body<LX, true>(p, blockIdx.x, threadIdx.x, threadIdx.y);
}

// Single spectral input, single spectral product (the Cahn-Hilliard form phi^n): the
// inverse transform of the row stays in registers and feeds the product and the forward
// transform directly, so shared memory holds only transpose buffers (no slot for the
// real-space input) and the input is read once instead of once per factor.  Columns at
// or beyond in_xcols[0] are known zero (dealiased channel) and are not loaded.
template <int LX, bool SP>
struct RowOneCfg {
  // resident CTAs per SM the register budget is sized for (RW*M = 128 threads each)
  static constexpr int kMinBlocks = (LineCfg<LX, SP>::R <= 16) ? 4 : ((LX <= 512) ? 3 : 2);
};

template <int LX, bool SP>
__device__ __forceinline__ void row_one_body(const XParams& p, int bx, int m, int rl) {
  using C = RowCfg<LX, SP>;
  constexpr int M = C::M, R = C::R, PL = C::PL, RW = C::RW;
  extern __shared__ float2 smem[];
  grid_dep_sync();
  if (p.members && !p.members[blockIdx.z].active) return;   // CTA-uniform
  const int row = bx * RW + rl;
  const bool live = row < p.rows;
  // two transpose buffers used in turn: a buffer is written again only after a barrier
  // that follows every read of its previous contents, so the write-after-read barriers
  // of a single buffer are not needed
  float2* TA = smem + rl * PL;
  float2* TB = smem + (RW + rl) * PL;
  const size_t rowoff = (size_t)blockIdx.z * p.mstride + (size_t)(live ? row : 0) * LX;
  const int xcols = p.in_xcols[0] > 0 ? p.in_xcols[0] : LX;
  float2 v[R];
  const float2* in = p.in[0] + rowoff;
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const int k = pos_step2<LX, SP>(m, i);
    v[i] = (live && k < xcols) ? in[k] : make_float2(0.f, 0.f);
    TA[pad_pos<LX, SP>(k)] = v[i];
  }
  __syncthreads();
  row_c2r<LX, SP>(v, TA, m, p.tw);
  inv_step2<LX, SP>(v, m, p.tw);
  inv_store_t<LX, SP>(v, m, [&](int n, float2 x) { TB[pad_pos<LX, SP>(n)] = x; });
  __syncthreads();
  inv_load_step1<LX, SP>(v, m, p.tw, [&](int n) { return TB[pad_pos<LX, SP>(n)]; });
  // v[r] = real pair (r[2n], r[2n+1]) at n = m + M r: raise to the product's order
  const int order = p.prod_n[0];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const float2 x = v[r];
    float2 acc = make_float2(p.out_scale, p.out_scale);
    for (int t = 0; t < order; ++t) {
      acc.x *= x.x;
      acc.y *= x.y;
    }
    v[r] = acc;
  }
  fwd_step1<LX, SP>(v, m, p.tw);
#pragma unroll
  for (int s = 0; s < R; ++s) TA[pad_pos<LX, SP>(pos_t1<LX, SP>(m, s))] = v[s];
  __syncthreads();
  fwd_load_step2<LX, SP>(v, m, p.tw, [&](int n) { return TA[pad_pos<LX, SP>(n)]; });
#pragma unroll
  for (int i = 0; i < R; ++i) TB[pad_pos<LX, SP>(pos_step2<LX, SP>(m, i))] = v[i];
  __syncthreads();
  row_r2c_store<LX, SP>(v, TB, m, p.tw, reinterpret_cast<float2*>(p.out[0]) + rowoff, live);
}

template <int LX, bool SP>
__global__ void __launch_bounds__(RowCfg<LX, SP>::M * RowCfg<LX, SP>::RW, RowOneCfg<LX, SP>::kMinBlocks)
row_pass_one(const XParams p) {
  row_one_body<LX, SP>(p, blockIdx.x, threadIdx.x, threadIdx.y);
}

// ------------------------------------------------------------------------------------
// line pass (strided axis): forward or inverse FFT of whole lines, in place or not
// ------------------------------------------------------------------------------------
// Grid: x = kx' tile (W columns), y = z (kGeoY3) / ky (kGeoZ3).  Block: (W, M, 1).
// smem: PL * W float2 (one transpose slot).  Up to 16 values per thread fit the register
// budget of four resident CTAs per SM (64 registers, no spills), 32 values that of two.
template <int L>
__global__ void __launch_bounds__(256, (LineCfg<L>::R <= 16) ? 4 : 2)
line_pass(const LineParams P) {
  constexpr int M = LineCfg<L>::M, R = LineCfg<L>::R;
  extern __shared__ float2 smem[];
  grid_dep_sync();
  if (P.members && !P.members[blockIdx.z].active) return;   // CTA-uniform
  const LineGeom<L, 1> g(P);
  float2 v[R];
  for (int c = 0; c < P.n_prod; ++c) {
    if (P.mode == kModeInv && g.kx0 > P.inv_xlimit[c]) continue;   // CTA-uniform
    float2* T = smem;
    const float2* in = g.at(P.prod_in[c]);
    float2* out = g.at(P.prod_out[c]);
    if (P.mode == kModeFwd) {
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = g.ok ? in[g.elem(pos_step1<L>(g.m, r))] : make_float2(0.f, 0.f);
      fwd_step1<L>(v, g.m, P.tw);
      if (c > 0) __syncthreads();   // the previous channel's reads of T
#pragma unroll
      for (int s = 0; s < R; ++s) T[g.sidx(0, pos_t1<L>(g.m, s))] = v[s];
      __syncthreads();
      fwd_load_step2<L>(v, g.m, P.tw, [&](int n) { return T[g.sidx(0, n)]; });
      if (g.ok) {
#pragma unroll
        for (int i = 0; i < R; ++i) out[g.elem(pos_step2<L>(g.m, i))] = v[i];
      }
    } else {
      const int keep = P.inv_lkeep[c];
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const int k = pos_step2<L>(g.m, i);
        const int nk = (k > L / 2) ? L - k : k;
        v[i] = (g.ok && (keep <= 0 || nk < keep)) ? in[g.elem(k)] : make_float2(0.f, 0.f);
      }
      inv_step2<L>(v, g.m, P.tw);
      if (c > 0) __syncthreads();   // the previous channel's reads of T
      inv_store_t<L>(v, g.m, [&](int n, float2 x) { T[g.sidx(0, n)] = x; });
      __syncthreads();
      inv_load_step1<L>(v, g.m, P.tw, [&](int n) { return T[g.sidx(0, n)]; });
      if (g.ok) {
#pragma unroll
        for (int r = 0; r < R; ++r) out[g.elem(pos_step1<L>(g.m, r))] = v[r];
      }
    }
  }
}

// Packed half spectrum -> reference-layout full complex spectrum.
__global__ void expand_spectrum(const ExpandParams p);
__global__ void compress_spectrum(const CompressParams p);
__global__ void mask_spectrum(const MaskParams p);

}  // namespace cupssgb
