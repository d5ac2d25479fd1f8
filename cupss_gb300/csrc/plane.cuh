// xy-plane pass of a 3D phase (sm_103a): the real-space product of one dealiased
// channel, computed plane by plane with the whole plane on chip.
//
// Input: the turnaround's z-inverted dealiased channel H'(kx', ky, z) (x and y spectral,
// z positional, packed half spectrum).  Only columns kx' < nc and rows |n_y| < ykeep
// carry content (the dealias mask); nothing else is read.  Output: the product
// G''(kx', ky, z) = FFT_xy[ scale * (IFFT_xy H')^order ] for every (kx', ky) of the
// plane -- what the reference computes with computeProduct_k + the term's forward FFT
// (src/term_kernels.cu:48-70, src/term.cpp:48-64) and the x/y parts of the field's
// inverse transforms (src/field.cpp:63-66), here without the three HBM round trips of
// a row pass and two y passes.
//
// One thread-block cluster of C CTAs holds one plane.  CTA r owns rows
// [r RY, (r+1) RY) (RY = LY/C) for the x stage and product columns [r CX, (r+1) CX)
// (CX = LX/C) for the y stages.  Its plane store S (LY rows x PS float2) holds, at its
// own rows, first the y-inverted input columns and then its part of the product; at the
// other rows, the product columns it owns as the other CTAs write them.
//   A  y-inverse of the input columns of this CTA (columns split evenly); each value is
//      written to the plane store of the CTA that owns its row (distributed shared
//      memory).                                                  -> cluster barrier
//   B  per own row: packed inverse real FFT, pointwise power, packed forward real FFT
//      (registers plus a per-row transpose buffer, warp-synchronous: the M threads of a
//      row are in one warp); each output bin goes to the CTA that owns its column.  A
//      row's store slot is overwritten only by the threads that read it, after they
//      read it.                                                  -> cluster barrier
//   C  forward y FFT of the owned columns, in place in the plane store, and the store
//      of the product plane to global memory (a warp stores 32 consecutive columns).
// No other CTA touches this CTA's shared memory after the second barrier, so a CTA may
// exit when its phase C ends.
#pragma once
#include <cooperative_groups.h>

#include "engine_types.h"
#include "fft.cuh"
#include "kernels.cuh"

namespace cupssgb {

template <int LX, int LY, int C>
struct PlaneCfg {
  static constexpr int NT = 512;                 // threads per CTA
  static constexpr int RY = LY / C;              // rows of one CTA (x stage)
  static constexpr int CX = LX / C;              // product columns of one CTA (y stages)
  static constexpr int MY = LineCfg<LY>::M, RYV = LineCfg<LY>::R;
  static constexpr int MX = LineCfg<LX>::M, RXV = LineCfg<LX>::R;
  static constexpr int LA = NT / MY;             // y lines per pass (phases A and C)
  static constexpr int RB = NT / MX;             // rows per pass (phase B)
  static constexpr int PLY = padded_len<LY>();
  static constexpr int PLX = RowCfg<LX, false>::PL;
  static constexpr int T_A = LA * PLY;           // float2 of the phase-A transpose buffer
  static constexpr int T_B = RB * PLX;           // float2 of the phase-B row buffers
  static constexpr int T_F2 = T_A > T_B ? T_A : T_B;
  static_assert(C == 1 || C == 2 || C == 4 || C == 8, "cluster of 1, 2, 4 or 8 CTAs");
  static_assert(LY % C == 0 && LX % C == 0, "the plane splits evenly");
  static_assert(RY % MY == 0, "a y line's registers split by owner at compile time");
  static_assert(CX % MX == 0, "a row's registers split by owner at compile time");
  static_assert(MX <= 32 && 32 % MX == 0, "the threads of a row are in one warp");
  static_assert(LA >= 32 || LA * MY == NT, "phase A/C lanes: consecutive columns");
  // dynamic shared memory for plane-store pitch ps
  static constexpr size_t smem_bytes(int ps) { return ((size_t)LY * ps + T_F2) * sizeof(float2); }
};

template <int LX, int LY, int C>
__global__ void __launch_bounds__(512, 1) plane_pass(const PlaneParams p) {
  namespace cg = cooperative_groups;
  using Q = PlaneCfg<LX, LY, C>;
  constexpr int MY = Q::MY, RYV = Q::RYV, MX = Q::MX, RXV = Q::RXV;
  constexpr int LA = Q::LA, RB = Q::RB, RY = Q::RY, CX = Q::CX, PLX = Q::PLX;
  constexpr int sx = 2 * LX;
  extern __shared__ float2 smem[];
  float2* S = smem;                         // plane store, LY rows of pitch ps
  float2* T = smem + (size_t)LY * p.ps;     // transpose buffers
  grid_dep_sync();
  if (p.members && !p.members[blockIdx.z].active) return;   // cluster-uniform (same z), before any barrier
  int r = 0;
  float2* Sr[C];                            // plane store of each CTA of the cluster
  if constexpr (C > 1) {
    cg::cluster_group cl = cg::this_cluster();
    r = (int)cl.block_rank();
#pragma unroll
    for (int q = 0; q < C; ++q) Sr[q] = cl.map_shared_rank(S, q);
  } else {
    Sr[0] = S;
  }
  auto cluster_sync = [&]() {
    if constexpr (C > 1) {
      cg::this_cluster().sync();
    } else {
      __syncthreads();
    }
  };
  // Distributed shared memory may be written only once every CTA of the cluster runs:
  // each thread arrives here and waits (once) just before its first remote store.
  if constexpr (C > 1) asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory");
  bool started = C == 1;
  auto wait_started = [&]() {
    if constexpr (C > 1) {
      if (!started) asm volatile("barrier.cluster.wait.aligned;" ::: "memory");
    }
    started = true;
  };
  const int tid = threadIdx.x;
  const int ps = p.ps;
  const int z = blockIdx.y;
  const size_t pbase = (size_t)blockIdx.z * p.mstride + (size_t)z * LY * LX;
  const float2* in = p.in + pbase;
  float2* out = p.out + pbase;

  // ---- A: y-inverse of this CTA's input columns -------------------------------------------
  {
    const int per = (p.nc + C - 1) / C;
    const int c0 = r * per, c1 = min(p.nc, c0 + per);
    const int w = tid % LA, m = tid / LA;
    for (int cb = c0; cb < c1; cb += LA) {
      const int c = cb + w;
      const bool live = c < c1;
      float2 v[RYV];
#pragma unroll
      for (int i = 0; i < RYV; ++i) {
        const int k = pos_step2<LY>(m, i);
        const int nk = (k > LY / 2) ? LY - k : k;
        v[i] = (live && nk < p.ykeep) ? in[(size_t)k * LX + c] : make_float2(0.f, 0.f);
      }
      inv_step2<LY>(v, m, p.tw);
      if (cb > c0) __syncthreads();   // the previous pass's reads of T
      inv_store_t<LY>(v, m, [&](int n, float2 x) { T[pad_pos<LY>(n) * LA + w] = x; });
      __syncthreads();
      inv_load_step1<LY>(v, m, p.tw, [&](int n) { return T[pad_pos<LY>(n) * LA + w]; });
      wait_started();   // CTA-uniform: every thread runs the same passes
      if (live) {
#pragma unroll
        for (int j = 0; j < RYV; ++j) {
          const int n = pos_step1<LY>(m, j);       // y row of register j
          Sr[j / (RY / MY)][n * ps + c] = v[j];    // owner of row n: j / (RY/MY)
        }
      }
    }
    wait_started();   // a CTA without input columns still completes the start barrier
  }
  cluster_sync();

  // ---- B: x stage of the own rows -------------------------------------------------------
  {
    const int m = tid % MX, q = tid / MX;
    float2* TB = T + q * PLX;
    const float2 wm = tw_load(p.tw, sx, m);
#pragma unroll 1
    for (int yb = 0; yb < RY; yb += RB) {
      // a pass can have more thread rows than the CTA has rows (small planes): the extra
      // rows compute on row 0 of the CTA's range (so every lane reaches the warp
      // barriers) and store nothing
      const bool live = yb + q < RY;
      const int y = r * RY + (live ? yb + q : 0);
      float2* row = S + y * ps;
      float2 v[RXV];
      // packed row X[k] (k < nc) and its C2R pre-processing with the mirror X[LX - k]
#pragma unroll
      for (int i = 0; i < RXV; ++i) {
        const int k = pos_step2<LX>(m, i);
        v[i] = k < p.nc ? row[k] : make_float2(0.f, 0.f);
      }
      static_for(make_iseq<RXV>{}, [&](auto I) {
        constexpr int i = decltype(I)::value;
        const int k = pos_step2<LX>(m, i);
        const int km = neg_mod(k, LX);
        const float2 mir = km < p.nc ? row[km] : make_float2(0.f, 0.f);
        if constexpr (RowTwSplit<LX, false>::value) {
          v[i] = c2r_pre_w(v[i], mir, k, row_twiddle<LX, false, i>(wm));
        } else {
          v[i] = c2r_pre(v[i], mir, k, sx, p.tw);
        }
      });
      inv_step2<LX>(v, m, p.tw);
      inv_store_t<LX>(v, m, [&](int n, float2 x) { TB[pad_pos<LX>(n)] = x; });
      __syncwarp();
      inv_load_step1<LX>(v, m, p.tw, [&](int n) { return TB[pad_pos<LX>(n)]; });
      // v[j] = real pair (r[2n], r[2n+1]), n = m + MX j: raise to the product's order
#pragma unroll
      for (int j = 0; j < RXV; ++j) {
        const float2 x = v[j];
        float2 acc = make_float2(p.out_scale, p.out_scale);
        for (int t = 0; t < p.order; ++t) {
          acc.x *= x.x;
          acc.y *= x.y;
        }
        v[j] = acc;
      }
      fwd_step1<LX>(v, m, p.tw);
      __syncwarp();   // every read of TB above is done
#pragma unroll
      for (int s = 0; s < RXV; ++s) TB[pad_pos<LX>(pos_t1<LX>(m, s))] = v[s];
      __syncwarp();
      fwd_load_step2<LX>(v, m, p.tw, [&](int n) { return TB[pad_pos<LX>(n)]; });
      __syncwarp();
#pragma unroll
      for (int i = 0; i < RXV; ++i) TB[pad_pos<LX>(pos_step2<LX>(m, i))] = v[i];
      __syncwarp();
      // R2C post-processing; bin k goes to the CTA owning column k (owner per register is
      // a compile-time constant: k = m + step2_off(i) with m < MX and CX a multiple of MX)
      static_for(make_iseq<RXV>{}, [&](auto I) {
        constexpr int i = decltype(I)::value;
        constexpr int own = step2_off<LX>(i) / CX;
        const int k = pos_step2<LX>(m, i);
        const float2 zm = TB[pad_pos<LX>(neg_mod(k, LX))];
        float2 x;
        if constexpr (RowTwSplit<LX, false>::value) {
          x = r2c_post_w(v[i], zm, k, row_twiddle<LX, false, i>(wm));
        } else {
          x = r2c_post(v[i], zm, k, sx, p.tw);
        }
        if (live) Sr[own][y * ps + (k - own * CX)] = x;
      });
      __syncwarp();   // TB is rewritten by the next row of this thread group
    }
  }
  cluster_sync();

  // ---- C: forward y FFT of the owned product columns, in place, and the store -------------
  {
    const int w = tid % LA, m = tid / LA;
    for (int cb = 0; cb < CX; cb += LA) {
      const int c = cb + w;
      const bool live = c < CX;
      const int cc = live ? c : 0;
      float2 v[RYV];
#pragma unroll
      for (int j = 0; j < RYV; ++j) v[j] = S[pos_step1<LY>(m, j) * ps + cc];
      fwd_step1<LY>(v, m, p.tw);
      __syncthreads();   // every thread's loads of this pass's columns are done
      if (live) {
#pragma unroll
        for (int s = 0; s < RYV; ++s) S[pos_t1<LY>(m, s) * ps + c] = v[s];
      }
      __syncthreads();
      fwd_load_step2<LY>(v, m, p.tw, [&](int n) { return S[n * ps + cc]; });
      if (live) {
        float2* o = out + r * CX + c;
#pragma unroll
        for (int i = 0; i < RYV; ++i) o[(size_t)pos_step2<LY>(m, i) * LX] = v[i];
      }
    }
  }
}

}  // namespace cupssgb
