// Thread -> (column, line, position) mapping shared by the line passes.
//
// A CTA owns W consecutive kx' columns of NL lines of length L along the line axis.
// Block (W, M, NL): threadIdx.x = column within the tile (fastest, so global
// accesses of one warp cover contiguous kx'), threadIdx.y = m (FFT thread of the
// line), threadIdx.z = line of the tile.  Geometries:
//   kGeoCol : lines along y of a 2D/1D array      elem = y*Lx + kx'
//   kGeoY3  : lines along y of a 3D array         elem = (z*sy + y)*Lx + kx', blockIdx.y = z
//   kGeoZ3  : lines along z of a 3D array         elem = (z*sy + ky)*Lx + kx', blockIdx.y = ky,
//             or, with NL = 2, the pair {p, sy-p} (p >= 1) / {0, sy/2} (p = 0) so that the
//             Hermitian partner (-ky, -kz) of every point of the packed column kx' = 0 is
//             in the same CTA.
// Shared-memory slots hold NL * PL * W float2, position n of line `line` of column w at
// (line*PL + pad_pos(n))*W + w.  In a batch, blockIdx.z is the member and every element
// index is offset by mbase = blockIdx.z * P.mstride.
#pragma once
#include "engine_types.h"
#include "fft.cuh"

namespace cupssgb {

// WT > 0: the tile width is a compile-time constant (generated kernels), so every
// shared-memory index below is a per-thread base plus an immediate offset.
//
// Paired z lines (NL = 2, the 3D turnaround): the packed column kx' = 0, whose modes
// need two updates each (the kx = 0 and kx = sx/2 planes), gets tiles of its own so
// that no warp mixes it with plain columns: tile index tx = ceil(Lx/W) holds, in thread
// column w, the pair ty*W + w of column 0; the regular tiles leave column 0 out.
// SP: the lines use the split FFT form (its padded line length).
template <int L, int NL, int WT = 0, bool SP = false>
struct LineGeom {
  static constexpr int PL = padded_len<L, SP>();
  int W, w, m, l, kx0, kxp, lineky;
  int pr;                // NL = 2: pair index of this thread's two lines
  bool packed_tile;      // NL = 2: this CTA works on the packed column kx' = 0
  bool idle;             // a packed-column CTA past the last pair (CTA-uniform)
  bool ok;
  int lofs, pstride;     // element offset of this thread's line (position 0) and stride, within a member
  size_t mbase;
  int slot_sz;
  __device__ __forceinline__ explicit LineGeom(const LineParams& P) {
    init(P, P.sy, P.sx / 2, blockIdx.x, blockIdx.y, threadIdx.x, threadIdx.y, threadIdx.z);
  }
  // Grid sizes from the caller (compile-time constants in generated kernels).
  __device__ __forceinline__ LineGeom(const LineParams& P, int sy, int Lx) {
    init(P, sy, Lx, blockIdx.x, blockIdx.y, threadIdx.x, threadIdx.y, threadIdx.z);
  }
  // Tile (tx, ty) and thread (w, m, l) given by the caller: a fused launch over several
  // grids maps its flat block index and thread index to them.
  __device__ __forceinline__ LineGeom(const LineParams& P, int sy, int Lx, int tx, int ty, int tw, int tm, int tl) {
    init(P, sy, Lx, tx, ty, tw, tm, tl);
  }
  __device__ __forceinline__ void init(const LineParams& P, int sy, int Lx, int tx, int ty, int tw, int tm, int tl) {
    W = WT > 0 ? WT : P.W;
    w = tw;
    m = tm;
    l = tl;
    kx0 = tx * W;
    kxp = kx0 + w;
    lineky = 0;
    pr = ty;
    packed_tile = false;
    idle = false;
    bool lineok = true;
    // the paired form (NL = 2) is only used along z
    const int geo = (NL == 2) ? (int)kGeoZ3 : P.geo;
    if (geo == kGeoCol) {
      lofs = kxp;
      pstride = Lx;
    } else if (geo == kGeoY3) {
      lofs = ty * sy * Lx + kxp;
      pstride = Lx;
    } else {
      if (NL == 2) {
        const int pairs = sy > 1 ? sy / 2 : 1;
        if (tx * W >= Lx) {
          packed_tile = true;
          kx0 = 0;
          kxp = 0;
          pr = ty * W + w;
          idle = ty * W >= pairs;
          lineok = pr < pairs;
        } else {
          lineok = kxp != 0;
        }
        lineky = (l == 0) ? pr : ((pr == 0) ? sy / 2 : sy - pr);
        lineok = lineok && !(l == 1 && sy == 1);
      } else {
        lineky = ty;
      }
      lofs = lineky * Lx + kxp;
      pstride = sy * Lx;
    }
    ok = (kxp < Lx) && lineok;
    mbase = (size_t)blockIdx.z * P.mstride;
    slot_sz = NL * PL * W;
  }
  // 32-bit element index within the member; at(p) is p moved to this CTA's member.
  __device__ __forceinline__ int elem(int pos) const { return lofs + pos * pstride; }
  template <class T>
  __device__ __forceinline__ T* at(T* p) const {
    return p + mbase;
  }
  __device__ __forceinline__ int sidx(int line, int pos) const { return (line * PL + pad_pos<L, SP>(pos)) * W + w; }
};

}  // namespace cupssgb
