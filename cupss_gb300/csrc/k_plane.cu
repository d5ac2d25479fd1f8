// xy-plane pass instantiations and dispatch by (Lx = sx/2, sy).
#include <cstdlib>

#include "launch.h"
#include "plane.cuh"

namespace cupssgb {

namespace {

constexpr int kMaxSmem = 227 * 1024;   // opt-in shared memory of one CTA on sm_100/sm_103

// plane-store pitch: room for nc input columns and the CX owned product columns, = 8 mod 16
// float2 (the two rows a half-warp touches in the x stage fall on disjoint banks)
int store_pitch(int nc, int cx) {
  int ps = nc > cx ? nc : cx;
  while (ps % 16 != 8) ++ps;
  return ps;
}

template <int LX, int LY, int C>
cudaError_t launch_t(const PlaneParams& p, int sz, int nz, cudaStream_t st, bool pdl) {
  using Q = PlaneCfg<LX, LY, C>;
  static std::atomic<unsigned long long> attr{0};   // devices with the smem limit raised
  const size_t smem = Q::smem_bytes(p.ps);
  if (smem > (size_t)kMaxSmem) return cudaErrorInvalidValue;
  cudaError_t e = raise_smem_limit((const void*)plane_pass<LX, LY, C>, attr, kMaxSmem);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cudaLaunchAttribute at[2];
  int na = 0;
  cfg.gridDim = dim3(C, sz, nz);
  cfg.blockDim = dim3(Q::NT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  if (C > 1) {
    at[na].id = cudaLaunchAttributeClusterDimension;
    at[na].val.clusterDim.x = C;
    at[na].val.clusterDim.y = 1;
    at[na].val.clusterDim.z = 1;
    ++na;
  }
  if (pdl) {
    at[na].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[na].val.programmaticStreamSerializationAllowed = 1;
    ++na;
  }
  cfg.attrs = at;
  cfg.numAttrs = na;
  return cudaLaunchKernelEx(&cfg, plane_pass<LX, LY, C>, p);
}

// The instantiated plane shapes: square xy planes from 16^2 to 256^2 (a 256^2 plane of
// 128 x 256 packed complex values is 256 KiB, split over a cluster of two CTAs).
struct Shape {
  int lx, ly, c, cx, t_f2;
};
template <int LX, int LY, int C>
constexpr Shape shape_of() {
  return Shape{LX, LY, C, PlaneCfg<LX, LY, C>::CX, PlaneCfg<LX, LY, C>::T_F2};
}
constexpr Shape kShapes[] = {shape_of<8, 16, 1>(),   shape_of<16, 32, 1>(),  shape_of<32, 64, 1>(),
                             shape_of<64, 128, 1>(), shape_of<64, 128, 2>(), shape_of<128, 256, 2>(),
                             shape_of<128, 256, 4>()};

// cluster size of a plane shape: the default (the first instantiated), or `want` when
// that one is instantiated too
int cluster_of(int Lx, int sy, int want) {
  int first = 0;
  for (const Shape& s : kShapes)
    if (s.lx == Lx && s.ly == sy) {
      if (!first) first = s.c;
      if (s.c == want) return want;
    }
  return first;
}

}  // namespace

int plane_cluster_override() {
  const char* e = std::getenv("CUPSSGB_PLANE_C");
  return e ? std::atoi(e) : 0;
}

int plane_pass_shape(int Lx, int sy, int nc, int* ps, size_t* smem, int want_c) {
  const int c = cluster_of(Lx, sy, want_c > 0 ? want_c : plane_cluster_override());
  for (const Shape& s : kShapes)
    if (s.lx == Lx && s.ly == sy && s.c == c) {
      const int pitch = store_pitch(nc, s.cx);
      const size_t bytes = ((size_t)s.ly * pitch + s.t_f2) * sizeof(float2);
      if (bytes > (size_t)kMaxSmem) return 0;
      if (ps) *ps = pitch;
      if (smem) *smem = bytes;
      return s.c;
    }
  return 0;
}

cudaError_t launch_plane_pass(const PlaneParams& p, int Lx, int sy, int sz, int nz, int c, cudaStream_t st,
                              bool pdl) {
  if (Lx == 8 && sy == 16 && c == 1) return launch_t<8, 16, 1>(p, sz, nz, st, pdl);
  if (Lx == 16 && sy == 32 && c == 1) return launch_t<16, 32, 1>(p, sz, nz, st, pdl);
  if (Lx == 32 && sy == 64 && c == 1) return launch_t<32, 64, 1>(p, sz, nz, st, pdl);
  if (Lx == 64 && sy == 128 && c == 1) return launch_t<64, 128, 1>(p, sz, nz, st, pdl);
  if (Lx == 64 && sy == 128 && c == 2) return launch_t<64, 128, 2>(p, sz, nz, st, pdl);
  if (Lx == 128 && sy == 256 && c == 2) return launch_t<128, 256, 2>(p, sz, nz, st, pdl);
  if (Lx == 128 && sy == 256 && c == 4) return launch_t<128, 256, 4>(p, sz, nz, st, pdl);
  return cudaErrorInvalidValue;
}

}  // namespace cupssgb
