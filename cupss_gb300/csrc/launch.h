// Host-side launchers for the engine kernels (implemented in k_*.cu).
#pragma once
#include <cuda_runtime.h>

#include <atomic>

#include "engine_types.h"

namespace cupssgb {

// Raises a kernel's dynamic shared-memory limit (220 KiB unless given) on the current
// device.  The attribute belongs to one device, so `done` records, one bit per device
// ordinal, the devices where it is set; the bit is set after a successful call, and two
// threads that race both make the (idempotent) call.
inline cudaError_t raise_smem_limit(const void* kernel, std::atomic<unsigned long long>& done,
                                    int bytes = 220 * 1024) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = (dev >= 0 && dev < 64) ? (1ull << dev) : 0ull;
  if (bit && (done.load(std::memory_order_acquire) & bit)) return cudaSuccess;
  e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess && bit) done.fetch_or(bit, std::memory_order_acq_rel);
  return e;
}

// Launch configuration; pdl: programmatic stream serialization, so the kernel may
// become resident while its predecessor in the stream drains (the step kernels wait
// for the predecessor's completion themselves, see grid_dep_sync).
struct LaunchCfg {
  cudaLaunchConfig_t cfg;
  cudaLaunchAttribute attr[1];
  LaunchCfg(dim3 grid, dim3 block, size_t smem, cudaStream_t st, bool pdl) {
    cfg = cudaLaunchConfig_t{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
  }
};

// Row pass over all rows (of nz batch members); picks the template by p.Lx.
cudaError_t launch_row_pass(const XParams& p, cudaStream_t st, int nz = 1, bool pdl = false);

// Line pass: grid.x = ceil(Lx/W) tiles, grid.y per geometry; nl = 2 for the paired
// 3D z-turnaround.  nslots = shared-memory slots the mode needs.
cudaError_t launch_line_pass(const LineParams& p, int nl, int nslots, dim3 grid, cudaStream_t st,
                             bool pdl = false);
// split: the lines use the split FFT form (LineCfg<L, true>)
size_t line_pass_smem(int L, int nl, int W, int nslots, bool split = false);
int line_threads(int L, int nl, int W, bool split = false);
// The generated turnaround runs lines of 512 and 1024 points in the split form (a 2D grid
// has only sx/2 such lines; on 3D grids its 16 values per thread leave more warps
// resident than the four-step form's 32: 512^3 turnaround 1.06 -> 0.78 ms).
bool turn_split_form(int L);
// CUPSSGB_SPLIT=0/1 forces the four-step / split form of lines of 512 and 1024 points in
// the row pass and the generated turnaround (-1: not set, the automatic choice)
int split_override();

// xy-plane pass of a 3D phase with one channel and one product (plane.cuh), over the sz
// planes of nz batch members, c CTAs per plane.  plane_pass_shape: 0 when the grid
// (Lx = sx/2, sy) has no plane-pass instantiation or its plane does not fit on chip, else
// the cluster size (want_c when that one is instantiated, else the shape's default;
// CUPSSGB_PLANE_C sets want_c when it is 0), with *ps the plane-store pitch for nc input
// columns and *smem the dynamic shared memory of one CTA.
int plane_pass_shape(int Lx, int sy, int nc, int* ps, size_t* smem, int want_c = 0);
int plane_cluster_override();   // CUPSSGB_PLANE_C, or 0
cudaError_t launch_plane_pass(const PlaneParams& p, int Lx, int sy, int sz, int nz, int c, cudaStream_t st,
                              bool pdl);

cudaError_t launch_expand(const ExpandParams& p, cudaStream_t st);
cudaError_t launch_compress(const CompressParams& p, cudaStream_t st);
cudaError_t launch_mask(const MaskParams& p, cudaStream_t st);
// Advances the step count of every active member by inc.
cudaError_t launch_tick(MemberK* members, int n, uint32_t inc, cudaStream_t st, bool pdl = false);
// The same for the member tables of several grid classes, in one launch.
cudaError_t launch_tick_multi(const MultiTickParams& p, cudaStream_t st, bool pdl = false);
// Row pass of a grid class as the fused launch runs it (the form launch_row_pass would pick for
// nz members): single-input form, split form, threads per row (M), rows per CTA (RW), dynamic
// shared memory and CTAs along x.
struct RowShape {
  bool one, split;
  int m, rw;
  size_t smem;
  int blocks;
};
RowShape row_pass_shape(const XParams& p, int nz);

// per-L launchers (one translation unit per group of sizes)
#define CUPSSGB_DECL_LINE(L) \
  cudaError_t launch_line_##L(const LineParams& p, int nl, size_t smem, dim3 grid, cudaStream_t st, bool pdl);
CUPSSGB_DECL_LINE(1) CUPSSGB_DECL_LINE(2) CUPSSGB_DECL_LINE(4) CUPSSGB_DECL_LINE(8)
CUPSSGB_DECL_LINE(16) CUPSSGB_DECL_LINE(32) CUPSSGB_DECL_LINE(64) CUPSSGB_DECL_LINE(128)
CUPSSGB_DECL_LINE(256) CUPSSGB_DECL_LINE(512) CUPSSGB_DECL_LINE(1024)
CUPSSGB_DECL_LINE(6) CUPSSGB_DECL_LINE(12) CUPSSGB_DECL_LINE(24) CUPSSGB_DECL_LINE(48)
CUPSSGB_DECL_LINE(96) CUPSSGB_DECL_LINE(192)
#undef CUPSSGB_DECL_LINE

}  // namespace cupssgb
