// Instantiates line_pass<L>, turn_pass<L, 1/2> and the launcher for one line length.
#pragma once
#include "kernels.cuh"
#include "launch.h"
#include "turn.cuh"

namespace cupssgb {
template <class K>
static cudaError_t set_smem_attr(K kernel, std::atomic<unsigned long long>& done) {
  return raise_smem_limit((const void*)kernel, done);
}
}  // namespace cupssgb

#define CUPSSGB_LINE_INST(L)                                                                    \
  namespace cupssgb {                                                                           \
  cudaError_t launch_line_##L(const LineParams& p, int nl, size_t smem, dim3 grid,              \
                              cudaStream_t st, bool pdl) {                                      \
    static std::atomic<unsigned long long> a0{0}, a1{0}, a2{0}; /* devices with the smem limit */ \
    LaunchCfg lc(grid, dim3(p.W, LineCfg<L>::M, nl), smem, st, pdl);                            \
    cudaError_t e = cudaSuccess;                                                                \
    if (p.mode != kModeTurn) {                                                                  \
      e = set_smem_attr(line_pass<L>, a0);                                                      \
      if (e == cudaSuccess) e = cudaLaunchKernelEx(&lc.cfg, line_pass<L>, p);                   \
    } else if (nl == 2) {                                                                       \
      e = set_smem_attr(turn_pass<L, 2>, a2);                                                   \
      if (e == cudaSuccess) e = cudaLaunchKernelEx(&lc.cfg, turn_pass<L, 2>, p);                \
    } else {                                                                                    \
      e = set_smem_attr(turn_pass<L, 1>, a1);                                                   \
      if (e == cudaSuccess) e = cudaLaunchKernelEx(&lc.cfg, turn_pass<L, 1>, p);                \
    }                                                                                           \
    return e;                                                                                   \
  }                                                                                             \
  }
