// Instantiates line_pass<L, 1/2> and its launcher for one line length.
#pragma once
#include "kernels.cuh"
#include "launch.h"

#define CUPSSGB_LINE_INST(L)                                                                   \
  namespace cupssgb {                                                                          \
  cudaError_t launch_line_##L(const LineParams& p, int nl, size_t smem, dim3 grid,             \
                              cudaStream_t st) {                                               \
    static bool attr1 = false, attr2 = false;                                                  \
    dim3 block(p.W, LineCfg<L>::M, nl);                                                        \
    if (nl == 2) {                                                                             \
      if (!attr2) {                                                                            \
        cudaError_t e = cudaFuncSetAttribute(line_pass<L, 2>,                                  \
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,     \
                                             220 * 1024);                                      \
        if (e != cudaSuccess) return e;                                                        \
        attr2 = true;                                                                          \
      }                                                                                        \
      line_pass<L, 2><<<grid, block, smem, st>>>(p);                                           \
    } else {                                                                                   \
      if (!attr1) {                                                                            \
        cudaError_t e = cudaFuncSetAttribute(line_pass<L, 1>,                                  \
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,     \
                                             220 * 1024);                                      \
        if (e != cudaSuccess) return e;                                                        \
        attr1 = true;                                                                          \
      }                                                                                        \
      line_pass<L, 1><<<grid, block, smem, st>>>(p);                                           \
    }                                                                                          \
    return cudaGetLastError();                                                                 \
  }                                                                                            \
  }
