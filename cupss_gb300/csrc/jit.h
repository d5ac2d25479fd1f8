// Runtime-specialised turnaround kernels (see jit.cpp).
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "engine_types.h"

namespace cupssgb {

// CUDA source of the turnaround kernel `cupssgb_turn` specialised to the update
// program described by p (its fields, terms and prefactor exponents), the grid
// (p.sx, p.sy, p.sz), L, NL, and, when p.W > 0, the tile width (p.W = 0: the width
// is read from the parameter block at run time).
// warps: resident warps per SM the kernel's register budget is sized for (the
// __launch_bounds__ minimum block count is warps * 32 / threads per block; with a
// width-generic kernel, p.W = 0, blocks of 256 threads are assumed).
// batched: numerical values come from the batch member's row of P.mvals.
// split: lines of 512 and 1024 points in the split FFT form (turn_split_form(L) is the
// automatic choice).
std::string jit_generate_turn(const LineParams& p, int L, int NL, int warps, bool batched, bool split);
// Compiles (once per source text) and returns the kernel handle.  Throws Error.
cudaKernel_t jit_kernel(const std::string& source, const char* entry);
// Compiles for sm_103a without loading (no GPU needed); returns "" or the log.
std::string jit_compile_only(const std::string& source, size_t* cubin_bytes);

}  // namespace cupssgb
