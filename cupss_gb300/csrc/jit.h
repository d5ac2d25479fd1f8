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
// min_blocks: the minimum resident CTAs per SM requested from the compiler.
// batched: numerical values come from the batch member's row of P.mvals.
std::string jit_generate_turn(const LineParams& p, int L, int NL, int min_blocks = 2, bool batched = false);
// Compiles (once per source text) and returns the kernel handle.  Throws Error.
cudaKernel_t jit_kernel(const std::string& source, const char* entry);
// Compiles for sm_103a without loading (no GPU needed); returns "" or the log.
std::string jit_compile_only(const std::string& source, size_t* cubin_bytes);

}  // namespace cupssgb
