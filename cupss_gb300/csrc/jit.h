// Runtime-specialised turnaround kernels (see jit.cpp).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

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
// One grid class of a fused launch: batched solvers of one system structure on different
// 1D/2D grids stepped with one launch per kernel (engine_multi.cpp).
struct MultiClassSpec {
  LineParams turn;   // the class's turnaround parameters; W = its tile width in the fused block
  int L;             // line length (sy)
  bool split;        // split FFT form of its lines
  int turn_tiles;    // CTAs along x of its turnaround
  int LX;            // packed row length (row pass)
  bool row_one;      // single-input single-product row form
  bool row_split;    // split form of its rows
  int row_m;         // threads per row
  int row_blocks;    // CTAs along x of its row pass
};
// Source of the fused turnaround `cupssgb_turn_multi` (turn_threads threads per CTA, at
// least turn_min_blocks CTAs resident per SM) and,
// with has_row, the fused row pass `cupssgb_row_multi` (128 threads per CTA) of one phase:
// class c takes the blockIdx.x range after classes 0..c-1 and its members are
// blockIdx.z < span[c] (MultiTurnParams / MultiRowParams in engine_types.h).
std::string jit_generate_multi(const std::vector<MultiClassSpec>& cls, bool has_row, bool batched, int turn_threads,
                               int turn_min_blocks, int row_min_blocks);
// The update program alone (struct GenProg): equal for two phases exactly when their
// update structure is equal (fields, terms, exponents, implicit and noise structure).
std::string jit_program_text(const LineParams& p, bool batched);
// Compiles (once per source text) and returns the kernel handle.  Throws Error.
cudaKernel_t jit_kernel(const std::string& source, const char* entry);
// Compiles for sm_103a without loading (no GPU needed); returns "" or the log.
std::string jit_compile_only(const std::string& source, size_t* cubin_bytes);

}  // namespace cupssgb
