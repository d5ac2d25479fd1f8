// Row-pass instantiations and dispatch by Lx = sx/2.
#include "kernels.cuh"
#include "launch.h"

namespace cupssgb {

// One spectral input raised to one spectral product (phi^n): the register-resident form.
static bool row_is_one(const XParams& p) {
  return p.n_in == 1 && p.n_prod == 1 && p.in_mode == kXInSpectral && p.out_mode == kXOutSpectral &&
         p.prod_n[0] >= 1 && p.prod_f[0][0] == 0;
}

template <int LX>
static cudaError_t launch_row_t(const XParams& p, cudaStream_t st, int nz, bool pdl) {
  using C = RowCfg<LX>;
  static bool attr = false, attr_one = false;
  dim3 block(C::M, C::RW);
  dim3 grid((p.rows + C::RW - 1) / C::RW, 1, nz);
  if (row_is_one(p)) {
    const size_t smem = 2 * (size_t)C::RW * C::PL * sizeof(float2);   // two transpose buffers
    if (!attr_one) {
      cudaError_t e = cudaFuncSetAttribute(row_pass_one<LX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           220 * 1024);
      if (e != cudaSuccess) return e;
      attr_one = true;
    }
    LaunchCfg lc(grid, block, smem, st, pdl);
    return cudaLaunchKernelEx(&lc.cfg, row_pass_one<LX>, p);
  }
  const size_t smem = (size_t)(1 + p.n_in) * C::RW * C::PL * sizeof(float2);
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(row_pass<LX>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         220 * 1024);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  LaunchCfg lc(grid, block, smem, st, pdl);
  return cudaLaunchKernelEx(&lc.cfg, row_pass<LX>, p);
}

template <int LX>
static size_t row_smem_t(int n_in) {
  using C = RowCfg<LX>;
  return (size_t)(1 + n_in) * C::RW * C::PL * sizeof(float2);
}

cudaError_t launch_row_pass(const XParams& p, cudaStream_t st, int nz, bool pdl) {
  switch (p.Lx) {
    case 1: return launch_row_t<1>(p, st, nz, pdl);
    case 2: return launch_row_t<2>(p, st, nz, pdl);
    case 4: return launch_row_t<4>(p, st, nz, pdl);
    case 8: return launch_row_t<8>(p, st, nz, pdl);
    case 16: return launch_row_t<16>(p, st, nz, pdl);
    case 32: return launch_row_t<32>(p, st, nz, pdl);
    case 64: return launch_row_t<64>(p, st, nz, pdl);
    case 128: return launch_row_t<128>(p, st, nz, pdl);
    case 256: return launch_row_t<256>(p, st, nz, pdl);
    case 512: return launch_row_t<512>(p, st, nz, pdl);
    case 1024: return launch_row_t<1024>(p, st, nz, pdl);
    default: return cudaErrorInvalidValue;
  }
}

size_t row_pass_smem(int Lx, int n_in) {
  switch (Lx) {
    case 1: return row_smem_t<1>(n_in);
    case 2: return row_smem_t<2>(n_in);
    case 4: return row_smem_t<4>(n_in);
    case 8: return row_smem_t<8>(n_in);
    case 16: return row_smem_t<16>(n_in);
    case 32: return row_smem_t<32>(n_in);
    case 64: return row_smem_t<64>(n_in);
    case 128: return row_smem_t<128>(n_in);
    case 256: return row_smem_t<256>(n_in);
    case 512: return row_smem_t<512>(n_in);
    case 1024: return row_smem_t<1024>(n_in);
    default: return 0;
  }
}

}  // namespace cupssgb
