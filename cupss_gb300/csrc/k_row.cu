// Row-pass instantiations and dispatch by Lx = sx/2 (2^a up to 1024, 3 * 2^a up to 192).
#include "kernels.cuh"
#include "launch.h"

namespace cupssgb {

// One spectral input raised to one spectral product (phi^n): the register-resident form.
static bool row_is_one(const XParams& p) {
  return p.n_in == 1 && p.n_prod == 1 && p.in_mode == kXInSpectral && p.out_mode == kXOutSpectral &&
         p.prod_n[0] >= 1 && p.prod_f[0][0] == 0;
}

template <int LX, bool SP>
static cudaError_t launch_row_form(const XParams& p, cudaStream_t st, int nz, bool pdl) {
  using C = RowCfg<LX, SP>;
  static std::atomic<unsigned long long> attr{0}, attr_one{0};   // devices with the smem limit raised
  dim3 block(C::M, C::RW);
  dim3 grid((p.rows + C::RW - 1) / C::RW, 1, nz);
  if (row_is_one(p)) {
    const size_t smem = 2 * (size_t)C::RW * C::PL * sizeof(float2);   // two transpose buffers
    const cudaError_t e = raise_smem_limit((const void*)row_pass_one<LX, SP>, attr_one);
    if (e != cudaSuccess) return e;
    LaunchCfg lc(grid, block, smem, st, pdl);
    return cudaLaunchKernelEx(&lc.cfg, row_pass_one<LX, SP>, p);
  }
  const size_t smem = (size_t)(1 + p.n_in) * C::RW * C::PL * sizeof(float2);
  void (*kern)(const XParams) = nullptr;
  if constexpr (SP) {
    kern = row_pass_split<LX>;
  } else {
    kern = row_pass<LX>;
  }
  const cudaError_t e = raise_smem_limit((const void*)kern, attr);
  if (e != cudaSuccess) return e;
  LaunchCfg lc(grid, block, smem, st, pdl);
  return cudaLaunchKernelEx(&lc.cfg, kern, p);
}

// Rows of 512 and 1024 points take the split line FFT (four times / twice the threads
// per row) when the pass has few rows: a 2D grid has only sy rows, which the four-step
// form covers with a few warps per SM.  Passes over many rows (3D grids, large batches)
// keep the four-step form, whose shared-memory traffic is lower.
static bool row_split(int Lx, long long rows) {
  if (Lx < 512) return false;
  const int o = split_override();
  return o >= 0 ? o == 1 : rows * (long long)line_m_of(Lx, false) < 64LL * 1024;
}

template <int LX>
static cudaError_t launch_row_t(const XParams& p, cudaStream_t st, int nz, bool pdl) {
  if constexpr (LX >= 512) {
    if (row_split(LX, (long long)p.rows * nz)) return launch_row_form<LX, true>(p, st, nz, pdl);
  }
  return launch_row_form<LX, false>(p, st, nz, pdl);
}

template <int LX, bool SP>
static RowShape row_shape_form(const XParams& p) {
  using C = RowCfg<LX, SP>;
  RowShape r;
  r.one = row_is_one(p);
  r.split = SP;
  r.m = C::M;
  r.rw = C::RW;
  r.smem = (r.one ? 2 : (size_t)(1 + p.n_in)) * C::RW * C::PL * sizeof(float2);
  r.blocks = (p.rows + C::RW - 1) / C::RW;
  return r;
}

template <int LX>
static RowShape row_shape_t(const XParams& p, int nz) {
  if constexpr (LX >= 512) {
    if (row_split(LX, (long long)p.rows * nz)) return row_shape_form<LX, true>(p);
  }
  return row_shape_form<LX, false>(p);
}

RowShape row_pass_shape(const XParams& p, int nz) {
  switch (p.Lx) {
    case 16: return row_shape_t<16>(p, nz);
    case 32: return row_shape_t<32>(p, nz);
    case 64: return row_shape_t<64>(p, nz);
    case 128: return row_shape_t<128>(p, nz);
    case 256: return row_shape_t<256>(p, nz);
    case 512: return row_shape_t<512>(p, nz);
    case 1024: return row_shape_t<1024>(p, nz);
    case 24: return row_shape_t<24>(p, nz);
    case 48: return row_shape_t<48>(p, nz);
    case 96: return row_shape_t<96>(p, nz);
    case 192: return row_shape_t<192>(p, nz);
    default: return RowShape{false, false, 0, 0, 0, 0};
  }
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
    // rows of 3 * 2^a packed points (sx = 6 .. 384)
    case 3: return launch_row_t<3>(p, st, nz, pdl);
    case 6: return launch_row_t<6>(p, st, nz, pdl);
    case 12: return launch_row_t<12>(p, st, nz, pdl);
    case 24: return launch_row_t<24>(p, st, nz, pdl);
    case 48: return launch_row_t<48>(p, st, nz, pdl);
    case 96: return launch_row_t<96>(p, st, nz, pdl);
    case 192: return launch_row_t<192>(p, st, nz, pdl);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace cupssgb
