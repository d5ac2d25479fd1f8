// Line-pass dispatch and the spectrum expansion kernel.
#include <cstdlib>
#include "kernels.cuh"
#include "launch.h"

namespace cupssgb {

static_assert(LineCfg<1>::M == 1 && LineCfg<8>::M == 2 && LineCfg<16>::M == 4 && LineCfg<256>::M == 16 &&
                  LineCfg<512>::M == 16 && LineCfg<1024>::M == 32 && LineCfg<256, true>::M == 16 &&
                  LineCfg<512, true>::M == 32 && LineCfg<1024, true>::M == 64 && LineCfg<96>::M == 4 &&
                  LineCfg<192>::M == 8 && LineCfg<6>::M == 1,
              "line_m_of must follow LineCfg");
static int pl_of(int L, bool split) { return L + L / line_m_of(L, split); }

size_t line_pass_smem(int L, int nl, int W, int nslots, bool split) {
  return (size_t)nslots * nl * pl_of(L, split) * W * sizeof(float2);
}
int line_threads(int L, int nl, int W, bool split) { return W * line_m_of(L, split) * nl; }
int split_override() {
  static const int v = [] {
    const char* e = std::getenv("CUPSSGB_SPLIT");
    return e ? (std::atoi(e) != 0 ? 1 : 0) : -1;
  }();
  return v;
}
bool turn_split_form(int L) {
  if (L < 512) return false;
  const int o = split_override();
  return o < 0 || o == 1;   // automatic: the split form
}

cudaError_t launch_line_pass(const LineParams& p, int nl, int nslots, dim3 grid, cudaStream_t st, bool pdl) {
  const size_t smem = line_pass_smem(p.L, nl, p.W, nslots > 0 ? nslots : 1);
  switch (p.L) {
    case 1: return launch_line_1(p, nl, smem, grid, st, pdl);
    case 2: return launch_line_2(p, nl, smem, grid, st, pdl);
    case 4: return launch_line_4(p, nl, smem, grid, st, pdl);
    case 8: return launch_line_8(p, nl, smem, grid, st, pdl);
    case 16: return launch_line_16(p, nl, smem, grid, st, pdl);
    case 32: return launch_line_32(p, nl, smem, grid, st, pdl);
    case 64: return launch_line_64(p, nl, smem, grid, st, pdl);
    case 128: return launch_line_128(p, nl, smem, grid, st, pdl);
    case 256: return launch_line_256(p, nl, smem, grid, st, pdl);
    case 512: return launch_line_512(p, nl, smem, grid, st, pdl);
    case 1024: return launch_line_1024(p, nl, smem, grid, st, pdl);
    case 6: return launch_line_6(p, nl, smem, grid, st, pdl);
    case 12: return launch_line_12(p, nl, smem, grid, st, pdl);
    case 24: return launch_line_24(p, nl, smem, grid, st, pdl);
    case 48: return launch_line_48(p, nl, smem, grid, st, pdl);
    case 96: return launch_line_96(p, nl, smem, grid, st, pdl);
    case 192: return launch_line_192(p, nl, smem, grid, st, pdl);
    default: return cudaErrorInvalidValue;
  }
}

__global__ void expand_spectrum(const ExpandParams p) {
  const size_t N = (size_t)p.sx * p.sy * p.sz;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < N;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int kx = (int)(idx % p.sx);
    const int ky = (int)((idx / p.sx) % p.sy);
    const int kz = (int)(idx / ((size_t)p.sx * p.sy));
    const int pky = neg_mod(ky, p.sy);
    const int pkz = neg_mod(kz, p.sz);
    float2 out;
    if (kx > 0 && 2 * kx < p.sx) {
      out = p.spec[((size_t)kz * p.sy + ky) * p.Lx + kx];
    } else if (2 * kx > p.sx) {
      out = c_conj(p.spec[((size_t)pkz * p.sy + pky) * p.Lx + (p.sx - kx)]);
    } else {
      const float2 z = p.spec[((size_t)kz * p.sy + ky) * p.Lx];
      const float2 zp = p.spec[((size_t)pkz * p.sy + pky) * p.Lx];
      out = unpack(z, zp, kx == 0 ? 0 : 1);
    }
    p.full[idx] = out;
  }
}

__global__ void compress_spectrum(const CompressParams p) {
  const size_t H = (size_t)p.Lx * p.sy * p.sz;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < H;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int kx = (int)(idx % p.Lx);
    const int ky = (int)((idx / p.Lx) % p.sy);
    const int kz = (int)(idx / ((size_t)p.Lx * p.sy));
    const int pky = neg_mod(ky, p.sy);
    const int pkz = neg_mod(kz, p.sz);
    const size_t row = ((size_t)kz * p.sy + ky) * p.sx, prow = ((size_t)pkz * p.sy + pky) * p.sx;
    float2 out;
    if (kx > 0) {
      // (F(k) + conj F(-k)) / 2, -k = (sx - kx, -ky, -kz)
      out = c_scale(c_add(p.full[row + kx], c_conj(p.full[prow + (p.sx - kx)])), 0.5f);
    } else {
      const float2 c0 = c_scale(c_add(p.full[row], c_conj(p.full[prow])), 0.5f);
      const int nx = p.sx / 2;
      const float2 cn = c_scale(c_add(p.full[row + nx], c_conj(p.full[prow + nx])), 0.5f);
      out = c_add(c0, c_muli(cn));
    }
    p.spec[idx] = out;
  }
}

__global__ void mask_spectrum(const MaskParams p) {
  const size_t H = (size_t)p.Lx * p.sy * p.sz;
  for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < H;
       idx += (size_t)gridDim.x * blockDim.x) {
    const int kx = (int)(idx % p.Lx);
    const int ky = (int)((idx / p.Lx) % p.sy);
    const int kz = (int)(idx / ((size_t)p.Lx * p.sy));
    auto keep = [&](int k, int n, int lim) { return ((k > (n >> 1)) ? n - k : k) <= lim; };
    const bool kyz = keep(ky, p.sy, p.ylim) && keep(kz, p.sz, p.zlim);
    float2 out = make_float2(0.f, 0.f);
    if (kx > 0) {
      if (kyz && keep(kx, p.sx, p.xlim)) out = c_scale(p.spec[idx], p.scale);
    } else {
      const int pky = neg_mod(ky, p.sy);
      const int pkz = neg_mod(kz, p.sz);
      const float2 z = p.spec[idx];
      const float2 zp = p.spec[((size_t)pkz * p.sy + pky) * p.Lx];
      const float2 c0 = unpack(z, zp, 0), cn = unpack(z, zp, 1);
      const float2 a = kyz ? c_scale(c0, p.scale) : make_float2(0.f, 0.f);
      const float2 b = (kyz && keep(p.sx / 2, p.sx, p.xlim)) ? c_scale(cn, p.scale) : make_float2(0.f, 0.f);
      out = c_add(a, c_muli(b));
    }
    p.out[idx] = out;
  }
}

__global__ void tick_members(MemberK* m, int n, uint32_t inc) {
  grid_dep_sync();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && m[i].active) m[i].step += inc;
}

cudaError_t launch_tick(MemberK* members, int n, uint32_t inc, cudaStream_t st, bool pdl) {
  LaunchCfg lc(dim3((n + 255) / 256), dim3(256), 0, st, pdl);
  return cudaLaunchKernelEx(&lc.cfg, tick_members, members, n, inc);
}

// blockIdx.y = grid class
__global__ void tick_members_multi(const MultiTickParams p) {
  grid_dep_sync();
  const int c = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < p.nc && i < p.n[c] && p.members[c][i].active) p.members[c][i].step += p.inc;
}

cudaError_t launch_tick_multi(const MultiTickParams& p, cudaStream_t st, bool pdl) {
  int nmax = 1;
  for (int c = 0; c < p.nc; ++c) nmax = p.n[c] > nmax ? p.n[c] : nmax;
  LaunchCfg lc(dim3((nmax + 255) / 256, p.nc), dim3(256), 0, st, pdl);
  return cudaLaunchKernelEx(&lc.cfg, tick_members_multi, p);
}

cudaError_t launch_compress(const CompressParams& p, cudaStream_t st) {
  const size_t H = (size_t)p.Lx * p.sy * p.sz;
  int blocks = (int)((H + 255) / 256);
  if (blocks > 152 * 16) blocks = 152 * 16;
  compress_spectrum<<<blocks, 256, 0, st>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_mask(const MaskParams& p, cudaStream_t st) {
  const size_t H = (size_t)p.Lx * p.sy * p.sz;
  int blocks = (int)((H + 255) / 256);
  if (blocks > 152 * 16) blocks = 152 * 16;
  mask_spectrum<<<blocks, 256, 0, st>>>(p);
  return cudaGetLastError();
}

cudaError_t launch_expand(const ExpandParams& p, cudaStream_t st) {
  const size_t N = (size_t)p.sx * p.sy * p.sz;
  int blocks = (int)((N + 255) / 256);
  if (blocks > 152 * 16) blocks = 152 * 16;
  expand_spectrum<<<blocks, 256, 0, st>>>(p);
  return cudaGetLastError();
}

}  // namespace cupssgb
