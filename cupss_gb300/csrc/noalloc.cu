// Forward transform of a real field that never allocates device memory.
//
// Some callers cannot let a library call cudaMalloc: a host application that hands
// all device memory out of its own fixed arena (an allocation behind its back breaks
// its accounting, or simply fails because the arena already holds the whole GPU), or
// code that runs where a new allocation would stall or be refused.  For them this
// file keeps the transform's working memory in a file-scope device array of fixed
// size, reserved when the library is loaded and held by every GPU that loads it
// until the process exits.  The caller passes the input and the output.
//
// Working memory: the packed half spectrum of the field (sx*sy*sz/2 complex values)
// and the twiddle table.  Maximum field size: kNoAllocMaxPoints points.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/cupss_gb300.h"
#include "engine_types.h"
#include "launch.h"

namespace cupssgb {
void set_last_error(const std::string& msg);   // capi.cpp
}

namespace {

constexpr long long kNoAllocMaxPoints = 1ll << 21;                 // e.g. 128^3 or 2048 x 1024
constexpr size_t kNoAllocHalf = (size_t)(kNoAllocMaxPoints / 2);   // complex values
constexpr int kTwLen = 4096;                                       // tables for L = 1..2048

static __device__ __align__(256) float2 g_noalloc_spectrum[kNoAllocHalf];   // 8 MiB
static __device__ __align__(256) float2 g_noalloc_twiddles[kTwLen];        // 32 KiB

struct DeviceSetup {
  bool done = false;
  float2* spectrum = nullptr;
  float2* twiddles = nullptr;
};
std::mutex g_setup_mu;
DeviceSetup g_setup[64];

// error messages go to cupssgb_last_error() of the calling thread
struct ErrorSink {
  ErrorSink& operator=(const std::string& m) {
    cupssgb::set_last_error(m);
    return *this;
  }
  void clear() { cupssgb::set_last_error(std::string()); }
};
ErrorSink g_noalloc_error;

bool pow2(int n) { return n >= 1 && (n & (n - 1)) == 0; }

// Host-side addresses of the device arrays for the current device.  The array names
// are host-side stand-ins in host code; only cudaGetSymbolAddress yields the device
// address that a kernel argument needs.
int setup_current_device(DeviceSetup** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    g_noalloc_error = std::string("cudaGetDevice: ") + cudaGetErrorString(e);
    return CUPSSGB_ERR_CUDA;
  }
  if (dev < 0 || dev >= 64) {
    g_noalloc_error = "device index out of range";
    return CUPSSGB_ERR_INVALID;
  }
  std::lock_guard<std::mutex> lk(g_setup_mu);
  DeviceSetup& s = g_setup[dev];
  if (!s.done) {
    e = cudaGetSymbolAddress((void**)&s.spectrum, g_noalloc_spectrum);
    if (e != cudaSuccess) {
      g_noalloc_error = std::string("cudaGetSymbolAddress(spectrum): ") + cudaGetErrorString(e);
      return CUPSSGB_ERR_CUDA;
    }
    e = cudaGetSymbolAddress((void**)&s.twiddles, g_noalloc_twiddles);
    if (e != cudaSuccess) {
      g_noalloc_error = std::string("cudaGetSymbolAddress(twiddles): ") + cudaGetErrorString(e);
      return CUPSSGB_ERR_CUDA;
    }
    // twiddle super-table: the table for length L at offset L holds exp(-2 pi i j/L)
    std::vector<float2> h(kTwLen);
    h[0] = make_float2(0.f, 0.f);
    for (int L = 1; L <= kTwLen / 2; L *= 2)
      for (int j = 0; j < L; ++j) {
        const double a = -2.0 * M_PI * (double)j / (double)L;
        h[L + j] = make_float2((float)std::cos(a), (float)std::sin(a));
      }
    e = cudaMemcpy(s.twiddles, h.data(), kTwLen * sizeof(float2), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      g_noalloc_error = std::string("twiddle upload: ") + cudaGetErrorString(e);
      return CUPSSGB_ERR_CUDA;
    }
    s.done = true;
  }
  *out = &s;
  return CUPSSGB_OK;
}

void fill_line(cupssgb::LineParams& p, int sx, int sy, int sz, int L, int geo, int mode, const float2* tw) {
  std::memset(&p, 0, sizeof(p));
  p.sx = sx;
  p.sy = sy;
  p.sz = sz;
  p.Lx = sx / 2;
  p.L = L;
  p.geo = geo;
  p.mode = mode;
  p.tw = tw;
  int W = 16;
  while (W > p.Lx) W /= 2;
  if (W < 1) W = 1;
  while (W > 1 && cupssgb::line_threads(L, 1, W) > 256) W /= 2;
  p.W = W;
}

cudaError_t line_fwd(int sx, int sy, int sz, int geo, float2* data, const float2* tw, cudaStream_t st) {
  cupssgb::LineParams p;
  const int L = (geo == cupssgb::kGeoZ3) ? sz : sy;
  fill_line(p, sx, sy, sz, L, geo, cupssgb::kModeFwd, tw);
  p.n_prod = 1;
  p.prod_in[0] = data;
  p.prod_out[0] = data;
  p.inv_xlimit[0] = p.Lx;
  dim3 grid((p.Lx + p.W - 1) / p.W, geo == cupssgb::kGeoY3 ? sz : (geo == cupssgb::kGeoZ3 ? sy : 1));
  return cupssgb::launch_line_pass(p, 1, 1, grid, st);
}

}  // namespace

extern "C" int cupssgb_real_to_fourier_noalloc(const float* real_dev, float* fourier_dev, int sx, int sy, int sz,
                                               void* stream) {
  g_noalloc_error.clear();
  if (!real_dev || !fourier_dev) {
    g_noalloc_error = "real_dev / fourier_dev is NULL";
    return CUPSSGB_ERR_INVALID;
  }
  if (!pow2(sx) || sx < 2 || sx > 2048 || !pow2(sy) || sy > 1024 || !pow2(sz) || sz > 1024) {
    g_noalloc_error = "grid sizes must be powers of two: 2 <= sx <= 2048, 1 <= sy, sz <= 1024";
    return CUPSSGB_ERR_UNSUPPORTED;
  }
  const long long n = (long long)sx * sy * sz;
  if (n > kNoAllocMaxPoints) {
    g_noalloc_error = "field of " + std::to_string(n) + " points exceeds the fixed working memory of " +
                      std::to_string(kNoAllocMaxPoints) + " points";
    return CUPSSGB_ERR_LIMIT;
  }
  if (((uintptr_t)real_dev & 7u) != 0 || ((uintptr_t)fourier_dev & 7u) != 0) {
    g_noalloc_error = "real_dev and fourier_dev must be 8-byte aligned";
    return CUPSSGB_ERR_INVALID;
  }
  DeviceSetup* ds = nullptr;
  int rc = setup_current_device(&ds);
  if (rc != CUPSSGB_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  float2* spec = ds->spectrum;
  // every element of spec that is read below is first written by the row pass of this
  // call (all rows, all columns), so nothing has to be cleared between calls
  cupssgb::XParams x;
  std::memset(&x, 0, sizeof(x));
  x.Lx = sx / 2;
  x.rows = sy * sz;
  x.in_mode = cupssgb::kXInReal;
  x.out_mode = cupssgb::kXOutSpectral;
  x.out_scale = 1.f;
  x.n_in = 1;
  x.in[0] = reinterpret_cast<const float2*>(real_dev);
  x.n_prod = 1;
  x.out[0] = spec;
  x.prod_n[0] = 1;
  x.prod_f[0][0] = 0;
  x.tw = ds->twiddles;
  cudaError_t e = cupssgb::launch_row_pass(x, st);
  const int dim = (sz == 1 && sy == 1) ? 1 : (sz == 1 ? 2 : 3);
  if (e == cudaSuccess && dim == 3) e = line_fwd(sx, sy, sz, cupssgb::kGeoY3, spec, ds->twiddles, st);
  if (e == cudaSuccess && dim == 3) e = line_fwd(sx, sy, sz, cupssgb::kGeoZ3, spec, ds->twiddles, st);
  if (e == cudaSuccess && dim == 2) e = line_fwd(sx, sy, sz, cupssgb::kGeoCol, spec, ds->twiddles, st);
  if (e == cudaSuccess) {
    cupssgb::ExpandParams ep;
    ep.sx = sx;
    ep.sy = sy;
    ep.sz = sz;
    ep.Lx = sx / 2;
    ep.spec = spec;
    ep.full = reinterpret_cast<float2*>(fourier_dev);
    e = cupssgb::launch_expand(ep, st);
  }
  if (e != cudaSuccess) {
    g_noalloc_error = std::string("launch: ") + cudaGetErrorString(e);
    return CUPSSGB_ERR_CUDA;
  }
  return CUPSSGB_OK;
}

