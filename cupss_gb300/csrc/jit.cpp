// Runtime specialisation of the turnaround kernel (NVRTC).
//
// The update program of a phase -- which fields, which terms (product / single field /
// constant), which q-monomials with which exponents, implicit and noise structure --
// is fixed once the equations are parsed.  The engine emits it as straight-line CUDA
// (numerical prefactor values stay in the kernel parameter block, so updateParameter
// needs no recompilation), compiles it for the running GPU with NVRTC and launches the
// cubin through the runtime's library API.  Compiled libraries are cached per process by
// device and source text, kernels by device, source and entry point: each device gets a
// build for its own architecture, with the shared-memory limit raised on that device.
#include "jit.h"

#include <nvrtc.h>

#include <algorithm>
#include <cstdlib>
#include <map>
#include <mutex>
#include <sstream>
#include <vector>

#include "engine.h"
#include "launch.h"
#include "jit_headers.inc"

namespace cupssgb {

namespace {

// Division and square root of the update programs (the implicit denominator, |q|,
// noise amplitudes, the Box-Muller radius) use the hardware approximations (about one
// ulp) instead of the IEEE-rounded sequences, whose range checks cost a branch and a
// dozen instructions per mode.
const char* const kJitFastOpts[] = {"--prec-div=false", "--prec-sqrt=false"};

std::mutex g_mu;
std::map<std::pair<int, std::string>, cudaLibrary_t> g_libs;   // (device, source) -> loaded library
std::map<std::pair<int, std::string>, cudaKernel_t> g_cache;   // (device, source + entry) -> kernel

std::string pow_expr(const char* base, int n) {
  if (n <= 0) return "";
  std::string s;
  for (int i = 0; i < n; ++i) s += std::string(i ? "*" : "") + base;
  return "*(" + s + ")";
}

// keep-test of one prefactor on the half spectrum (see term_mult in point_math.cuh)
std::string keep_expr(int s, const PresK& p, bool* never) {
  const int a = p.iqx & 1, b = p.iqy & 1, c = p.iqz & 1;
  *never = false;
  if (!a && !b && !c) {
    if (s & 1) *never = true;
    return "";
  }
  std::ostringstream os;
  os << "(((" << (s & 1);
  if (a) os << " ^ (vp.nyx ? 0 : 1)";
  if (b) os << " ^ (vp.nyy ? 0 : 1)";
  if (c) os << " ^ (vp.nyz ? 0 : 1)";
  os << ") & 1) == 0)";
  return os.str();
}

}  // namespace

namespace {

// struct GenProg: the update program of the phase described by p (see jit_generate_turn).
std::string gen_prog(const LineParams& p, bool batched) {
  // numerical values: the parameter block (one system) or the batch member's row
  auto pre = [&](int k) {
    return batched ? "__ldg(mv + " + std::to_string(k) + ")" : "P.pres[" + std::to_string(k) + "].pre";
  };
  auto nbase = [&](int fi) {
    return batched ? "__ldg(mv + kMaxPres + " + std::to_string(fi) + ")"
                   : "P.f[" + std::to_string(fi) + "].noise_base";
  };
  std::ostringstream o;
  o << "struct GenProg {\n"
    << "  static constexpr bool kUnroll = true;\n"
    << "  template <class F>\n"
    << "  __device__ __forceinline__ static float2 eval(const LineParams& P, int fi, const VPoint& vp, "
       "const F& fx) {\n"
    << "    const float q2 = vp.q2;\n"
    << (batched ? "    const float* mv = P.mvals + (size_t)blockIdx.z * kMemberVals;\n" : "")
    << "    switch (fi) {\n";
  for (int fi = 0; fi < p.nf; ++fi) {
    const FieldK& K = p.f[fi];
    bool need_iq = false, need_iqd = false;
    for (int t = 0; t < K.nterms; ++t) {
      const TermK& T = p.term[K.term0 + t];
      for (int j = 0; j < T.npres; ++j) need_iq |= p.pres[T.pres0 + j].invq > 0;
    }
    if (K.noisy && K.noise_invq) need_iq = true;
    for (int j = 0; j < K.nimp; ++j)
      if (p.pres[K.imp0 + j].invq != 0) (K.dynamic ? need_iqd : need_iq) = true;
    o << "      case " << fi << ": {\n";
    if (need_iq) o << "        const float iq = vp.origin ? 0.f : 1.0f / sqrtf(q2);\n";
    if (need_iqd) o << "        const float iqd = (vp.kx > 0 || vp.ky > 0) ? 1.0f / sqrtf(q2) : 0.f;\n";
    o << "        float2 acc = make_float2(0.f, 0.f);\n";
    for (int t = 0; t < K.nterms; ++t) {
      const TermK& T = p.term[K.term0 + t];
      if (T.kind == kTermMerged) continue;   // summed into another term's product channel
      o << "        {\n          float mt = 0.f;\n";
      for (int j = 0; j < T.npres; ++j) {
        const PresK& pr = p.pres[T.pres0 + j];
        bool never = false;
        const std::string keep = keep_expr(T.s, pr, &never);
        if (never) continue;
        std::ostringstream term;
        term << pre(T.pres0 + j) << pow_expr("q2", pr.q2n) << pow_expr("vp.qx", pr.iqx)
             << pow_expr("vp.qy", pr.iqy) << pow_expr("vp.qz", pr.iqz) << pow_expr("iq", pr.invq);
        if (keep.empty()) o << "          mt += " << term.str() << ";\n";
        else o << "          if " << keep << " mt += " << term.str() << ";\n";
      }
      if (T.kind == kTermProduct) o << "          const float2 src = fx.prod(" << T.src << ");\n";
      else if (T.kind == kTermSingle) o << "          const float2 src = fx.src(" << T.src << ");\n";
      else
        o << "          const float2 src = vp.origin ? make_float2((float)P.sx * (float)P.sy * (float)P.sz, "
             "0.f) : make_float2(0.f, 0.f);\n";
      o << "          float2 c = c_scale(src, mt);\n";
      if (T.s) o << "          c = c_muli(c);\n";
      o << "          acc = c_add(acc, c);\n        }\n";
    }
    std::ostringstream amp;
    if (K.noisy) {
      amp << nbase(fi);
      if (K.noise_q2n) amp << "*sqrtf(1.f" << pow_expr("q2", K.noise_q2n) << ")";
      if (K.noise_invq) amp << "*sqrtf(1.f" << pow_expr("iq", K.noise_invq) << ")";
    }
    const std::string noise = "fx.xi";
    std::ostringstream imp;
    for (int j = 0; j < K.nimp; ++j) {
      const PresK& pr = p.pres[K.imp0 + j];
      imp << (j ? " + " : "") << pre(K.imp0 + j) << pow_expr("q2", pr.q2n)
          << pow_expr(K.dynamic ? "iqd" : "iq", pr.invq);
    }
    if (K.dynamic) {
      o << "        float2 nv = c_add(fx.src(" << K.self_src << "), c_scale(acc, P.dt));\n";
      if (K.noisy) o << "        nv = c_add(nv, c_scale(" << noise << ", " << amp.str() << "));\n";
      if (K.nimp > 0)
        o << "        { const float rd = 1.0f / (1.f - P.dt * (" << imp.str()
          << ")); nv = make_float2(nv.x * rd, nv.y * rd); }\n";
    } else {
      if (K.nterms > 0) o << "        float2 nv = acc;\n";
      else o << "        float2 nv = fx.src(" << K.self_src << ");\n";
      if (K.noisy) {
        if (K.nterms > 0) o << "        nv = c_add(nv, c_scale(" << noise << ", " << amp.str() << "));\n";
        else o << "        nv = c_scale(" << noise << ", " << amp.str() << ");\n";
      }
      if (K.nimp > 0)
        o << "        if (!vp.origin) { const float rd = 1.0f / (" << imp.str()
          << "); nv = make_float2(nv.x * rd, nv.y * rd); }\n";
    }
    o << "        return nv;\n      }\n";
  }
  o << "    }\n    return make_float2(0.f, 0.f);\n  }\n};\n";
  return o.str();
}

// struct <name>: the phase structure and grid a turnaround is specialised for.
std::string gen_spec(const LineParams& p, const std::string& name, bool early_noise, bool split) {
  std::ostringstream o;
  o << "struct " << name << " {\n"
    << "  static constexpr int kNF = " << p.nf << ";\n"
    << "  static constexpr int kNProd = " << p.n_prod << ";\n"
    << "  static constexpr int kSX = " << p.sx << ", kSY = " << p.sy << ", kSZ = " << p.sz << ";\n"
    << "  static constexpr int kW = " << p.W << ";\n"
    << "  static constexpr bool kEarlyNoise = " << (early_noise ? "true" : "false") << ";\n"
    << "  static constexpr bool kSplit = " << (split ? "true" : "false") << ";\n"
    << "};\n";
  return o.str();
}

// overlap of the first field's noise with the first product's loads: for spectra that
// do not stay in the L2 (64 MB and more per array); CUPSSGB_EARLY_NOISE=0/1 overrides
bool early_noise_for(const LineParams& p) {
  bool early = (double)p.Lx * p.sy * p.sz * 8.0 >= 64.0 * 1024 * 1024;
  if (const char* e = std::getenv("CUPSSGB_EARLY_NOISE")) early = std::string(e) == "1";
  return early;
}

}  // namespace

std::string jit_generate_turn(const LineParams& p, int L, int NL, int warps, bool batched, bool split_form) {
  // block = (W, M, NL) threads
  const bool split = split_form && L >= 512;
  const int M = line_threads(L, 1, 1, split);   // LineCfg<L, split>::M
  const int threads = p.W > 0 ? p.W * M * NL : 256;
  const int min_blocks = std::max(1, warps * 32 / threads);
  std::ostringstream o;
  o << "#include \"turn.cuh\"\n"
    << "namespace cupssgb {\n"
    << gen_prog(p, batched) << gen_spec(p, "GenSpec", early_noise_for(p), split)
    << "}  // namespace cupssgb\n"
    << "extern \"C\" __global__ void __launch_bounds__(" << threads << ", " << min_blocks
    << ") cupssgb_turn(const cupssgb::LineParams P) {\n"
    << "  cupssgb::turn_body<" << L << ", " << NL << ", cupssgb::GenProg, cupssgb::GenSpec>(P);\n}\n";
  return o.str();
}

std::string jit_program_text(const LineParams& p, bool batched) { return gen_prog(p, batched); }

std::string jit_generate_multi(const std::vector<MultiClassSpec>& cls, bool has_row, bool batched, int turn_threads,
                               int turn_min_blocks, int row_min_blocks) {
  std::ostringstream o;
  o << "#include \"turn.cuh\"\n#include \"kernels.cuh\"\nnamespace cupssgb {\n" << gen_prog(cls[0].turn, batched);
  for (size_t c = 0; c < cls.size(); ++c)
    o << gen_spec(cls[c].turn, "GenSpec" + std::to_string(c), early_noise_for(cls[c].turn), cls[c].split);
  o << "}  // namespace cupssgb\n";
  // turnaround: flat blocks of turn_threads = W_c * M_c threads
  o << "extern \"C\" __global__ void __launch_bounds__(" << turn_threads << ", " << turn_min_blocks
    << ") cupssgb_turn_multi(const cupssgb::MultiTurnParams MP) {\n"
    << "  const int bx = blockIdx.x;\n  const int tid = threadIdx.x;\n";
  int b0 = 0;
  for (size_t c = 0; c < cls.size(); ++c) {
    const int b1 = b0 + cls[c].turn_tiles;
    const int W = cls[c].turn.W;
    o << "  " << (c ? "else " : "") << "if (bx < " << b1 << ") {\n"
      << "    if ((int)blockIdx.z >= MP.span[" << c << "]) return;\n"
      << "    cupssgb::turn_body_at<" << cls[c].L << ", 1, cupssgb::GenProg, cupssgb::GenSpec" << c << ">(MP.p[" << c
      << "], bx - " << b0 << ", 0, tid % " << W << ", tid / " << W << ", 0);\n  }\n";
    b0 = b1;
  }
  o << "}\n";
  if (has_row) {
    o << "extern \"C\" __global__ void __launch_bounds__(128, " << row_min_blocks
      << ") cupssgb_row_multi(const cupssgb::MultiRowParams MP) {\n"
      << "  const int bx = blockIdx.x;\n  const int tid = threadIdx.x;\n";
    b0 = 0;
    for (size_t c = 0; c < cls.size(); ++c) {
      const int b1 = b0 + cls[c].row_blocks;
      const int M = cls[c].row_m;
      o << "  " << (c ? "else " : "") << "if (bx < " << b1 << ") {\n"
        << "    if ((int)blockIdx.z >= MP.span[" << c << "]) return;\n"
        << "    cupssgb::" << (cls[c].row_one ? "row_one_body" : "row_pass_body") << "<" << cls[c].LX << ", "
        << (cls[c].row_split ? "true" : "false") << ">(MP.x[" << c << "], bx - " << b0 << ", tid % " << M
        << ", tid / " << M << ");\n  }\n";
      b0 = b1;
    }
    o << "}\n";
  }
  return o.str();
}

cudaKernel_t jit_kernel(const std::string& source, const char* entry) {
  std::lock_guard<std::mutex> lk(g_mu);
  int dev = 0, major = 0, minor = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) throw Error(kErrCuda, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  const std::pair<int, std::string> kkey{dev, source + '\n' + entry};
  auto it = g_cache.find(kkey);
  if (it != g_cache.end()) return it->second;
  cudaLibrary_t lib = nullptr;
  auto lit = g_libs.find({dev, source});
  if (lit != g_libs.end()) {
    lib = lit->second;
  } else {
    if (cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess)
      throw Error(kErrCuda, "compute capability query failed");
    // sm_103a on GB300; other Blackwell parts get their own arch-specific target
    const std::string arch = "--gpu-architecture=sm_" + std::to_string(major * 10 + minor) + "a";
    nvrtcProgram prog;
    if (nvrtcCreateProgram(&prog, source.c_str(), "cupssgb_turn.cu", kJitNumHeaders, kJitHeaderSources,
                           kJitHeaderNames) != NVRTC_SUCCESS)
      throw Error(kErrCuda, "nvrtcCreateProgram failed");
    const char* opts[] = {arch.c_str(), "--std=c++17", "-lineinfo", kJitFastOpts[0], kJitFastOpts[1]};
    const nvrtcResult rc = nvrtcCompileProgram(prog, 5, opts);
    if (rc != NVRTC_SUCCESS) {
      size_t n = 0;
      nvrtcGetProgramLogSize(prog, &n);
      std::string log(n, '\0');
      nvrtcGetProgramLog(prog, &log[0]);
      nvrtcDestroyProgram(&prog);
      throw Error(kErrCuda, "NVRTC compilation of the update program failed:\n" + log);
    }
    size_t n = 0;
    nvrtcGetCUBINSize(prog, &n);
    std::vector<char> cubin(n);
    nvrtcGetCUBIN(prog, cubin.data());
    nvrtcDestroyProgram(&prog);
    e = cudaLibraryLoadData(&lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e != cudaSuccess) throw Error(kErrCuda, std::string("cudaLibraryLoadData: ") + cudaGetErrorString(e));
    g_libs[{dev, source}] = lib;
  }
  cudaKernel_t k;
  e = cudaLibraryGetKernel(&k, lib, entry);
  if (e != cudaSuccess) throw Error(kErrCuda, std::string("cudaLibraryGetKernel: ") + cudaGetErrorString(e));
  e = cudaFuncSetAttribute((const void*)k, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
  if (e != cudaSuccess) throw Error(kErrCuda, std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
  g_cache[kkey] = k;
  return k;
}

std::string jit_compile_only(const std::string& source, size_t* cubin_bytes) {
  nvrtcProgram prog;
  if (nvrtcCreateProgram(&prog, source.c_str(), "cupssgb_turn.cu", kJitNumHeaders, kJitHeaderSources,
                         kJitHeaderNames) != NVRTC_SUCCESS)
    return "nvrtcCreateProgram failed";
  const char* opts[] = {"--gpu-architecture=sm_103a", "--std=c++17", "-lineinfo", kJitFastOpts[0], kJitFastOpts[1]};
  const nvrtcResult rc = nvrtcCompileProgram(prog, 5, opts);
  size_t n = 0;
  nvrtcGetProgramLogSize(prog, &n);
  std::string log(n, '\0');
  nvrtcGetProgramLog(prog, &log[0]);
  if (rc == NVRTC_SUCCESS && cubin_bytes) nvrtcGetCUBINSize(prog, cubin_bytes);
  nvrtcDestroyProgram(&prog);
  return rc == NVRTC_SUCCESS ? std::string() : log;
}

}  // namespace cupssgb
