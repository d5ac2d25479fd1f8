// Batches: one solver holding many independent systems of the same structure and grid.
//
// All member arrays of a field live in one allocation, member m at m * (Lx*sy*sz)
// elements, and every step launch covers all members with blockIdx.z = member.  What
// differs between members lives in device tables that the kernels index by
// blockIdx.z: the numerical prefactor values and noise amplitudes of each phase
// (LineParams::mvals) and the Philox key, step count and active flag (MemberK).  The
// step count advances on the device (one tiny kernel per step), so the launch
// parameters of a step do not change from step to step and whole runs of steps are
// replayed from CUDA graphs.  The turnaround tile width of each phase is picked at
// prepare by timing the candidates on the batch itself.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <sstream>

#include "engine.h"
#include "jit.h"
#include "launch.h"
#include "tune_cache.h"

namespace cupssgb {

void Solver::set_members(int n) {
  if (prepared_) throw Error(kErrState, "set_members after prepare");
  if (n < 1 || n > 65535) throw Error(kErrInvalid, "a batch holds 1 to 65535 members");
  nmem_ = n;
  mspan_ = n;
  batch_ = true;
  mfields_.clear();
  members_h_.assign(n, MemberK{0u, 0u, 0u, 1u});
  for (int m = 0; m < n; ++m) {
    // default: member m draws from seed + m (member 0 = the solver's seed)
    const uint64_t s = seed_ + (uint64_t)m;
    members_h_[m].key0 = (uint32_t)(s & 0xffffffffu);
    members_h_[m].key1 = (uint32_t)(s >> 32);
  }
}

void Solver::check_member(int m) const {
  if (m < 0 || m >= nmem_) throw Error(kErrInvalid, "bad member index");
}

void Solver::check_same_monomials(const std::vector<HostPres>& a, const std::vector<HostPres>& b) const {
  if (a.size() != b.size()) throw Error(kErrInvalid, "members differ only in prefactor values");
  for (size_t j = 0; j < a.size(); ++j)
    if (a[j].q2n != b[j].q2n || a[j].iqx != b[j].iqx || a[j].iqy != b[j].iqy || a[j].iqz != b[j].iqz ||
        a[j].invq != b[j].invq)
      throw Error(kErrInvalid, "members differ only in prefactor values, not in q-monomials");
}

namespace {
void ensure_member_fields(std::vector<std::vector<HostField>>& mf, int n, const std::vector<HostField>& base) {
  if ((int)mf.size() != n) mf.assign(n, base);
}
}  // namespace

void Solver::set_member_term_pres(int m, int f, int t, const std::vector<HostPres>& p) {
  if (!batch_) throw Error(kErrState, "not a batch");
  check_member(m);
  if (f < 0 || f >= nfields() || t < 0 || t >= (int)fields_[f].terms.size())
    throw Error(kErrInvalid, "bad term index");
  check_same_monomials(fields_[f].terms[t].pres, p);
  ensure_member_fields(mfields_, nmem_, fields_);
  mfields_[m][f].terms[t].pres = p;
  mvals_dirty_ = true;
  merge_check_ = prepared_;
}

void Solver::set_member_implicit(int m, int f, const std::vector<HostPres>& p) {
  if (!batch_) throw Error(kErrState, "not a batch");
  check_member(m);
  if (f < 0 || f >= nfields()) throw Error(kErrInvalid, "bad field index");
  check_same_monomials(fields_[f].implicit, p);
  ensure_member_fields(mfields_, nmem_, fields_);
  mfields_[m][f].implicit = p;
  mvals_dirty_ = true;
}

void Solver::set_member_noise(int m, int f, const HostPres& amp) {
  if (!batch_) throw Error(kErrState, "not a batch");
  check_member(m);
  if (f < 0 || f >= nfields()) throw Error(kErrInvalid, "bad field index");
  if (!fields_[f].noisy) throw Error(kErrInvalid, "the field has no noise");
  check_same_monomials({fields_[f].noise}, {amp});
  ensure_member_fields(mfields_, nmem_, fields_);
  mfields_[m][f].noise = amp;
  mvals_dirty_ = true;
}

void Solver::set_member_seed(int m, uint64_t seed) {
  if (!batch_) throw Error(kErrState, "not a batch");
  check_member(m);
  members_h_[m].key0 = (uint32_t)(seed & 0xffffffffu);
  members_h_[m].key1 = (uint32_t)(seed >> 32);
  if (prepared_)
    check(cudaMemcpyAsync(&members_d_[m].key0, &members_h_[m].key0, 2 * sizeof(uint32_t), cudaMemcpyHostToDevice,
                          stream_),
          "member key upload");
}

void Solver::set_member_active(int m, bool on) {
  if (!batch_) throw Error(kErrState, "not a batch");
  check_member(m);
  members_h_[m].active = on ? 1u : 0u;
  if (prepared_)
    check(cudaMemcpyAsync(&members_d_[m].active, &members_h_[m].active, sizeof(uint32_t), cudaMemcpyHostToDevice,
                          stream_),
          "member flag upload");
  // step launches cover members [0, last active]: a sparsely filled pool does not launch
  // (and retire) the CTAs of its empty slots beyond that
  int span = 1;
  for (int k = nmem_ - 1; k >= 0; --k)
    if (members_h_[k].active) {
      span = k + 1;
      break;
    }
  if (span != mspan_) {
    mspan_ = span;
    invalidate_graphs();
  }
}

void Solver::reset_member(int m) {
  if (!batch_) throw Error(kErrState, "not a batch");
  if (!prepared_) throw Error(kErrState, "reset_member before prepare");
  check_member(m);
  members_h_[m].step = 0u;
  check(cudaMemcpyAsync(&members_d_[m].step, &members_h_[m].step, sizeof(uint32_t), cudaMemcpyHostToDevice,
                        stream_),
        "member step upload");
  const size_t off = (size_t)m * half_, bytes = half_ * sizeof(float2);
  for (int f = 0; f < nfields(); ++f) {
    check(cudaMemsetAsync(state_[0][f] + off, 0, bytes, stream_), "member reset");
    check(cudaMemsetAsync(state_[1][f] + off, 0, bytes, stream_), "member reset");
    // the dealiased copies start at zero, as in a fresh solver
    if (chan_[f]) check(cudaMemsetAsync(chan_[f] + off, 0, bytes, stream_), "member reset");
    if (chanz_[f]) check(cudaMemsetAsync(chanz_[f] + off, 0, bytes, stream_), "member reset");
  }
}

long long Solver::member_step(int m) {
  if (!batch_) return step_;
  check_member(m);
  if (!prepared_) return 0;
  MemberK k;
  check(cudaStreamSynchronize(stream_), "member step sync");
  check(cudaMemcpy(&k, &members_d_[m], sizeof(MemberK), cudaMemcpyDeviceToHost), "member step read");
  return (long long)k.step;
}

void Solver::upload_member_values() {
  ensure_member_fields(mfields_, nmem_, fields_);
  std::vector<float> vals((size_t)nmem_ * kMemberVals);
  for (Phase& P : phases_) {
    if (P.fields.empty()) continue;
    std::fill(vals.begin(), vals.end(), 0.f);
    for (int m = 0; m < nmem_; ++m) {
      LineParams p;
      int nslots = 0;
      bool any_chan = false;
      fill_turn(P, p, nslots, any_chan, &mfields_[m]);
      float* row = vals.data() + (size_t)m * kMemberVals;
      for (int k = 0; k < kMaxPres; ++k) row[k] = p.pres[k].pre;
      for (int fi = 0; fi < p.nf; ++fi) row[kMaxPres + fi] = p.f[fi].noise_base;
    }
    // pageable source: the call returns once the data is staged
    check(cudaMemcpyAsync(mvals_d_[P.id], vals.data(), vals.size() * sizeof(float), cudaMemcpyHostToDevice,
                          stream_),
          "member value upload");
  }
  check(cudaStreamSynchronize(stream_), "member value upload");
  mvals_dirty_ = false;
}

void Solver::zero_dynamic_buffers() {
  const size_t bytes = half_ * (size_t)nmem_ * sizeof(float2);
  for (int f = 0; f < nfields(); ++f) {
    check(cudaMemsetAsync(state_[0][f], 0, bytes, stream_), "buffer reset");
    check(cudaMemsetAsync(state_[1][f], 0, bytes, stream_), "buffer reset");
    if (chan_[f]) check(cudaMemsetAsync(chan_[f], 0, bytes, stream_), "buffer reset");
    if (chanz_[f]) check(cudaMemsetAsync(chanz_[f], 0, bytes, stream_), "buffer reset");
  }
  for (Phase& P : phases_)
    for (float2* b : P.prodbuf)
      if (b) check(cudaMemsetAsync(b, 0, bytes, stream_), "buffer reset");
  std::fill(par_.begin(), par_.end(), 0);
}

// Autotuner.  For every phase it times the launch shapes of the phase on the solver
// itself (one warm-up and three timed runs of the whole phase per candidate) and keeps the
// fastest, one dimension after the other (2-4 only from 2^20 grid points times members on):
//   1. the turnaround's tile width W (up to four widths);
//   2. the resident-warp target its registers are sized for (16 and 24 warps per SM);
//   3. lines of 512 and 1024 points: the split or the four-step FFT form;
//   4. 3D plane mode, the phase with the product: CTAs per plane of the xy-plane pass.
// The phases run on the zeroed buffers of a freshly prepared solver; every buffer is
// zeroed again afterwards and no step is counted.  The winners are stored in the tune
// cache (tune_cache.cpp) under a key naming the GPU, the grid, the batch span and the
// phase's update program, and a later solver with the same key takes them from there
// without timing.  CUPSSGB_TUNE=0 skips all of it (rule-based shapes); CUPSSGB_TURN_W
// fixes W.
void Solver::autotune() {
  const int L = turn_len();
  const int nl = (dim_ == 3) ? 2 : 1;
  const char* te = std::getenv("CUPSSGB_TUNE");
  const bool tune_on = !(te && std::string(te) == "0");
  cudaEvent_t a, b;
  check(cudaEventCreate(&a), "cudaEventCreate");
  check(cudaEventCreate(&b), "cudaEventCreate");
  const long long l0 = launches_;
  tuning_ = true;
  const int span0 = mspan_;
  // time the members as they are (an ensemble: all of them); a pool prepared with every
  // slot free is timed with one member, the load a server pool mostly runs at
  std::vector<MemberK> all = members_h_;
  bool any = false;
  for (const MemberK& k : all) any = any || k.active != 0u;
  if (!any) {
    all[0].active = 1u;
    mspan_ = 1;
  }
  check(cudaMemcpyAsync(members_d_, all.data(), all.size() * sizeof(MemberK), cudaMemcpyHostToDevice, stream_),
        "member upload");
  bool plane_tuned = false;
  for (Phase& P : phases_) {
    P.tune_ms.clear();
    P.tune_cached = false;
    P.tune_pdl = -1;
    if (P.fields.empty()) continue;
    LineParams p;
    int nslots = 0;
    bool any_chan = false;
    fill_turn(P, p, nslots, any_chan);
    const int wmax = pick_w(L, nl, nslots, 0, phase_split(P));
    if (turn_w_ > 0) {
      P.tuned_w = std::min(turn_w_, wmax);
      continue;
    }
    if (!tune_on) continue;
    const std::string key = tune_key(P);
    std::string cached;
    if (tune_cache_lookup(key, &cached) && apply_tune_value(P, cached, wmax)) {
      P.tune_cached = true;
      if (!P.products.empty()) plane_tuned = true;
      continue;
    }
    auto time_phase = [&](const std::string& what) {
      run_phase(P);
      check(cudaEventRecord(a, stream_), "cudaEventRecord");
      for (int r = 0; r < 3; ++r) run_phase(P);
      check(cudaEventRecord(b, stream_), "cudaEventRecord");
      check(cudaEventSynchronize(b), "cudaEventSynchronize");
      float ms = 0.f;
      check(cudaEventElapsedTime(&ms, a, b), "cudaEventElapsedTime");
      P.tune_ms.push_back({what, ms / 3.0});
      return ms / 3.0;
    };
    // 1-3 in the phase's current form; returns the best time
    const bool deep = (double)npoints() * mspan_ >= (double)(1 << 20);
    std::string tag;   // label prefix of the candidates' times ("row:" when re-timed)
    auto shape_search = [&]() {
      // 1. tile width
      std::vector<int> cands;
      for (int w = wmax; w >= 2 && cands.size() < 4; w /= 2) cands.push_back(w);
      if (cands.empty()) cands.push_back(wmax);
      double best = 1e30;
      int best_w = wmax;
      for (int w : cands) {
        P.tuned_w = w;
        const double ms = time_phase(tag + "W=" + std::to_string(w));
        if (ms < best) {
          best = ms;
          best_w = w;
        }
      }
      P.tuned_w = best_w;
      // the other dimensions need kernels of their own (compiled at prepare); below 2^20
      // grid points (times members) a step is launch-bound and W is all that is timed
      if (use_jit_ && deep) {
        // 2. resident-warp target (a kernel compiled for each)
        const int w0 = phase_warps(P);
        const int alt = w0 == 16 ? 24 : 16;
        P.tuned_warps = alt;
        const double ms = time_phase(tag + "warps=" + std::to_string(alt));
        if (ms < best) best = ms;
        else P.tuned_warps = w0;
        // 3. FFT form of 512- and 1024-point lines (the width must suit the other form too)
        if (L >= 512 && split_override() < 0) {
          const bool s0 = phase_split(P);
          P.tuned_split = s0 ? 0 : 1;
          if (P.tuned_w <= pick_w(L, nl, nslots, 0, !s0)) {
            const double ms2 = time_phase(tag + "split=" + (s0 ? "0" : "1"));
            if (ms2 < best) best = ms2;
            else P.tuned_split = s0 ? 1 : 0;
          } else {
            P.tuned_split = s0 ? 1 : 0;
          }
        }
      }
      return best;
    };
    double best = shape_search();
    // 4. 3D products: the xy-plane pass (each instantiated cluster size) or the row pass
    //    with two y line passes (one choice per solver, made on its first product phase)
    if (plane_ok_ && plane_env_ < 0 && deep && !P.products.empty() && !plane_tuned) {
      plane_tuned = true;
      const int g = P.xin[0];
      const int nc = std::min(Lx_, sx_ / (alias_order_[g] + 1) + 1);
      if (plane_cluster_override() <= 0) {
        const int c0 = plane_pass_shape(Lx_, sy_, nc, nullptr, nullptr, plane_c_);
        for (int c : {1, 2, 4, 8}) {
          if (c == c0 || plane_pass_shape(Lx_, sy_, nc, nullptr, nullptr, c) != c) continue;
          const int keep = plane_c_;
          plane_c_ = c;
          const double ms = time_phase("plane_c=" + std::to_string(c));
          if (ms < best) best = ms;
          else plane_c_ = keep;
        }
      }
      plane_ = false;
      const double ms = time_phase("plane=0");
      if (ms < best) {
        // the row-pass form wins: its own tile width, warps and line form (1-3 above were
        // timed in the plane form)
        const int w1 = P.tuned_w, warps1 = P.tuned_warps, split1 = P.tuned_split;
        P.tuned_warps = 0;
        P.tuned_split = -1;
        tag = "row:";
        best = shape_search();
        if (ms < best) {   // the shape found in the plane form stays the faster
          best = ms;
          P.tuned_w = w1;
          P.tuned_warps = warps1;
          P.tuned_split = split1;
        }
      } else {
        plane_ = true;
      }
    }
    P.tune_best_ms = best;
    tune_cache_store(key, tune_value(P, best));
  }
  // 5. programmatic dependent launch, timed on whole 16-step graphs with and without it:
  //    it hides the launch gap between short kernels, but the next kernel's CTAs then hold
  //    SM slots (waiting for the previous kernel's end) that a kernel with a tail of CTAs
  //    could use -- measured either way on this GPU depending on the grid.
  if (tune_on && pdl_env_ < 0 && turn_w_ <= 0) {
    bool have = true;
    int cached_pdl = -1;
    for (const Phase& P : phases_) {
      if (P.fields.empty()) continue;
      if (!P.tune_cached || P.tune_pdl < 0) have = false;
      cached_pdl = P.tune_pdl;
    }
    if (have && cached_pdl >= 0) {
      pdl_ = cached_pdl == 1;
    } else {
      const long long s0 = step_;
      auto time_graph = [&](bool on) {
        pdl_ = on;
        invalidate_graphs();
        run_graph(0);   // captured and run once: warm-up
        check(cudaEventRecord(a, stream_), "cudaEventRecord");
        run_graph(0);
        run_graph(0);
        check(cudaEventRecord(b, stream_), "cudaEventRecord");
        check(cudaEventSynchronize(b), "cudaEventSynchronize");
        float ms = 0.f;
        check(cudaEventElapsedTime(&ms, a, b), "cudaEventElapsedTime");
        return (double)ms / (2 * kGraphChunks[0]);
      };
      pdl_ms_[1] = time_graph(true);
      pdl_ms_[0] = time_graph(false);
      pdl_ = pdl_ms_[1] <= pdl_ms_[0];
      invalidate_graphs();
      step_ = s0;
      for (Phase& P : phases_)
        if (!P.fields.empty()) {
          P.tune_pdl = pdl_ ? 1 : 0;
          tune_cache_store(tune_key(P), tune_value(P, P.tune_best_ms));
        }
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  tuning_ = false;
  mspan_ = span0;
  launches_ = l0;
  check(cudaMemcpyAsync(members_d_, members_h_.data(), members_h_.size() * sizeof(MemberK), cudaMemcpyHostToDevice,
                        stream_),
        "member upload");
  zero_dynamic_buffers();
  check(cudaStreamSynchronize(stream_), "autotune");
}

// Cache key of a phase: the GPU (name and multiprocessors), the grid, the batch span, the
// plane mode and a hash of the phase's width-generic update program at the default shape
// (which fixes the structure of the update).  kTuneFormat changes when kernels change in
// a way that makes old timings meaningless.
std::string Solver::tune_key(const Phase& P) {
  constexpr int kTuneFormat = 2;
  int dev = 0;
  check(cudaGetDevice(&dev), "cudaGetDevice");
  cudaDeviceProp pr;
  check(cudaGetDeviceProperties(&pr, dev), "cudaGetDeviceProperties");
  std::string gpu = pr.name;
  for (char& ch : gpu)
    if (ch == ' ' || ch == '\t' || ch == '/') ch = '_';
  LineParams p;
  int nslots = 0;
  bool any_chan = false;
  fill_turn(P, p, nslots, any_chan);
  p.W = 0;
  const int L = turn_len();
  const std::string src = jit_generate_turn(p, L, dim_ == 3 ? 2 : 1, turn_warps_, batch_, turn_split_form(L));
  char h[17];
  std::snprintf(h, sizeof(h), "%016llx", (unsigned long long)fnv1a64(src));
  std::ostringstream os;
  os << "v" << kTuneFormat << "/" << gpu << "/sm" << pr.multiProcessorCount << "/" << sx_ << "x" << sy_ << "x" << sz_
     << "/m" << mspan_ << "/p" << P.id << "/plane" << (plane_ok_ ? 1 : 0) << "/jit" << (use_jit_ ? 1 : 0) << "/" << h;
  return os.str();
}

std::string Solver::tune_value(const Phase& P, double ms) const {
  std::ostringstream os;
  os << "W=" << P.tuned_w << " warps=" << phase_warps(P) << " split=" << (phase_split(P) ? 1 : 0)
     << " plane=" << (plane_ ? 1 : 0) << " plane_c=" << plane_c_ << " ms=" << ms;
  if (P.tune_pdl >= 0) os << " pdl=" << P.tune_pdl;
  return os.str();
}

bool Solver::apply_tune_value(Phase& P, const std::string& v, int wmax_rule) {
  double w = 0, warps = 0, split = -1, pc = 0, pl = 0;
  if (!tune_value_get(v, "W", &w) || !tune_value_get(v, "warps", &warps) || !tune_value_get(v, "split", &split) ||
      !tune_value_get(v, "plane_c", &pc) || !tune_value_get(v, "plane", &pl))
    return false;
  const int L = turn_len();
  const int nl = (dim_ == 3) ? 2 : 1;
  LineParams p;
  int nslots = 0;
  bool any_chan = false;
  fill_turn(P, p, nslots, any_chan);
  const bool sp = use_jit_ && L >= 512 && split > 0.5;
  const int wmax = use_jit_ ? pick_w(L, nl, nslots, 0, sp) : wmax_rule;
  const int wi = (int)w;
  if (wi < 1 || wi > wmax || (wi & (wi - 1)) != 0 || warps < 8 || warps > 64) return false;
  int c = (int)pc;
  if (plane_ok_ && plane_env_ < 0 && !P.products.empty()) {
    if (pl > 0.5 && c > 0) {
      const int g = P.xin[0];
      const int nc = std::min(Lx_, sx_ / (alias_order_[g] + 1) + 1);
      if (plane_pass_shape(Lx_, sy_, nc, nullptr, nullptr, c) != c) return false;
      plane_c_ = c;
    }
    plane_ = pl > 0.5;
  }
  P.tuned_w = wi;
  P.tuned_warps = (int)warps;
  if (L >= 512) P.tuned_split = sp ? 1 : 0;
  double pdl = -1;
  P.tune_pdl = (tune_value_get(v, "pdl", &pdl) && (pdl == 0.0 || pdl == 1.0)) ? (int)pdl : -1;
  if (tune_value_get(v, "ms", &pdl)) P.tune_best_ms = pdl;
  return true;
}

size_t Solver::estimate_bytes(int members) {
  if (members < 1) throw Error(kErrInvalid, "members >= 1");
  if (!prepared_) build_plan();
  const size_t half = (size_t)Lx_ * sy_ * sz_, arr = half * sizeof(float2) * (size_t)members;
  size_t b = 2 * 2048 * sizeof(float2) + npoints() * sizeof(float) + half * sizeof(float2);   // tables, scratch
  for (int f = 0; f < nfields(); ++f) {
    b += 2 * arr;
    if (alias_order_[f] > 1) b += (dim_ == 3 ? 2 : 1) * arr;
  }
  for (const Phase& P : phases_) b += (size_t)P.nchan * arr;   // one buffer per product channel
  if (members > 1 || batch_) b += (size_t)members * (sizeof(MemberK) + 2 * kMemberVals * sizeof(float));
  return b;
}

bool Solver::idle() {
  if (!stream_) return true;
  const cudaError_t e = cudaStreamQuery(stream_);
  if (e == cudaSuccess) return true;
  if (e == cudaErrorNotReady) return false;
  check(e, "cudaStreamQuery");
  return false;
}

std::string Solver::tune_report() const {
  std::ostringstream os;
  os << "{";
  bool first = true;
  for (const Phase& P : phases_) {
    if (P.fields.empty()) continue;
    if (!first) os << ", ";
    first = false;
    os << "\"phase" << P.id << "\": {\"W\": " << P.tuned_w << ", \"warps\": " << phase_warps(P)
       << ", \"split\": " << (phase_split(P) ? 1 : 0) << ", \"plane\": " << (plane_ ? 1 : 0)
       << ", \"plane_c\": " << plane_c_ << ", \"cached\": " << (P.tune_cached ? "true" : "false") << ", \"ms\": {";
    for (size_t i = 0; i < P.tune_ms.size(); ++i)
      os << (i ? ", " : "") << "\"" << P.tune_ms[i].first << "\": " << P.tune_ms[i].second;
    os << "}}";
  }
  // programmatic dependent launch: the choice, and the 16-step graph times when timed here
  os << (first ? "" : ", ") << "\"pdl\": " << (pdl_ ? 1 : 0);
  if (pdl_ms_[0] > 0.0) os << ", \"pdl_ms_per_step\": {\"off\": " << pdl_ms_[0] << ", \"on\": " << pdl_ms_[1] << "}";
  os << "}";
  return os.str();
}

void Solver::invalidate_graphs() {
  for (auto& row : graph_)
    for (cudaGraphExec_t& g : row)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
}

// Records kGraphChunks[c] steps starting at ping-pong parity `parity` into a graph and
// instantiates it.  Nothing runs: the step count, launch count and parities are restored
// afterwards, and run_graph applies the chunk's effect on them when it replays it.
void Solver::capture_graph(int c, int parity) {
  const int n = kGraphChunks[c];
  const long long s0 = step_, l0 = launches_;
  const std::vector<int> par0 = par_;
  std::fill(par_.begin(), par_.end(), parity);
  cudaGraph_t g = nullptr;
  auto restore = [&] {
    step_ = s0;
    launches_ = l0;
    par_ = par0;
  };
  check(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
  try {
    // the launches of step s use step count + s; one counter update ends the graph
    for (int s = 0; s < n; ++s) step_once((uint32_t)s, s == n - 1);
  } catch (...) {
    cudaStreamEndCapture(stream_, &g);
    if (g) cudaGraphDestroy(g);
    restore();
    throw;
  }
  const long long nl = launches_ - l0;
  restore();
  check(cudaStreamEndCapture(stream_, &g), "cudaStreamEndCapture");
  cudaGraphExec_t ex = nullptr;
  const cudaError_t e = cudaGraphInstantiate(&ex, g, 0);
  cudaGraphDestroy(g);
  check(e, "cudaGraphInstantiate");
  // the graph's work is uploaded to the device now, not at its first replay
  check(cudaGraphUpload(ex, stream_), "cudaGraphUpload");
  graph_[c][parity] = ex;
  graph_launches_[c] = nl;
}

void Solver::capture_all_graphs() {
  for (int c = 0; c < 3; ++c)
    for (int parity = 0; parity < 2; ++parity)
      if (!graph_[c][parity]) capture_graph(c, parity);
  check(cudaStreamSynchronize(stream_), "graph upload");
}

// Replays chunk c from the graph for the current ping-pong parity (every field flips
// once per step, so all fields share one parity).
void Solver::run_graph(int c) {
  const int key = par_.empty() ? 0 : par_[0];
  if (!graph_[c][key]) capture_graph(c, key);
  check(cudaGraphLaunch(graph_[c][key], stream_), "cudaGraphLaunch");
  launches_ += graph_launches_[c];
  step_ += kGraphChunks[c];
  if (kGraphChunks[c] & 1)
    for (int& p : par_) p ^= 1;
}

}  // namespace cupssgb
