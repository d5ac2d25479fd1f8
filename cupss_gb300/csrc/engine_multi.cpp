// Fused stepping of several batched solvers on different grids (see engine_multi.h).
#include "engine_multi.h"

#include <algorithm>
#include <cstring>
#include <sstream>

#include "fft.cuh"
#include "jit.h"
#include "launch.h"
#include "tune_cache.h"

namespace cupssgb {

namespace {
constexpr size_t kMaxFusedSmem = 220 * 1024;
}

void MultiStep::check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw Error(kErrCuda, std::string(what) + ": " + cudaGetErrorString(e));
}

std::string MultiStep::unsupported(const std::vector<Solver*>& s, bool need_prepared) {
  if (s.empty() || (int)s.size() > kMaxClasses)
    return "fused stepping takes 1 to " + std::to_string(kMaxClasses) + " grid classes";
  for (Solver* S : s) {
    if (!S->batch_) return "every class must be a batched solver";
    if (S->prepared_) continue;
    if (need_prepared) return "every class must be a prepared batched solver";
    S->build_plan();
  }
  for (size_t c = 0; c < s.size(); ++c) {
    const Solver& S = *s[c];
    if (S.dim_ > 2) return "fused stepping covers 1D and 2D grids";
    if (!S.use_jit_) return "fused stepping needs the generated update programs";
    for (int ph = 0; ph < 2; ++ph) {
      const Solver::Phase& P = S.phases_[ph];
      const Solver::Phase& P0 = s[0]->phases_[ph];
      if (P.fields != P0.fields || P.products != P0.products || P.xin != P0.xin || P.prod_add != P0.prod_add ||
          P.term_slot != P0.term_slot)
        return "the classes differ in system structure";
      if (P.fields.empty() || c == 0) continue;
      LineParams p, p0;
      int nslots = 0;
      bool any_chan = false;
      S.fill_turn(P, p, nslots, any_chan);
      s[0]->fill_turn(P0, p0, nslots, any_chan);
      if (jit_program_text(p, true) != jit_program_text(p0, true)) return "the classes differ in their update programs";
    }
  }
  for (int ph = 0; ph < 2; ++ph) {
    PhaseK K;
    const std::string why = plan_phase(s, ph, K, nullptr);
    if (!why.empty()) return why;
  }
  return std::string();
}

MultiStep::MultiStep(const std::vector<Solver*>& s)
    : s_(s), mt_(new MultiTurnParams), mr_(new MultiRowParams) {
  const std::string why = unsupported(s);
  if (!why.empty()) throw Error(kErrUnsupported, why);
  check(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking), "cudaStreamCreate");
  check(cudaEventCreateWithFlags(&ev_, cudaEventDisableTiming), "cudaEventCreate");
  pdl_ = s_[0]->pdl_;   // class 0's own choice until choose() times both
  class_ev_.resize(s_.size());
  for (cudaEvent_t& e : class_ev_) check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
  build();
}

MultiStep::~MultiStep() {
  if (stream_) cudaStreamSynchronize(stream_);
  for (auto& row : graph_)
    for (cudaGraphExec_t& g : row)
      if (g) cudaGraphExecDestroy(g);
  for (cudaEvent_t e : class_ev_)
    if (e) cudaEventDestroy(e);
  if (ev_) cudaEventDestroy(ev_);
  if (stream_) cudaStreamDestroy(stream_);
}

// The turnaround CTA of a fused launch has one thread count T for every class: class c's
// lines of L_c = sy_c points take M_c threads each in the class's own FFT form (the one
// its solver uses), and its tile is W_c = T / M_c columns (columns past sx_c/2 are idle
// threads: every access of the turnaround is guarded for them).  T is the tile of the
// class with the most points times its line threads, so that class -- which takes most
// of the time -- runs with the tile width and resident-warp target tuned for it.
std::string MultiStep::plan_phase(const std::vector<Solver*>& s, int ph, PhaseK& K, std::string* src) {
  K = PhaseK();
  const Solver::Phase& P0 = s[0]->phases_[ph];
  K.active = !P0.fields.empty();
  if (!K.active) return std::string();
  K.has_row = !P0.products.empty();
  const size_t nc = s.size();
  std::vector<MultiClassSpec> specs(nc);
  std::vector<int> nslots(nc), M(nc);
  size_t dom = 0;
  double most = -1.0;
  for (size_t c = 0; c < nc; ++c) {
    const Solver& S = *s[c];
    const Solver::Phase& P = S.phases_[ph];
    bool any_chan = false;
    S.fill_turn(P, specs[c].turn, nslots[c], any_chan);
    specs[c].L = S.sy_;
    specs[c].split = S.phase_split(P);
    M[c] = line_m_of(S.sy_, specs[c].split);
    if (M[c] < 1) return "no line FFT form for a grid of the ensemble";
    const double pts = (double)S.npoints() * S.mspan_;
    if (pts > most) {
      most = pts;
      dom = c;
    }
  }
  const Solver& D = *s[dom];
  int T = D.phase_turn_w(D.phases_[ph], nslots[dom]) * M[dom];
  for (int m : M) T = std::max(T, m);
  T = std::min(std::max(T, 32), 1024);
  for (size_t c = 0; c < nc; ++c)
    if (T % M[c] != 0) return "a grid of the ensemble does not fit the fused turnaround block";
  K.turn_threads = T;
  const int min_blocks = std::max(1, D.phase_warps(D.phases_[ph]) * 32 / T);
  bool all_one = true;
  int tiles = 0, blocks = 0;
  for (size_t c = 0; c < nc; ++c) {
    const Solver& S = *s[c];
    const Solver::Phase& P = S.phases_[ph];
    MultiClassSpec& sp = specs[c];
    const int W = T / M[c];
    sp.turn.W = W;
    sp.turn_tiles = (S.Lx_ + W - 1) / W;
    const size_t smem = line_pass_smem(S.sy_, 1, W, nslots[c], sp.split);
    if (smem > kMaxFusedSmem) return "fused turnaround shared memory";
    K.turn_w.push_back(W);
    K.turn_tiles.push_back(sp.turn_tiles);
    tiles += sp.turn_tiles;
    K.turn_smem = std::max(K.turn_smem, smem);
    if (K.has_row) {
      XParams x;
      S.row_params(P, x);
      const RowShape r = row_pass_shape(x, S.mspan_);
      if (r.m <= 0 || r.m * r.rw != 128 || r.smem > kMaxFusedSmem)
        return "a grid of the ensemble does not fit the fused row pass block";
      sp.LX = S.Lx_;
      sp.row_one = r.one;
      sp.row_split = r.split;
      sp.row_m = r.m;
      sp.row_blocks = r.blocks;
      all_one = all_one && r.one;
      K.row_blocks.push_back(r.blocks);
      blocks += r.blocks;
      K.row_smem = std::max(K.row_smem, r.smem);
    }
  }
  K.turn_grid = dim3(tiles, 1, 1);
  K.row_grid = dim3(blocks, 1, 1);
  if (src) *src = jit_generate_multi(specs, K.has_row, true, T, min_blocks, all_one ? 3 : 2);
  return std::string();
}

std::string MultiStep::generated_source(const std::vector<Solver*>& s, int ph) {
  if (ph < 0 || ph > 1) throw Error(kErrInvalid, "phase must be 0 or 1");
  const std::string why = unsupported(s, false);
  if (!why.empty()) throw Error(kErrUnsupported, why);
  PhaseK K;
  std::string src;
  plan_phase(s, ph, K, &src);
  return src;
}

void MultiStep::build() {
  epoch_.clear();
  for (Solver* S : s_) epoch_.push_back(S->plan_epoch_);
  for (int ph = 0; ph < 2; ++ph) {
    PhaseK& K = ph_[ph];
    std::string src;
    const std::string why = plan_phase(s_, ph, K, &src);
    if (!why.empty()) throw Error(kErrUnsupported, why);
    if (!K.active) continue;
    src_hash_ = fnv1a64(std::to_string(src_hash_) + src);
    K.turn = jit_kernel(src, "cupssgb_turn_multi");
    if (K.has_row) K.row = jit_kernel(src, "cupssgb_row_multi");
  }
}

void MultiStep::launch_phase(int ph, uint32_t off) {
  PhaseK& K = ph_[ph];
  if (!K.active) return;
  MultiTurnParams& mt = *mt_;
  MultiRowParams& mr = *mr_;
  std::memset(&mt, 0, sizeof(mt));
  std::memset(&mr, 0, sizeof(mr));
  int zmax = 1;
  for (size_t c = 0; c < s_.size(); ++c) {
    Solver& S = *s_[c];
    const Solver::Phase& P = S.phases_[ph];
    int nslots = 0;
    bool any_chan = false;
    S.fill_turn(P, mt.p[c], nslots, any_chan);
    mt.p[c].W = K.turn_w[c];
    mt.p[c].members = S.members_d_;
    mt.p[c].step_off = off;
    mt.p[c].mstride = S.half_;
    mt.p[c].mvals = S.mvals_d_[P.id];
    mt.span[c] = S.mspan_;
    zmax = std::max(zmax, S.mspan_);
    if (K.has_row) {
      S.row_params(P, mr.x[c]);
      mr.span[c] = S.mspan_;
    }
  }
  const bool pdl = pdl_;
  if (K.has_row) {
    void* args[] = {(void*)&mr};
    LaunchCfg lc(dim3(K.row_grid.x, 1, zmax), dim3(128), K.row_smem, stream_, pdl);
    check(cudaLaunchKernelExC(&lc.cfg, (const void*)K.row, args), "fused row pass");
    ++launches_;
  }
  {
    void* args[] = {(void*)&mt};
    LaunchCfg lc(dim3(K.turn_grid.x, 1, zmax), dim3(K.turn_threads), K.turn_smem, stream_, pdl);
    check(cudaLaunchKernelExC(&lc.cfg, (const void*)K.turn, args), "fused turnaround");
    ++launches_;
  }
  for (Solver* S : s_)
    for (int f : S->phases_[ph].fields) S->par_[f] ^= 1;
}

// One step of every class; its noise uses each member's step count + off.
void MultiStep::step_once(uint32_t off, bool tick) {
  launch_phase(0, off);
  launch_phase(1, off);
  if (tick) {
    MultiTickParams tp;
    std::memset(&tp, 0, sizeof(tp));
    tp.nc = (int)s_.size();
    tp.inc = off + 1u;
    for (size_t c = 0; c < s_.size(); ++c) {
      tp.members[c] = s_[c]->members_d_;
      tp.n[c] = s_[c]->nmem_;
    }
    check(launch_tick_multi(tp, stream_, pdl_), "member step counts");
    ++launches_;
  }
}

void MultiStep::capture(int c, int parity) {
  const int n = Solver::kGraphChunks[c];
  const long long l0 = launches_;
  std::vector<std::vector<int>> par0;
  for (Solver* S : s_) {
    par0.push_back(S->par_);
    std::fill(S->par_.begin(), S->par_.end(), parity);
  }
  auto restore = [&] {
    launches_ = l0;
    for (size_t k = 0; k < s_.size(); ++k) s_[k]->par_ = par0[k];
  };
  cudaGraph_t g = nullptr;
  check(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
  try {
    for (int st = 0; st < n; ++st) step_once((uint32_t)st, st == n - 1);
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
  check(cudaGraphUpload(ex, stream_), "cudaGraphUpload");
  graph_[c][parity] = ex;
  graph_launches_[c] = nl;
}

void MultiStep::advance(int nsteps) {
  if (nsteps < 0) throw Error(kErrInvalid, "nsteps < 0");
  if (!fused_) {
    // each class on its own stream, concurrently
    for (Solver* S : s_) S->advance(nsteps);
    return;
  }
  for (size_t c = 0; c < s_.size(); ++c) {
    Solver* S = s_[c];
    if (S->mvals_dirty_) S->upload_member_values();
    S->check_merges();
    if (S->plan_epoch_ != epoch_[c])
      throw Error(kErrState, "a grid class was re-planned (merged product terms now differ): create the fused "
                             "stepper again");
  }
  const int parity = s_[0]->par_.empty() ? 0 : s_[0]->par_[0];
  for (Solver* S : s_)
    for (int p : S->par_)
      if (p != parity) throw Error(kErrState, "the grid classes were stepped apart from the fused stepper");
  // graphs hold the member spans of their capture: recapture after a span changed
  std::vector<int> span;
  for (Solver* S : s_) span.push_back(S->mspan_);
  if (span != graph_span_) {
    invalidate();
    graph_span_ = span;
  }
  // after everything queued on the classes' streams (uploads)
  for (size_t c = 0; c < s_.size(); ++c) {
    check(cudaEventRecord(class_ev_[c], s_[c]->stream_), "cudaEventRecord");
    check(cudaStreamWaitEvent(stream_, class_ev_[c], 0), "cudaStreamWaitEvent");
  }
  for (int c = 0; c < 3; ++c)
    for (; nsteps >= Solver::kGraphChunks[c]; nsteps -= Solver::kGraphChunks[c]) {
      const int key = s_[0]->par_.empty() ? 0 : s_[0]->par_[0];
      if (!graph_[c][key]) capture(c, key);
      check(cudaGraphLaunch(graph_[c][key], stream_), "cudaGraphLaunch");
      launches_ += graph_launches_[c];
      for (Solver* S : s_) {
        S->step_ += Solver::kGraphChunks[c];
        if (Solver::kGraphChunks[c] & 1)
          for (int& p : S->par_) p ^= 1;
      }
    }
  // the classes' later work (readouts) after the steps
  check(cudaEventRecord(ev_, stream_), "cudaEventRecord");
  for (Solver* S : s_) check(cudaStreamWaitEvent(S->stream_, ev_, 0), "cudaStreamWaitEvent");
}

void MultiStep::invalidate() {
  check(cudaStreamSynchronize(stream_), "cudaStreamSynchronize");
  for (auto& row : graph_)
    for (cudaGraphExec_t& g : row)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
}

void MultiStep::restart() {
  for (Solver* S : s_) {
    S->zero_dynamic_buffers();
    for (MemberK& k : S->members_h_) k.step = 0u;
    check(cudaMemcpyAsync(S->members_d_, S->members_h_.data(), S->members_h_.size() * sizeof(MemberK),
                          cudaMemcpyHostToDevice, S->stream_),
          "member upload");
    S->step_ = 0;
    check(cudaStreamSynchronize(S->stream_), "restart");
  }
}

std::string MultiStep::choice_key() const {
  int dev = 0;
  check(cudaGetDevice(&dev), "cudaGetDevice");
  cudaDeviceProp pr;
  check(cudaGetDeviceProperties(&pr, dev), "cudaGetDeviceProperties");
  std::string gpu = pr.name;
  for (char& ch : gpu)
    if (ch == ' ' || ch == '\t' || ch == '/') ch = '_';
  std::ostringstream os;
  os << "multi1/" << gpu << "/sm" << pr.multiProcessorCount << "/";
  for (const Solver* S : s_) os << S->sx_ << "x" << S->sy_ << "x" << S->sz_ << "m" << S->mspan_ << ",";
  char h[17];
  std::snprintf(h, sizeof(h), "%016llx", (unsigned long long)src_hash_);
  os << "/" << h;
  return os.str();
}

void MultiStep::choose() {
  chosen_ = true;
  const std::string key = choice_key();
  std::string cached;
  double f = -1.0, pd = -1.0;
  if (tune_cache_lookup(key, &cached) && tune_value_get(cached, "fused", &f) && (f == 0.0 || f == 1.0) &&
      tune_value_get(cached, "pdl", &pd) && (pd == 0.0 || pd == 1.0) &&
      tune_value_get(cached, "ms_fused", &ms_fused_) && tune_value_get(cached, "ms_grouped", &ms_grouped_)) {
    if (pdl_ != (pd == 1.0)) {
      pdl_ = pd == 1.0;
      invalidate();
    }
    fused_ = f == 1.0;
    choice_cached_ = true;
    return;
  }
  constexpr int kSteps = 16;
  const long long l0 = launches_;
  std::vector<long long> sl0;
  for (Solver* S : s_) sl0.push_back(S->launches_);
  cudaEvent_t a = nullptr, b = nullptr;
  check(cudaEventCreate(&a), "cudaEventCreate");
  check(cudaEventCreate(&b), "cudaEventCreate");
  auto timed = [&](bool fused) {
    fused_ = fused;
    advance(kSteps);   // warm-up: graphs captured
    check(cudaStreamSynchronize(stream_), "choose");
    for (Solver* S : s_) check(cudaStreamSynchronize(S->stream_), "choose");
    check(cudaEventRecord(a, stream_), "cudaEventRecord");
    for (Solver* S : s_) check(cudaStreamWaitEvent(S->stream_, a, 0), "cudaStreamWaitEvent");
    if (fused) {
      advance(kSteps);   // waits on the class streams, which wait on a
    } else {
      advance(kSteps);
      for (size_t c = 0; c < s_.size(); ++c) {
        check(cudaEventRecord(class_ev_[c], s_[c]->stream_), "cudaEventRecord");
        check(cudaStreamWaitEvent(stream_, class_ev_[c], 0), "cudaStreamWaitEvent");
      }
    }
    check(cudaEventRecord(b, stream_), "cudaEventRecord");
    check(cudaEventSynchronize(b), "cudaEventSynchronize");
    float ms = 0.f;
    check(cudaEventElapsedTime(&ms, a, b), "cudaEventElapsedTime");
    return (double)ms / kSteps;
  };
  try {
    // the fused launches without and with programmatic dependent launch (graphs of each)
    for (int on = 0; on < 2; ++on) {
      pdl_ = on == 1;
      invalidate();
      ms_fused_pdl_[on] = timed(true);
    }
    pdl_ = ms_fused_pdl_[1] < ms_fused_pdl_[0];
    invalidate();
    ms_fused_ = ms_fused_pdl_[pdl_ ? 1 : 0];
    ms_grouped_ = timed(false);
  } catch (...) {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    fused_ = true;
    throw;
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  fused_ = ms_fused_ <= ms_grouped_;
  launches_ = l0;
  for (size_t c = 0; c < s_.size(); ++c) s_[c]->launches_ = sl0[c];
  restart();
  std::ostringstream v;
  v << "fused=" << (fused_ ? 1 : 0) << " pdl=" << (pdl_ ? 1 : 0) << " ms_fused=" << ms_fused_
    << " ms_grouped=" << ms_grouped_;
  tune_cache_store(key, v.str());
}

std::string MultiStep::describe() const {
  std::ostringstream os;
  os << "{\"classes\": [";
  for (size_t c = 0; c < s_.size(); ++c) {
    const Solver& S = *s_[c];
    os << (c ? ", " : "") << "{\"grid\": [" << S.sx_ << ", " << S.sy_ << ", " << S.sz_ << "], \"members\": "
       << S.nmem_;
    for (int ph = 0; ph < 2; ++ph) {
      const PhaseK& K = ph_[ph];
      if (!K.active) continue;
      os << ", \"phase" << ph << "\": {\"W\": " << K.turn_w[c] << ", \"turn_threads\": " << K.turn_threads
         << ", \"turn_ctas\": " << K.turn_tiles[c];
      if (K.has_row) os << ", \"row_ctas\": " << K.row_blocks[c];
      os << "}";
    }
    os << "}";
  }
  os << "], \"launches_per_step\": " << ((ph_[0].active ? 1 + ph_[0].has_row : 0) + (ph_[1].active ? 1 + ph_[1].has_row : 0))
     << ", \"form\": \"" << (fused_ ? "fused" : "grouped") << "\"";
  os << ", \"pdl\": " << (pdl_ ? 1 : 0);
  if (chosen_) {
    os << ", \"ms_per_step\": {\"fused\": " << ms_fused_ << ", \"grouped\": " << ms_grouped_;
    if (ms_fused_pdl_[0] > 0.0)
      os << ", \"fused_pdl_off\": " << ms_fused_pdl_[0] << ", \"fused_pdl_on\": " << ms_fused_pdl_[1];
    os << "}, \"cached\": " << (choice_cached_ ? "true" : "false");
  }
  os << "}";
  return os.str();
}

}  // namespace cupssgb
