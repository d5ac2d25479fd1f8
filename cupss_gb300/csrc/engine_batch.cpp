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
#include <cstring>
#include <sstream>

#include "engine.h"
#include "launch.h"

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
    for (float2* b : P.prodbuf) check(cudaMemsetAsync(b, 0, bytes, stream_), "buffer reset");
  std::fill(par_.begin(), par_.end(), 0);
}

// Times each candidate tile width of every phase's turnaround on the solver itself
// (one warm-up and three timed runs of the whole phase) and keeps the fastest.  The
// phases run on the zeroed buffers of a freshly prepared solver; every buffer is
// zeroed again afterwards and no step is counted.  Runs for single systems too: a 2D
// grid has only Lx/W turnaround CTAs, so narrow tiles can win on large 2D grids.
void Solver::autotune() {
  const int L = (dim_ == 3) ? sz_ : sy_;
  const int nl = (dim_ == 3) ? 2 : 1;
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
  for (Phase& P : phases_) {
    P.tune_ms.clear();
    if (P.fields.empty()) continue;
    LineParams p;
    int nslots = 0;
    bool any_chan = false;
    fill_turn(P, p, nslots, any_chan);
    const int wmax = pick_w(L, nl, nslots, 0, turn_split());
    if (turn_w_ > 0) {
      P.tuned_w = std::min(turn_w_, wmax);
      continue;
    }
    std::vector<int> cands;
    for (int w = wmax; w >= 2 && cands.size() < 4; w /= 2) cands.push_back(w);
    if (cands.empty()) cands.push_back(wmax);
    double best = 1e30;
    int best_w = wmax;
    for (int w : cands) {
      P.tuned_w = w;
      run_phase(P);
      check(cudaEventRecord(a, stream_), "cudaEventRecord");
      for (int r = 0; r < 3; ++r) run_phase(P);
      check(cudaEventRecord(b, stream_), "cudaEventRecord");
      check(cudaEventSynchronize(b), "cudaEventSynchronize");
      float ms = 0.f;
      check(cudaEventElapsedTime(&ms, a, b), "cudaEventElapsedTime");
      P.tune_ms.push_back({w, ms / 3.0});
      if (ms < best) {
        best = ms;
        best_w = w;
      }
    }
    P.tuned_w = best_w;
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

size_t Solver::estimate_bytes(int members) {
  if (members < 1) throw Error(kErrInvalid, "members >= 1");
  if (!prepared_) build_plan();
  const size_t half = (size_t)Lx_ * sy_ * sz_, arr = half * sizeof(float2) * (size_t)members;
  size_t b = 2 * 2048 * sizeof(float2) + npoints() * sizeof(float) + half * sizeof(float2);   // tables, scratch
  const bool plane = prepared_ ? plane_ : decide_plane();
  for (int f = 0; f < nfields(); ++f) {
    b += 2 * arr;
    if (alias_order_[f] > 1) b += (dim_ == 3 && !plane ? 2 : 1) * arr;
  }
  for (const Phase& P : phases_) b += P.products.size() * arr;
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
    os << "\"phase" << P.id << "\": {\"W\": " << P.tuned_w << ", \"ms\": {";
    for (size_t i = 0; i < P.tune_ms.size(); ++i)
      os << (i ? ", " : "") << "\"" << P.tune_ms[i].first << "\": " << P.tune_ms[i].second;
    os << "}}";
  }
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
