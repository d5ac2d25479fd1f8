// GB300 pseudospectral engine: plan compilation, device buffers, step driver.
#include "engine.h"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <sstream>

#include "fft.cuh"
#include "jit.h"
#include "launch.h"

namespace cupssgb {

namespace {
constexpr float kPiF = 3.1415926535f;   // the reference's PI (inc/cupss/defines.h:57)

bool pow2(int n) { return n >= 1 && (n & (n - 1)) == 0; }
// 3 * 2^a with a >= 1 (even, so that Nyquist bins and Hermitian line pairs exist)
bool three_pow2(int n) { return n >= 6 && n % 3 == 0 && pow2(n / 3) && n % 2 == 0; }
// supported axis lengths: 2^a up to pow2_max, 3 * 2^a up to odd_max
bool axis_ok(int n, int pow2_max, int odd_max) { return (pow2(n) && n <= pow2_max) || (three_pow2(n) && n <= odd_max); }

std::string cuda_msg(cudaError_t e, const char* what) {
  std::ostringstream os;
  os << what << ": " << cudaGetErrorString(e);
  return os.str();
}
}  // namespace

Solver::Solver(int sx, int sy, int sz, float dx, float dy, float dz, float dt)
    : sx_(sx), sy_(sy), sz_(sz), dx_(dx), dy_(dy), dz_(dz), dt_(dt) {
  const char* jit = std::getenv("CUPSSGB_JIT");
  use_jit_ = !(jit && std::string(jit) == "0");
  // turnaround launch shape: tile width and resident CTAs per SM (tuning knobs)
  if (const char* w = std::getenv("CUPSSGB_TURN_W")) turn_w_ = std::atoi(w);
  if (const char* b = std::getenv("CUPSSGB_TURN_WARPS")) turn_warps_ = std::max(1, std::atoi(b));
  if (const char* d = std::getenv("CUPSSGB_PDL")) {
    pdl_ = std::string(d) != "0";
    pdl_env_ = pdl_ ? 1 : 0;
  }
  if (const char* d = std::getenv("CUPSSGB_PLANE")) plane_env_ = std::string(d) == "0" ? 0 : 1;
  if (sx < 2 || !axis_ok(sx, 2048, 384) || !axis_ok(sy, 1024, 192) || !axis_ok(sz, 1024, 192))
    throw Error(kErrUnsupported,
                "grid sizes must be 2^a or 3*2^a: sx in [2, 2048] (3*2^a up to 384), sy and sz in [1, 1024] "
                "(3*2^a up to 192)");
  // dimension rule of the reference (src/evolver.cpp:22-36)
  dim_ = (sz == 1 && sy == 1) ? 1 : (sz == 1 ? 2 : 3);
  Lx_ = sx / 2;
  // field constructor q-steps (src/field_init.cpp:207-213), float arithmetic
  stepq_[0] = 2.0f * kPiF / (dx * (float)sx);
  stepq_[1] = 2.0f * kPiF / (dy * (float)sy);
  stepq_[2] = 2.0f * kPiF / (dz * (float)sz);
}

Solver::~Solver() {
  for (cudaStream_t st : level_streams_)
    if (st) cudaStreamSynchronize(st);
  if (out_stream_) cudaStreamSynchronize(out_stream_);
  for (cudaEvent_t e : out_ready_)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : out_free_)
    if (e) cudaEventDestroy(e);
  if (out_stream_) cudaStreamDestroy(out_stream_);
  if (up_stream_) cudaStreamSynchronize(up_stream_);
  for (int b = 0; b < 2; ++b) {
    if (up_ready_[b]) cudaEventDestroy(up_ready_[b]);
    if (up_free_[b]) cudaEventDestroy(up_free_[b]);
  }
  if (up_stream_) cudaStreamDestroy(up_stream_);
  for (auto& row : graph_)
    for (cudaGraphExec_t& g : row)
      if (g) cudaGraphExecDestroy(g);
  for (cudaEvent_t e : ev_pool_) cudaEventDestroy(e);
  for (void* p : allocs_) cudaFree(p);
  for (cudaStream_t st : level_streams_)
    if (st) cudaStreamDestroy(st);
  if (level_ev_) cudaEventDestroy(level_ev_);
}

void Solver::check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw Error(kErrCuda, cuda_msg(e, what));
}

// Device allocation owned by the solver, zeroed on the solver's stream unless `zero` is
// false (a buffer that another stream fills completely before anything reads it: a
// zeroing queued on the solver's stream could land after that stream's writes).
void* Solver::dalloc(size_t bytes, bool zero) {
  void* p = nullptr;
  check(cudaMalloc(&p, bytes), "cudaMalloc");
  allocs_.push_back(p);
  dev_bytes_ += bytes;
  if (zero) check(cudaMemsetAsync(p, 0, bytes, stream_), "cudaMemsetAsync");
  return p;
}

int Solver::add_field(bool dynamic) {
  if (prepared_) throw Error(kErrState, "add_field after prepare");
  if (!mfields_.empty()) throw Error(kErrState, "add_field after batch member values were set");
  if ((int)fields_.size() >= kMaxFields) throw Error(kErrLimit, "too many fields");
  HostField f;
  f.dynamic = dynamic;
  fields_.push_back(f);
  return (int)fields_.size() - 1;
}

void Solver::set_implicit(int f, const std::vector<HostPres>& p) {
  if (f < 0 || f >= nfields()) throw Error(kErrInvalid, "bad field index");
  if (prepared_ && p.size() != fields_[f].implicit.size())
    throw Error(kErrState, "the number of implicit prefactors cannot change after prepare");
  fields_[f].implicit = p;
  invalidate_graphs();
}

int Solver::add_term(int f, const std::vector<int>& product, const std::vector<HostPres>& p) {
  if (f < 0 || f >= nfields()) throw Error(kErrInvalid, "bad field index");
  if (prepared_) throw Error(kErrState, "add_term after prepare");
  if (!mfields_.empty()) throw Error(kErrState, "add_term after batch member values were set");
  if (p.empty()) throw Error(kErrInvalid, "term without prefactors");
  for (int g : product)
    if (g < 0 || g >= nfields()) throw Error(kErrInvalid, "bad product field index");
  if ((int)product.size() > kMaxOrder) throw Error(kErrLimit, "product order too large");
  HostTerm t;
  t.product = product;
  t.pres = p;
  fields_[f].terms.push_back(t);
  return (int)fields_[f].terms.size() - 1;
}

void Solver::set_term_pres(int f, int t, const std::vector<HostPres>& p) {
  if (f < 0 || f >= nfields() || t < 0 || t >= (int)fields_[f].terms.size())
    throw Error(kErrInvalid, "bad term index");
  if (p.size() != fields_[f].terms[t].pres.size())
    throw Error(kErrInvalid, "prefactor count of a term cannot change");
  fields_[f].terms[t].pres = p;
  merge_check_ = true;
  invalidate_graphs();
}

void Solver::set_noise(int f, bool on, const HostPres& amp) {
  if (f < 0 || f >= nfields()) throw Error(kErrInvalid, "bad field index");
  if (prepared_ && on != fields_[f].noisy) throw Error(kErrState, "noise cannot be switched after prepare");
  fields_[f].noisy = on;
  fields_[f].noise = amp;
  invalidate_graphs();
}

void Solver::set_seed(uint64_t s) {
  seed_ = s;
  if (batch_) return;   // batch members keep their own seeds
  members_h_.assign(1, MemberK{(uint32_t)(s & 0xffffffffu), (uint32_t)(s >> 32), 0u, 1u});
  if (prepared_) {
    check(cudaMemcpyAsync(members_d_, members_h_.data(), 2 * sizeof(uint32_t), cudaMemcpyHostToDevice, stream_),
          "seed upload");
    check(cudaStreamSynchronize(stream_), "seed upload");
  }
}

void Solver::set_dt(float dt) {
  dt_ = dt;
  invalidate_graphs();
  if (batch_ && prepared_) mvals_dirty_ = true;   // noise bases depend on dt
}

void Solver::build_plan() {
  const int F = nfields();
  alias_order_.assign(F, 1);
  chan_wide_.assign(F, 0);
  // term::prepareDevice (src/term_init.cpp:108-133): fields in products of size >= 2
  // are dealiased for the largest such product.
  for (const HostField& f : fields_)
    for (const HostTerm& t : f.terms)
      if (t.product.size() >= 2)
        for (int g : t.product)
          alias_order_[g] = std::max(alias_order_[g], (int)t.product.size());
  const char* me = std::getenv("CUPSSGB_MERGE");
  if (me && std::string(me) == "0") merge_off_ = true;
  for (int ph = 0; ph < 2; ++ph) {
    Phase& P = phases_[ph];
    P = Phase();
    P.id = ph;
    for (int f = 0; f < F; ++f)
      if ((int)fields_[f].dynamic == ph) P.fields.push_back(f);
    plan_products(P, !merge_off_);
    if ((int)P.fields.size() > kMaxPhaseFields) throw Error(kErrLimit, "too many fields in a phase");
    if ((int)P.products.size() > kMaxProd) throw Error(kErrLimit, "too many distinct products");
    if ((int)P.xin.size() > kMaxXIn) throw Error(kErrLimit, "too many fields in products");
    int nt = 0, np = 0;
    for (int f : P.fields) {
      nt += (int)fields_[f].terms.size();
      np += (int)fields_[f].implicit.size();
      for (const HostTerm& t : fields_[f].terms) np += (int)t.pres.size();
    }
    if (nt > kMaxTerms) throw Error(kErrLimit, "too many terms in a phase");
    if (np > kMaxPres) throw Error(kErrLimit, "too many prefactors in a phase");
  }
}

// Stream priorities of the device: least (the default) down to greatest, numerically;
// level l maps to max(greatest, least - l), its index among the solver's streams to l
// clamped the same way.
static void priority_of(int level, int max_index, int* prio, int* index) {
  int least = 0, greatest = 0;
  if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess)
    throw Error(kErrCuda, "cudaDeviceGetStreamPriorityRange failed");
  *prio = std::max(std::max(greatest, least - max_index), least - level);
  *index = least - *prio;
}

namespace {
bool same_pres(const std::vector<HostPres>& a, const std::vector<HostPres>& b) {
  if (a.size() != b.size()) return false;
  for (size_t j = 0; j < a.size(); ++j)
    if (a[j].pre != b[j].pre || a[j].q2n != b[j].q2n || a[j].iqx != b[j].iqx || a[j].iqy != b[j].iqy ||
        a[j].iqz != b[j].iqz || a[j].invq != b[j].invq)
      return false;
  return true;
}
}  // namespace

void Solver::plan_products(Phase& P, bool merge) {
  P.products.clear();
  P.prod_add.clear();
  P.term_slot.clear();
  P.xin.clear();
  P.chan_buf.clear();
  P.groups.clear();
  P.nchan = 0;
  // the phase's product terms (field, term) and their product keys, in term order
  struct PT {
    int f, t;
    std::vector<int> key;
  };
  std::vector<PT> pts;
  for (int f : P.fields)
    for (size_t t = 0; t < fields_[f].terms.size(); ++t) {
      const HostTerm& ht = fields_[f].terms[t];
      if (ht.product.size() < 2) continue;
      std::vector<int> key = ht.product;
      std::sort(key.begin(), key.end());
      pts.push_back({f, (int)t, key});
      for (int g : key)
        if (std::find(P.xin.begin(), P.xin.end(), g) == P.xin.end()) P.xin.push_back(g);
    }
  auto uses = [&](const std::vector<int>& key) {
    int n = 0;
    for (const PT& q : pts) n += q.key == key;
    return n;
  };
  auto pres_of = [&](int f, int t, int m) -> const std::vector<HostPres>& {
    return (m < 0 ? fields_ : mfields_[m])[f].terms[t].pres;
  };
  // group: index into pts -> group id (-1: alone)
  std::vector<int> gid(pts.size(), -1);
  std::vector<std::vector<int>> groups;
  if (merge) {
    for (size_t i = 0; i < pts.size(); ++i) {
      if (gid[i] >= 0 || uses(pts[i].key) != 1) continue;
      std::vector<int> g{(int)i};
      for (size_t j = i + 1; j < pts.size(); ++j) {
        if (gid[j] >= 0 || pts[j].f != pts[i].f || uses(pts[j].key) != 1) continue;
        bool same = same_pres(pres_of(pts[i].f, pts[i].t, -1), pres_of(pts[j].f, pts[j].t, -1));
        for (int m = 0; same && m < (int)mfields_.size(); ++m)
          same = same_pres(pres_of(pts[i].f, pts[i].t, m), pres_of(pts[j].f, pts[j].t, m));
        if (same) g.push_back((int)j);
      }
      if (g.size() < 2) continue;
      for (int k : g) gid[k] = (int)groups.size();
      groups.push_back(g);
    }
  }
  // channels in term order: a group's products one after the other, then its own
  // buffer; a product that is not merged gets one channel however many terms use it
  std::vector<int> chan_of_term(pts.size(), -1);
  for (size_t i = 0; i < pts.size(); ++i) {
    if (chan_of_term[i] != -1) continue;
    if (gid[i] >= 0) {
      const std::vector<int>& g = groups[gid[i]];
      std::vector<std::pair<int, int>> members;
      for (size_t k = 0; k < g.size(); ++k) {
        P.products.push_back(pts[g[k]].key);
        P.prod_add.push_back(k > 0 ? 1 : 0);
        chan_of_term[g[k]] = k == 0 ? P.nchan : -2;
        members.push_back({pts[g[k]].f, pts[g[k]].t});
      }
      P.groups.push_back(members);
    } else {
      auto it = std::find(P.products.begin(), P.products.end(), pts[i].key);
      if (it != P.products.end()) {
        // used by an earlier term: that term's channel (a product used twice is never merged)
        for (size_t j = 0; j < i; ++j)
          if (pts[j].key == pts[i].key) {
            chan_of_term[i] = chan_of_term[j];
            break;
          }
        continue;
      }
      P.products.push_back(pts[i].key);
      P.prod_add.push_back(0);
      chan_of_term[i] = P.nchan;
      P.groups.push_back({});
    }
    P.chan_buf.push_back((int)P.products.size() - 1);
    ++P.nchan;
  }
  // slots of every term of the phase, in the order fill_turn walks them
  size_t k = 0;
  for (int f : P.fields)
    for (const HostTerm& ht : fields_[f].terms) {
      if (ht.product.size() < 2) {
        P.term_slot.push_back(-1);
        continue;
      }
      P.term_slot.push_back(chan_of_term[k++]);
    }
}

bool Solver::merges_hold() const {
  for (const Phase& P : phases_)
    for (const auto& g : P.groups)
      for (size_t k = 1; k < g.size(); ++k) {
        if (!same_pres(fields_[g[0].first].terms[g[0].second].pres, fields_[g[k].first].terms[g[k].second].pres))
          return false;
        for (const auto& mf : mfields_)
          if (!same_pres(mf[g[0].first].terms[g[0].second].pres, mf[g[k].first].terms[g[k].second].pres))
            return false;
      }
  return true;
}

void Solver::check_merges() {
  if (!merge_check_) return;
  merge_check_ = false;
  if (merge_off_ || merges_hold()) return;
  // re-plan without merging: a product keeps the buffer it has (a merged channel's is its
  // last product's); the others get one now
  merge_off_ = true;
  const size_t hall = half_ * (size_t)nmem_;
  for (Phase& P : phases_) {
    std::vector<std::pair<std::vector<int>, float2*>> bufs;
    for (size_t q = 0; q < P.products.size() && q < P.prodbuf.size(); ++q)
      if (P.prodbuf[q]) bufs.push_back({P.products[q], P.prodbuf[q]});
    plan_products(P, false);
    P.prodbuf.assign(P.products.size(), nullptr);
    for (size_t q = 0; q < P.products.size(); ++q) {
      for (const auto& b : bufs)
        if (b.first == P.products[q]) P.prodbuf[q] = b.second;
      if (!P.prodbuf[q]) P.prodbuf[q] = (float2*)dalloc(hall * sizeof(float2));
    }
    P.jit_sig.clear();
  }
  ++plan_epoch_;
  invalidate_graphs();
}

void Solver::set_stream_priority(int level) {
  if (level < 0) throw Error(kErrInvalid, "priority level < 0");
  if (!prepared_) {
    stream_level_ = level;
    return;
  }
  int prio = 0, idx = 0;
  priority_of(level, kMaxLevels - 1, &prio, &idx);
  if (idx == level_index_) return;
  if (!level_streams_[idx])
    check(cudaStreamCreateWithPriority(&level_streams_[idx], cudaStreamNonBlocking, prio), "cudaStreamCreate");
  if (!level_ev_) check(cudaEventCreateWithFlags(&level_ev_, cudaEventDisableTiming), "cudaEventCreate");
  // everything queued so far comes first
  check(cudaEventRecord(level_ev_, stream_), "cudaEventRecord");
  check(cudaStreamWaitEvent(level_streams_[idx], level_ev_, 0), "cudaStreamWaitEvent");
  stream_ = level_streams_[idx];
  level_index_ = idx;
}

void Solver::prepare() {
  if (prepared_) throw Error(kErrState, "prepare called twice");
  int dev = 0;
  check(cudaGetDevice(&dev), "cudaGetDevice");
  int prio = 0;
  priority_of(stream_level_, kMaxLevels - 1, &prio, &level_index_);
  check(cudaStreamCreateWithPriority(&stream_, cudaStreamNonBlocking, prio), "cudaStreamCreate");
  level_streams_[level_index_] = stream_;
  build_plan();
  half_ = (size_t)Lx_ * sy_ * sz_;
  const size_t half = half_;
  const size_t hall = half_ * (size_t)nmem_;   // all members
  const int F = nfields();
  // twiddle super-table (fft.cuh: tw_base): lengths 2^a up to 2048 and 3 * 2^a up to 1536
  {
    std::vector<float2> h(kTwLen);
    fill_twiddle_table(h.data());
    tw_ = (float2*)dalloc(h.size() * sizeof(float2));
    check(cudaMemcpyAsync(tw_, h.data(), h.size() * sizeof(float2), cudaMemcpyHostToDevice, stream_),
          "twiddle upload");
  }
  state_[0].assign(F, nullptr);
  state_[1].assign(F, nullptr);
  chan_.assign(F, nullptr);
  chanz_.assign(F, nullptr);
  par_.assign(F, 0);
  // the plane pass is a candidate of the tuner; both forms keep their channel buffers
  plane_ok_ = decide_plane();
  plane_ = plane_ok_;
  for (int f = 0; f < F; ++f) {
    state_[0][f] = (float2*)dalloc(hall * sizeof(float2));
    state_[1][f] = (float2*)dalloc(hall * sizeof(float2));
    if (alias_order_[f] > 1) {
      chan_[f] = (float2*)dalloc(hall * sizeof(float2));
      if (dim_ == 3) chanz_[f] = (float2*)dalloc(hall * sizeof(float2));
    }
  }
  // one buffer per product channel (a merged channel's sits at its last product)
  for (Phase& P : phases_) {
    P.prodbuf.assign(P.products.size(), nullptr);
    for (int c = 0; c < P.nchan; ++c) P.prodbuf[P.chan_buf[c]] = (float2*)dalloc(hall * sizeof(float2));
  }
  scratch_real_ = (float*)dalloc(npoints() * sizeof(float));
  scratch_spec_ = (float2*)dalloc(half * sizeof(float2));
  // key, step count and active flag of each member (one for a single system)
  if (!batch_)
    members_h_.assign(1, MemberK{(uint32_t)(seed_ & 0xffffffffu), (uint32_t)(seed_ >> 32), 0u, 1u});
  members_d_ = (MemberK*)dalloc((size_t)nmem_ * sizeof(MemberK));
  check(cudaMemcpyAsync(members_d_, members_h_.data(), (size_t)nmem_ * sizeof(MemberK), cudaMemcpyHostToDevice,
                        stream_),
        "member upload");
  if (batch_)
    for (int ph = 0; ph < 2; ++ph) mvals_d_[ph] = (float*)dalloc((size_t)nmem_ * kMemberVals * sizeof(float));
  check(cudaStreamSynchronize(stream_), "prepare sync");
  prepared_ = true;
  if (batch_) upload_member_values();
  if (use_jit_) {
    // compile the specialised update programs now, not inside the first step
    const int L = (dim_ == 3) ? sz_ : sy_;
    const int nl = (dim_ == 3) ? 2 : 1;
    for (Phase& P : phases_) {
      if (P.fields.empty()) continue;
      LineParams p;
      int nslots = 0;
      bool any_chan = false;
      fill_turn(P, p, nslots, any_chan);
      jit_kernel(turn_source(P, p, L, nl), "cupssgb_turn");
    }
  }
  autotune();
  if (use_jit_) {
    // the kernels of the tuned tile widths, compiled now rather than inside the first step
    const int L = (dim_ == 3) ? sz_ : sy_;
    const int nl = (dim_ == 3) ? 2 : 1;
    for (Phase& P : phases_) {
      if (P.fields.empty()) continue;
      LineParams p;
      int nslots = 0;
      bool any_chan = false;
      fill_turn(P, p, nslots, any_chan);
      p.W = P.tuned_w > 0 ? P.tuned_w : pick_w(L, nl, nslots, turn_rows(), phase_split(P));
      if (turn_w_ > 0 && turn_w_ < p.W && P.tuned_w <= 0) p.W = turn_w_;
      jit_kernel(turn_source(P, p, L, nl), "cupssgb_turn");
    }
  }
  // A batch's launches follow its active span, which changes as members come and go, so
  // its graphs are captured on first use; a single system's are final here.
  if (!batch_) capture_all_graphs();
}

// Multiprocessors of the current device (152 on a GB300; also the answer without a GPU).
static int sm_count() {
  int dev = 0, v = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) !=
                                                cudaSuccess || v <= 0) {
    cudaGetLastError();
    return 152;
  }
  return v;
}

int Solver::phase_turn_w(const Phase& P, int nslots) const {
  if (P.tuned_w > 0) return P.tuned_w;
  const int W = pick_w(turn_len(), dim_ == 3 ? 2 : 1, nslots, turn_rows(), phase_split(P));
  return (turn_w_ > 0 && turn_w_ < W) ? turn_w_ : W;
}

bool Solver::phase_split(const Phase& P) const {
  if (!use_jit_ || turn_len() < 512) return false;
  if (P.tuned_split >= 0 && split_override() < 0) return P.tuned_split == 1;
  return turn_split_form(turn_len());
}

int Solver::pick_w(int L, int nl, int nslots, int other, bool split) const {
  int W = 16;
  while (W > Lx_) W /= 2;
  if (W < 1) W = 1;
  while (W > 1 && (line_threads(L, nl, W, split) > 256 ||
                   line_pass_smem(L, nl, W, std::max(nslots, 1), split) > 200 * 1024))
    W /= 2;
  if (line_pass_smem(L, nl, W, std::max(nslots, 1), split) > 220 * 1024)
    throw Error(kErrLimit, "phase needs more shared memory than one CTA has");
  // a single system whose grid has fewer tiles than the GPU has SMs (2D grids with long
  // lines): narrower tiles put every SM to work.  Batches multiply the tiles by their
  // members and tune the width by measurement instead.
  if (!batch_ && other > 0) {
    const int sms = sm_count();
    while (W > 2 && (long long)((Lx_ + W - 1) / W) * other < sms) W /= 2;
  }
  return W;
}

void Solver::fill_line_common(LineParams& p, int L, int geo, int mode) const {
  std::memset(&p, 0, sizeof(p));
  p.sx = sx_;
  p.sy = sy_;
  p.sz = sz_;
  p.Lx = Lx_;
  p.L = L;
  p.geo = geo;
  p.mode = mode;
  p.stepqx = stepq_[0];
  p.stepqy = stepq_[1];
  p.stepqz = stepq_[2];
  p.dt = dt_;
  const double N = (double)npoints();
  p.invN = 1.0f / (float)N;   // normalize_k (src/field_kernels.cu:124)
  p.sqrtN = (float)std::sqrt(N);
  p.sqrtHalfN = (float)std::sqrt(N / 2.0);
  p.tw = tw_;
}

void Solver::line_fwd_inv(int geo, int mode, const float2* in, float2* out, int xlimit, bool batch, int lkeep,
                          bool pdl) {
  LineParams p;
  const int L = (geo == kGeoY3 || geo == kGeoCol) ? sy_ : sz_;
  fill_line_common(p, L, geo, mode);
  p.W = pick_w(L, 1, 1, geo == kGeoY3 ? sz_ : (geo == kGeoZ3 ? sy_ : 1));
  p.n_prod = 1;
  p.prod_in[0] = in;
  p.prod_out[0] = out;
  p.inv_xlimit[0] = xlimit;
  p.inv_lkeep[0] = lkeep;
  if (batch) {
    p.mstride = half_;
    p.members = members_d_;
  }
  // masked inverse (dealiased channel): narrower tiles waste fewer masked columns and
  // give more CTAs to a pass that touches only part of the grid
  if (mode == kModeInv && xlimit < Lx_ - 1) p.W = std::min(p.W, 8);
  int tiles = (Lx_ + p.W - 1) / p.W;
  if (mode == kModeInv) tiles = std::min(tiles, xlimit / p.W + 1);   // tiles past the limit stay zero
  dim3 grid(tiles, geo == kGeoY3 ? sz_ : (geo == kGeoZ3 ? sy_ : 1), batch ? mspan_ : 1);
  check(launch_line_pass(p, 1, 1, grid, stream_, pdl), "line pass");
  ++launches_;
}

// Page-locked host memory (cudaMallocHost / cudaHostAlloc / cudaHostRegister) is mapped
// into the device's address space: get_real's row pass writes the field to it directly
// over the host link (about 10% faster than a copy out of device memory for a 64 MiB field
// on a GB300), and set_real copies from it asynchronously on an input stream.  nullptr for
// pageable memory, an address not 16-byte aligned, or CUPSSGB_HOST_DIRECT=0.
static void* host_direct(const void* p) {
  const char* e = std::getenv("CUPSSGB_HOST_DIRECT");
  if ((e && std::string(e) == "0") || !p || (reinterpret_cast<uintptr_t>(p) & 15u) != 0) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || !a.devicePointer) return nullptr;
  return (reinterpret_cast<uintptr_t>(a.devicePointer) & 15u) == 0 ? a.devicePointer : nullptr;
}

bool Solver::set_real(int f, const float* src, bool on_device, int m) {
  if (!prepared_) throw Error(kErrState, "set_real before prepare");
  if (f < 0 || f >= nfields()) throw Error(kErrInvalid, "bad field index");
  check_member(m);
  const size_t n = npoints();
  const float* in = scratch_real_;
  int b = -1;
  if (!on_device && host_direct(src)) {
    // page-locked source: copied on the input stream into a staging buffer, so that the
    // copy overlaps what the solver stream still runs (the previous step, its output)
    if (!up_stream_) check(cudaStreamCreateWithFlags(&up_stream_, cudaStreamNonBlocking), "input stream");
    b = up_next_;
    up_next_ ^= 1;
    if (!up_stage_[b]) {
      up_stage_[b] = (float*)dalloc(n * sizeof(float), false);   // the copy below fills it
      check(cudaEventCreateWithFlags(&up_ready_[b], cudaEventDisableTiming), "cudaEventCreate");
      check(cudaEventCreateWithFlags(&up_free_[b], cudaEventDisableTiming), "cudaEventCreate");
    } else {
      check(cudaStreamWaitEvent(up_stream_, up_free_[b], 0), "cudaStreamWaitEvent");
    }
    check(cudaMemcpyAsync(up_stage_[b], src, n * sizeof(float), cudaMemcpyHostToDevice, up_stream_), "set_real copy");
    check(cudaEventRecord(up_ready_[b], up_stream_), "cudaEventRecord");
    check(cudaStreamWaitEvent(stream_, up_ready_[b], 0), "cudaStreamWaitEvent");
    in = up_stage_[b];
  } else {
    check(cudaMemcpyAsync(scratch_real_, src, n * sizeof(float),
                          on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, stream_),
          "set_real copy");
  }
  float2* st = state_[par_[f]][f] + (size_t)m * half_;
  XParams x;
  std::memset(&x, 0, sizeof(x));
  x.Lx = Lx_;
  x.rows = sy_ * sz_;
  x.in_mode = kXInReal;
  x.out_mode = kXOutSpectral;
  x.out_scale = 1.f;
  x.n_in = 1;
  x.in[0] = reinterpret_cast<const float2*>(in);
  x.n_prod = 1;
  x.out[0] = st;
  x.prod_n[0] = 1;
  x.prod_f[0][0] = 0;
  x.tw = tw_;
  check(launch_row_pass(x, stream_), "row pass (upload)");
  ++launches_;
  if (b >= 0) check(cudaEventRecord(up_free_[b], stream_), "cudaEventRecord");
  if (dim_ == 3) {
    line_fwd_inv(kGeoY3, kModeFwd, st, st, Lx_);
    line_fwd_inv(kGeoZ3, kModeFwd, st, st, Lx_);
  } else if (sy_ > 1) {
    line_fwd_inv(kGeoCol, kModeFwd, st, st, Lx_);
  }
  return b >= 0;
}

void Solver::to_real_scratch(int f, int m, float* dst) {
  const float2* st = state_[par_[f]][f] + (size_t)m * half_;
  const float2* spec = st;
  if (dim_ == 3) {
    line_fwd_inv(kGeoZ3, kModeInv, st, scratch_spec_, Lx_);
    line_fwd_inv(kGeoY3, kModeInv, scratch_spec_, scratch_spec_, Lx_);
    spec = scratch_spec_;
  } else if (sy_ > 1) {
    line_fwd_inv(kGeoCol, kModeInv, st, scratch_spec_, Lx_);
    spec = scratch_spec_;
  }
  XParams x;
  std::memset(&x, 0, sizeof(x));
  x.Lx = Lx_;
  x.rows = sy_ * sz_;
  x.in_mode = kXInSpectral;
  x.out_mode = kXOutReal;
  x.out_scale = 1.0f / (float)npoints();
  x.n_in = 1;
  x.in[0] = spec;
  x.n_prod = 1;
  x.out[0] = dst ? dst : scratch_real_;
  x.prod_n[0] = 1;
  x.prod_f[0][0] = 0;
  x.tw = tw_;
  check(launch_row_pass(x, stream_), "row pass (materialise)");
  ++launches_;
}

void Solver::snapshot_real(int f, float* host_dst, cudaEvent_t done) {
  if (!prepared_) throw Error(kErrState, "snapshot before prepare");
  if (f < 0 || f >= nfields()) throw Error(kErrInvalid, "bad field index");
  if (!host_dst) throw Error(kErrInvalid, "null host buffer");
  if (!out_stream_) {
    check(cudaStreamCreateWithFlags(&out_stream_, cudaStreamNonBlocking), "output stream");
    out_stage_.assign(2 * nfields(), nullptr);
    out_ready_.assign(2 * nfields(), nullptr);
    out_free_.assign(2 * nfields(), nullptr);
    out_next_.assign(nfields(), 0);
  }
  // two staging buffers per field, used in turn: the field of one snapshot is written
  // while the copy of the previous one still runs
  const int k = 2 * f + out_next_[f];
  out_next_[f] ^= 1;
  if (!out_stage_[k]) {
    out_stage_[k] = (float*)dalloc(npoints() * sizeof(float));
    check(cudaEventCreateWithFlags(&out_ready_[k], cudaEventDisableTiming), "cudaEventCreate");
    check(cudaEventCreateWithFlags(&out_free_[k], cudaEventDisableTiming), "cudaEventCreate");
  } else {
    // the copy of this buffer's previous snapshot must have left it
    check(cudaStreamWaitEvent(stream_, out_free_[k], 0), "cudaStreamWaitEvent");
  }
  to_real_scratch(f, 0, out_stage_[k]);
  check(cudaEventRecord(out_ready_[k], stream_), "cudaEventRecord");
  check(cudaStreamWaitEvent(out_stream_, out_ready_[k], 0), "cudaStreamWaitEvent");
  check(cudaMemcpyAsync(host_dst, out_stage_[k], npoints() * sizeof(float), cudaMemcpyDeviceToHost, out_stream_),
        "snapshot copy");
  check(cudaEventRecord(out_free_[k], out_stream_), "cudaEventRecord");
  if (done) check(cudaEventRecord(done, out_stream_), "cudaEventRecord");
}

void Solver::get_real(int f, float* dst, bool on_device, int m) {
  if (!prepared_) throw Error(kErrState, "get_real before prepare");
  if (f < 0 || f >= nfields()) throw Error(kErrInvalid, "bad field index");
  check_member(m);
  if (float* d = on_device ? nullptr : static_cast<float*>(host_direct(dst))) {
    to_real_scratch(f, m, d);   // the row pass stores the field in host memory
    check(cudaStreamSynchronize(stream_), "get_real sync");
    return;
  }
  to_real_scratch(f, m);
  check(cudaMemcpyAsync(dst, scratch_real_, npoints() * sizeof(float),
                        on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, stream_),
        "get_real copy");
  if (!on_device) check(cudaStreamSynchronize(stream_), "get_real sync");
}

void Solver::row_pass_simple(int in_mode, const void* in, int out_mode, void* out, float scale) {
  XParams x;
  std::memset(&x, 0, sizeof(x));
  x.Lx = Lx_;
  x.rows = sy_ * sz_;
  x.in_mode = in_mode;
  x.out_mode = out_mode;
  x.out_scale = scale;
  x.n_in = 1;
  x.in[0] = reinterpret_cast<const float2*>(in);
  x.n_prod = 1;
  x.out[0] = out;
  x.prod_n[0] = 1;
  x.prod_f[0][0] = 0;
  x.tw = tw_;
  check(launch_row_pass(x, stream_), "row pass");
  ++launches_;
}

void Solver::forward_lines(float2* st) {
  if (dim_ == 3) {
    line_fwd_inv(kGeoY3, kModeFwd, st, st, Lx_);
    line_fwd_inv(kGeoZ3, kModeFwd, st, st, Lx_);
  } else if (sy_ > 1) {
    line_fwd_inv(kGeoCol, kModeFwd, st, st, Lx_);
  }
}

void Solver::get_real_pairs_device(int f, float2* dst) {
  if (!prepared_) throw Error(kErrState, "get_real before prepare");
  if (f < 0 || f >= nfields()) throw Error(kErrInvalid, "bad field index");
  const float2* st = state_[par_[f]][f];
  const float2* spec = st;
  if (dim_ == 3) {
    line_fwd_inv(kGeoZ3, kModeInv, st, scratch_spec_, Lx_);
    line_fwd_inv(kGeoY3, kModeInv, scratch_spec_, scratch_spec_, Lx_);
    spec = scratch_spec_;
  } else if (sy_ > 1) {
    line_fwd_inv(kGeoCol, kModeInv, st, scratch_spec_, Lx_);
    spec = scratch_spec_;
  }
  row_pass_simple(kXInSpectral, spec, kXOutRealPair, dst, 1.0f / (float)npoints());
}

void Solver::get_dealiased_pairs_device(int f, float2* dst) {
  if (!prepared_) throw Error(kErrState, "get_dealiased before prepare");
  if (f < 0 || f >= nfields() || alias_order_[f] <= 1) throw Error(kErrInvalid, "field has no dealiased copy");
  // Rebuilt from the state rather than read from the channel: after a real-space
  // callback the channel holds the callback's full x spectrum, and the turnaround
  // rewrites only the columns below the dealias limit.
  channel_from_state(f, scratch_spec_);
  row_pass_simple(kXInSpectral, scratch_spec_, kXOutRealPair, dst, 1.0f);
}

void Solver::channel_from_state(int f, float2* dst) {
  // dst <- inverse y/z lines of (masked state / N): the channel layout (x spectrum,
  // y and z positional) that the row pass turns into the dealiased real field.
  MaskParams mp;
  mp.sx = sx_;
  mp.sy = sy_;
  mp.sz = sz_;
  mp.Lx = Lx_;
  mp.xlim = sx_ / (alias_order_[f] + 1);
  mp.ylim = sy_ / (alias_order_[f] + 1);
  mp.zlim = sz_ / (alias_order_[f] + 1);
  mp.scale = 1.0f / (float)npoints();
  mp.spec = state_[par_[f]][f];
  mp.out = scratch_spec_;
  check(launch_mask(mp, stream_), "mask spectrum");
  ++launches_;
  if (dim_ == 3) {
    line_fwd_inv(kGeoZ3, kModeInv, scratch_spec_, scratch_spec_, Lx_);
    line_fwd_inv(kGeoY3, kModeInv, scratch_spec_, dst, Lx_);
  } else if (sy_ > 1) {
    line_fwd_inv(kGeoCol, kModeInv, scratch_spec_, dst, Lx_);
  } else if (dst != scratch_spec_) {
    check(cudaMemcpyAsync(dst, scratch_spec_, (size_t)Lx_ * sizeof(float2), cudaMemcpyDeviceToDevice, stream_),
          "channel copy");
  }
}

// Masked, 1/N-scaled state, z-inverted: the layout the turnaround leaves for the plane
// pass (x and y spectral, z positional).
void Solver::channelz_from_state(int f, float2* dst) {
  MaskParams mp;
  mp.sx = sx_;
  mp.sy = sy_;
  mp.sz = sz_;
  mp.Lx = Lx_;
  mp.xlim = sx_ / (alias_order_[f] + 1);
  mp.ylim = sy_ / (alias_order_[f] + 1);
  mp.zlim = sz_ / (alias_order_[f] + 1);
  mp.scale = 1.0f / (float)npoints();
  mp.spec = state_[par_[f]][f];
  mp.out = dst;
  check(launch_mask(mp, stream_), "mask spectrum");
  ++launches_;
  line_fwd_inv(kGeoZ3, kModeInv, dst, dst, Lx_);
}

bool Solver::plane_phase(const Phase& P) const {
  if (dim_ != 3 || P.xin.size() != 1 || P.products.size() != 1) return false;
  const int g = P.xin[0];
  const int nc = std::min(Lx_, sx_ / (alias_order_[g] + 1) + 1);
  return plane_pass_shape(Lx_, sy_, nc, nullptr, nullptr) > 0;
}

bool Solver::decide_plane() const {
  if (dim_ != 3 || plane_env_ == 0) return false;
  bool any = false;
  for (const Phase& P : phases_) {
    if (P.products.empty()) continue;
    if (!plane_phase(P)) return false;
    any = true;
  }
  return any;
}

// The row-pass channels are the y-inverses of the plane-pass channels.
void Solver::sync_row_channels() {
  for (int f = 0; f < nfields(); ++f)
    if (alias_order_[f] > 1)
      line_fwd_inv(kGeoY3, kModeInv, chanz_[f], chan_[f], sx_ / (alias_order_[f] + 1), batch_,
                   sy_ / (alias_order_[f] + 1) + 1);
}

// A real-space callback can give a dealiased field content at every wavenumber, which
// the plane store is not sized for: the solver goes back to the row-pass form.
void Solver::leave_plane_mode() {
  if (!plane_) return;
  sync_row_channels();
  plane_ = false;
  plane_ok_ = false;
  invalidate_graphs();
}

void Solver::set_fourier_device(int f, const float2* full) {
  if (!prepared_) throw Error(kErrState, "set_fourier before prepare");
  if (f < 0 || f >= nfields()) throw Error(kErrInvalid, "bad field index");
  CompressParams cp;
  cp.sx = sx_;
  cp.sy = sy_;
  cp.sz = sz_;
  cp.Lx = Lx_;
  cp.full = full;
  cp.spec = state_[par_[f]][f];
  check(launch_compress(cp, stream_), "compress spectrum");
  ++launches_;
  if (alias_order_[f] > 1) {
    if (plane_) channelz_from_state(f, chanz_[f]);
    else channel_from_state(f, chan_[f]);
  }
}

void Solver::set_real_pairs_device(int f, const float2* real, const float2* dealiased) {
  if (!prepared_) throw Error(kErrState, "set_real before prepare");
  if (f < 0 || f >= nfields()) throw Error(kErrInvalid, "bad field index");
  float2* st = state_[par_[f]][f];
  row_pass_simple(kXInRealPair, real, kXOutSpectral, st, 1.0f);
  forward_lines(st);
  if (alias_order_[f] > 1) {
    // the channel is the x spectrum scaled by 1/sx (see channel_from_state)
    if (dealiased) {
      leave_plane_mode();
      row_pass_simple(kXInRealPair, dealiased, kXOutSpectral, chan_[f], 1.0f / (float)sx_);
      chan_wide_[f] = 1;
    } else if (plane_) {
      channelz_from_state(f, chanz_[f]);
    } else {
      channel_from_state(f, chan_[f]);
    }
  }
}

void Solver::advance_phase(int phase) {
  if (!prepared_) throw Error(kErrState, "advance before prepare");
  if (phase < 0 || phase > 1) throw Error(kErrInvalid, "phase is 0 (non-dynamic) or 1 (dynamic)");
  if (batch_) throw Error(kErrUnsupported, "phase-wise stepping (callbacks) is for single systems");
  check_merges();
  run_phase(phases_[phase]);
  if (phase == 1) {
    check(launch_tick(members_d_, nmem_, 1u, stream_), "member step count");
    ++launches_;
    ++step_;
  }
}

void Solver::get_fourier(int f, float2* dst, bool on_device, int m) {
  if (!prepared_) throw Error(kErrState, "get_fourier before prepare");
  if (f < 0 || f >= nfields()) throw Error(kErrInvalid, "bad field index");
  check_member(m);
  float2* out = dst;
  if (!on_device) {
    if (!scratch_full_) scratch_full_ = (float2*)dalloc(npoints() * sizeof(float2));
    out = scratch_full_;
  }
  ExpandParams e;
  e.sx = sx_;
  e.sy = sy_;
  e.sz = sz_;
  e.Lx = Lx_;
  e.spec = state_[par_[f]][f] + (size_t)m * half_;
  e.full = out;
  check(launch_expand(e, stream_), "expand spectrum");
  ++launches_;
  if (!on_device) {
    check(cudaMemcpyAsync(dst, scratch_full_, npoints() * sizeof(float2), cudaMemcpyDeviceToHost,
                          stream_),
          "get_fourier copy");
    check(cudaStreamSynchronize(stream_), "get_fourier sync");
  }
}

void Solver::synchronize() {
  if (up_stream_) check(cudaStreamSynchronize(up_stream_), "synchronize");
  if (stream_) check(cudaStreamSynchronize(stream_), "synchronize");
  if (out_stream_) check(cudaStreamSynchronize(out_stream_), "synchronize");
}

void Solver::fill_turn(const Phase& P, LineParams& p, int& nslots, bool& any_chan,
                       const std::vector<HostField>* fields) const {
  const std::vector<HostField>& FS = fields ? *fields : fields_;
  const int geo = (dim_ == 3) ? kGeoZ3 : kGeoCol;
  const int L = (dim_ == 3) ? sz_ : sy_;
  const bool have_dev = prepared_;
  any_chan = false;
  fill_line_common(p, L, geo, kModeTurn);
  p.n_prod = P.nchan;
  for (int q = 0; q < p.n_prod; ++q) p.prod_in[q] = have_dev ? P.prodbuf[P.chan_buf[q]] : nullptr;
  for (int g = 0; g < nfields(); ++g) p.state[g] = (have_dev ? state_[par_[g]][g] : nullptr);
  p.key0 = (uint32_t)(seed_ & 0xffffffffu);
  p.key1 = (uint32_t)(seed_ >> 32);
  p.step = (uint32_t)step_;
  p.nf = (int)P.fields.size();
  int nt = 0, npres = 0, ts = 0;
  for (int fi = 0; fi < p.nf; ++fi) {
    const int f = P.fields[fi];
    const HostField& hf = FS[f];
    FieldK& K = p.f[fi];
    K.cur = have_dev ? state_[par_[f]][f] : nullptr;
    K.next = have_dev ? state_[par_[f] ^ 1][f] : nullptr;
    K.chan = (alias_order_[f] > 1) ? (have_dev ? (dim_ == 3 ? chanz_[f] : chan_[f]) : (float2*)&p) : nullptr;
    any_chan = any_chan || (K.chan != nullptr);
    K.dynamic = hf.dynamic ? 1 : 0;
    K.noisy = hf.noisy ? 1 : 0;
    K.order = alias_order_[f];
    K.fid = f;
    K.chan_xlimit = sx_ / (K.order + 1);
    K.chan_ylimit = sy_ / (K.order + 1);
    K.chan_zlimit = sz_ / (K.order + 1);
    K.term0 = nt;
    K.nterms = (int)hf.terms.size();
    // states this field's update reads: its own (dynamic, or non-dynamic without terms)
    // and the sources of its single-field terms, each prefetched into one slot
    K.nsrc = 0;
    K.self_src = -1;
    auto src_slot = [&](int g) {
      for (int j = 0; j < K.nsrc; ++j)
        if (K.src[j] == g) return j;
      if (K.nsrc >= kMaxSrc) throw Error(kErrLimit, "a field reads too many other fields");
      K.src[K.nsrc] = g;
      return K.nsrc++;
    };
    if (hf.dynamic || hf.terms.empty()) K.self_src = src_slot(f);
    for (size_t t = 0; t < hf.terms.size(); ++t, ++ts) {
      const HostTerm& ht = hf.terms[t];
      TermK& T = p.term[nt++];
      if (ht.product.empty()) {
        T.kind = kTermConst;
        T.src = 0;
      } else if (ht.product.size() == 1) {
        T.kind = kTermSingle;
        T.src = src_slot(ht.product[0]);
      } else if (P.term_slot[ts] == -2) {
        T.kind = kTermMerged;   // summed into its group's first term's channel
        T.src = 0;
      } else {
        T.kind = kTermProduct;
        T.src = P.term_slot[ts];
      }
      // precomputePrefactors sign rule (src/term_init.cpp:145-156)
      const int s = (ht.pres[0].iqx + ht.pres[0].iqy + ht.pres[0].iqz) % 2;
      T.s = s;
      T.pres0 = npres;
      T.npres = (int)ht.pres.size();
      for (const HostPres& hp : ht.pres) {
        const int u = hp.iqx + hp.iqy + hp.iqz;
        const int negate = -2 * (((u - s) / 2) % 2) + 1;
        PresK& K2 = p.pres[npres++];
        K2.pre = hp.pre * (float)negate;
        K2.q2n = hp.q2n;
        K2.iqx = hp.iqx;
        K2.iqy = hp.iqy;
        K2.iqz = hp.iqz;
        K2.invq = hp.invq;
      }
    }
    K.imp0 = npres;
    K.nimp = (int)hf.implicit.size();
    for (const HostPres& hp : hf.implicit) {
      PresK& K2 = p.pres[npres++];
      K2.pre = hp.pre;
      K2.q2n = hp.q2n;
      K2.iqx = hp.iqx;
      K2.iqy = hp.iqy;
      K2.iqz = hp.iqz;
      K2.invq = hp.invq;
    }
    if (hf.noisy) {
      // precalculateImplicit noise factor (src/field_init.cpp:239-241, 269-278)
      const float ddx = (float)(2.0 * (double)kPiF / (double)(stepq_[0] * (float)sx_));
      const float ddy = (float)(2.0 * (double)kPiF / (double)(stepq_[1] * (float)sy_));
      const float ddz = (float)(2.0 * (double)kPiF / (double)(stepq_[2] * (float)sz_));
      float base = std::sqrt(dt_ / (ddx * ddy * ddz) * hf.noise.pre);
      if (!hf.dynamic) base *= 1.0f / std::sqrt(dt_);   // setNotDynamic_k (field_kernels.cu:155)
      K.noise_base = base;
      K.noise_q2n = hf.noise.q2n;
      K.noise_invq = hf.noise.invq;
    }
  }
  int max_src = 0;
  for (int fi = 0; fi < p.nf; ++fi) max_src = std::max(max_src, p.f[fi].nsrc);
  p.src_slots = max_src;
  // the inverse transform of the dealiased copies reuses slot 0 when the phase has one
  // field; with several, it gets its own so the next field's states can stream in
  const int data_slots = p.n_prod + max_src;
  const bool own_tslot = any_chan && (p.nf > 1 || data_slots == 0);
  p.tslot = own_tslot ? data_slots : 0;
  nslots = data_slots + (own_tslot ? 1 : 0);
}

const std::string& Solver::turn_source(Phase& P, const LineParams& p, int L, int nl) {
  std::vector<int> sig = {L, nl, p.nf, p.n_prod, p.sx, p.sy, p.sz, p.W};
  for (int fi = 0; fi < p.nf; ++fi) {
    const FieldK& K = p.f[fi];
    sig.insert(sig.end(), {K.dynamic, K.noisy, K.nterms, K.term0, K.nimp, K.imp0, K.noise_q2n, K.noise_invq,
                           K.self_src, K.nsrc});
  }
  int np = 0;
  for (int t = 0; t < kMaxTerms; ++t) {
    const TermK& T = p.term[t];
    sig.insert(sig.end(), {T.kind, T.src, T.s, T.npres, T.pres0});
    np = std::max(np, T.pres0 + T.npres);
  }
  for (int fi = 0; fi < p.nf; ++fi) np = std::max(np, p.f[fi].imp0 + p.f[fi].nimp);
  for (int j = 0; j < np; ++j) {
    const PresK& q = p.pres[j];
    sig.insert(sig.end(), {q.q2n, q.iqx, q.iqy, q.iqz, q.invq});
  }
  sig.push_back(phase_warps(P));
  sig.push_back(phase_split(P) ? 1 : 0);
  sig.push_back(batch_ ? 1 : 0);
  if (sig != P.jit_sig) {
    P.jit_sig = sig;
    P.jit_src = jit_generate_turn(p, L, nl, phase_warps(P), batch_, phase_split(P));
  }
  return P.jit_src;
}

std::vector<std::string> Solver::generated_sources() {
  if (!prepared_) build_plan();
  std::vector<std::string> out;
  const int L = (dim_ == 3) ? sz_ : sy_;
  const int nl = (dim_ == 3) ? 2 : 1;
  for (Phase& P : phases_) {
    if (P.fields.empty()) continue;
    LineParams p;
    int nslots = 0;
    bool any_chan = false;
    fill_turn(P, p, nslots, any_chan);
    out.push_back(jit_generate_turn(p, L, nl, phase_warps(P), batch_, phase_split(P)));
  }
  return out;
}

void Solver::run_phase(Phase& P) {
  if (P.fields.empty()) return;
  // ---- xy-plane pass (3D, one channel, one product): the product plane by plane ----
  if (!P.products.empty() && plane_) {
    const int g = P.xin[0];
    PlaneParams pp;
    std::memset(&pp, 0, sizeof(pp));
    pp.nc = std::min(Lx_, sx_ / (alias_order_[g] + 1) + 1);
    pp.ykeep = sy_ / (alias_order_[g] + 1) + 1;
    size_t smem = 0;
    const int cl = plane_pass_shape(Lx_, sy_, pp.nc, &pp.ps, &smem, plane_c_);
    if (cl <= 0) throw Error(kErrUnsupported, "plane pass shape");
    pp.order = (int)P.products[0].size();
    pp.out_scale = 1.f;
    pp.in = chanz_[g];
    pp.out = P.prodbuf[0];
    pp.tw = tw_;
    pp.members = members_d_;
    if (batch_) pp.mstride = half_;
    mark_begin();
    check(launch_plane_pass(pp, Lx_, sy_, sz_, batch_ ? mspan_ : 1, cl, stream_, pdl_), "plane pass");
    mark_end("plane_pass");
    ++launches_;
  }
  // ---- row pass: real-space products of the dealiased copies ----
  if (!P.products.empty() && !plane_) {
    XParams x;
    row_params(P, x);
    mark_begin();
    check(launch_row_pass(x, stream_, batch_ ? mspan_ : 1, pdl_), "row pass");
    mark_end("row_pass");
    ++launches_;
    if (dim_ == 3) {
      for (int c = 0; c < P.nchan; ++c) {
        float2* b = P.prodbuf[P.chan_buf[c]];
        mark_begin();
        line_fwd_inv(kGeoY3, kModeFwd, b, b, Lx_, batch_, 0, pdl_);
        mark_end("line_fwd_y");
      }
    }
  }
  // ---- turnaround ----
  const int geo = (dim_ == 3) ? kGeoZ3 : kGeoCol;
  const int L = (dim_ == 3) ? sz_ : sy_;
  const int nl = (dim_ == 3) ? 2 : 1;
  LineParams p;
  int nslots = 0;
  bool any_chan = false;
  fill_turn(P, p, nslots, any_chan);
  p.W = phase_turn_w(P, nslots);
  p.members = members_d_;
  p.step_off = step_off_;
  if (batch_) {
    p.mstride = half_;
    p.mvals = mvals_d_[P.id];
  }
  // 3D: one more tile index for the packed column kx' = 0 (see LineGeom)
  dim3 grid((Lx_ + p.W - 1) / p.W + (dim_ == 3 ? 1 : 0), dim_ == 3 ? std::max(sy_ / 2, 1) : 1,
            batch_ ? mspan_ : 1);
  mark_begin();
  if (use_jit_) {
    // the kernel is compiled for the tuned tile width; while tuning, one width-generic
    // kernel serves every candidate
    LineParams ps = p;
    if (tuning_) ps.W = 0;
    const std::string& src = turn_source(P, ps, L, nl);
    cudaKernel_t k = jit_kernel(src, "cupssgb_turn");
    dim3 block(p.W, line_threads(L, 1, 1, phase_split(P)), nl);
    void* args[] = {(void*)&p};
    LaunchCfg lc(grid, block, line_pass_smem(L, nl, p.W, nslots, phase_split(P)), stream_, pdl_);
    check(cudaLaunchKernelExC(&lc.cfg, (const void*)k, args), "turnaround (generated)");
  } else {
    check(launch_line_pass(p, nl, nslots, grid, stream_, pdl_), "turnaround");
  }
  mark_end(dim_ == 3 ? "turnaround_z" : "turnaround_y");
  ++launches_;
  for (int f : P.fields) par_[f] ^= 1;
  if (dim_ == 3 && any_chan && !plane_) {
    for (int f : P.fields)
      if (alias_order_[f] > 1) {
        mark_begin();
        // rows |n_y| > sy/(order+1) of the z-inverted channel are masked (zero)
        line_fwd_inv(kGeoY3, kModeInv, chanz_[f], chan_[f], sx_ / (alias_order_[f] + 1), batch_,
                     sy_ / (alias_order_[f] + 1) + 1, pdl_);
        mark_end("line_inv_y");
      }
  }
}

void Solver::row_params(const Phase& P, XParams& x) const {
  std::memset(&x, 0, sizeof(x));
  x.Lx = Lx_;
  x.rows = sy_ * sz_;
  x.in_mode = kXInSpectral;
  x.out_mode = kXOutSpectral;
  x.out_scale = 1.f;
  x.n_in = (int)P.xin.size();
  for (int i = 0; i < x.n_in; ++i) {
    const int g = P.xin[i];
    x.in[i] = g < (int)chan_.size() ? chan_[g] : nullptr;   // no buffers before prepare (source generation)
    // columns beyond the dealias limit of the channel are zero: not read
    x.in_xcols[i] = chan_wide_[g] ? 0 : std::min(Lx_, sx_ / (alias_order_[g] + 1) + 1);
  }
  x.n_prod = (int)P.products.size();
  for (int q = 0; q < x.n_prod; ++q) {
    x.prod_add[q] = P.prod_add[q];
    x.out[q] = q < (int)P.prodbuf.size() ? P.prodbuf[q] : nullptr;
    x.prod_n[q] = (int)P.products[q].size();
    for (int t = 0; t < x.prod_n[q]; ++t) {
      const int g = P.products[q][t];
      x.prod_f[q][t] = (int)(std::find(P.xin.begin(), P.xin.end(), g) - P.xin.begin());
    }
  }
  x.tw = tw_;
  x.members = members_d_;
  if (batch_) x.mstride = half_;
}

void Solver::mark_begin() {
  if (!timing_) return;
  if (ev_used_ + 2 > ev_pool_.size()) {
    for (int i = 0; i < 64; ++i) {
      cudaEvent_t e;
      check(cudaEventCreate(&e), "cudaEventCreate");
      ev_pool_.push_back(e);
    }
  }
  check(cudaEventRecord(ev_pool_[ev_used_], stream_), "cudaEventRecord");
  ev_marks_.push_back({std::string(), ev_used_});
  ev_used_ += 2;
}

void Solver::mark_end(const char* kind) {
  if (!timing_) return;
  const size_t b = ev_marks_.back().second;
  ev_marks_.back().first = kind;
  check(cudaEventRecord(ev_pool_[b + 1], stream_), "cudaEventRecord");
  if (ev_used_ + 2 > 4096) flush_timing();
}

void Solver::flush_timing() {
  if (ev_marks_.empty()) return;
  check(cudaStreamSynchronize(stream_), "timing sync");
  for (const auto& mk : ev_marks_) {
    float ms = 0.f;
    check(cudaEventElapsedTime(&ms, ev_pool_[mk.second], ev_pool_[mk.second + 1]), "cudaEventElapsedTime");
    bool found = false;
    for (auto& kt : ktimes_)
      if (kt.first == mk.first) {
        kt.second.first += 1;
        kt.second.second += ms;
        found = true;
      }
    if (!found) ktimes_.push_back({mk.first, {1, (double)ms}});
  }
  ev_marks_.clear();
  ev_used_ = 0;
}

void Solver::set_kernel_timing(bool on) {
  if (timing_ && !on) flush_timing();
  timing_ = on;
  if (on) {
    ktimes_.clear();
    ev_marks_.clear();
    ev_used_ = 0;
  }
}

std::string Solver::kernel_report() {
  flush_timing();
  std::ostringstream os;
  os << "{";
  for (size_t i = 0; i < ktimes_.size(); ++i) {
    if (i) os << ", ";
    os << "\"" << ktimes_[i].first << "\": {\"launches\": " << ktimes_[i].second.first
       << ", \"ms\": " << ktimes_[i].second.second << "}";
  }
  os << "}";
  return os.str();
}

double Solver::time_advance(int nsteps) {
  cudaEvent_t a, b;
  check(cudaEventCreate(&a), "cudaEventCreate");
  check(cudaEventCreate(&b), "cudaEventCreate");
  check(cudaEventRecord(a, stream_), "cudaEventRecord");
  advance(nsteps);
  check(cudaEventRecord(b, stream_), "cudaEventRecord");
  check(cudaEventSynchronize(b), "cudaEventSynchronize");
  float ms = 0.f;
  check(cudaEventElapsedTime(&ms, a, b), "cudaEventElapsedTime");
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms;
}

// One time step; its noise uses step count + off.  tick: advance the device step counts.
void Solver::step_once(uint32_t off, bool tick) {
  step_off_ = off;
  run_phase(phases_[0]);
  run_phase(phases_[1]);
  step_off_ = 0;
  if (tick) {
    check(launch_tick(members_d_, nmem_, off + 1u, stream_, pdl_), "member step count");
    ++launches_;
  }
  ++step_;
}

void Solver::advance(int nsteps) {
  if (!prepared_) throw Error(kErrState, "advance before prepare");
  if (batch_ && mvals_dirty_) upload_member_values();
  check_merges();
  if (!timing_) {
    for (int c = 0; c < 3; ++c)
      for (; nsteps >= kGraphChunks[c]; nsteps -= kGraphChunks[c]) run_graph(c);
  }
  for (int s = 0; s < nsteps; ++s) step_once(0, true);
}

}  // namespace cupssgb
