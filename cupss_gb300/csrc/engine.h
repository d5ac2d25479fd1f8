// GB300 pseudospectral engine: host planner and device state for one system.
//
// A system is a set of scalar fields on an sx*sy*sz periodic grid.  Each field
// carries implicit q-monomials, explicit terms (a product of fields times a sum of
// q-monomials) and optional Gaussian noise -- exactly the IR that the reference's
// parser produces (src/parser.cpp:628-767) and that its field/term classes execute
// (src/field.cpp, src/term.cpp).  The engine executes one reference time step
// (src/evolver.cpp:199-226) as two phases (non-dynamic fields, then dynamic ones),
// each phase = [row pass computing the real-space products] + [line-pass turnaround
// doing the Fourier-space update], with 3D adding a y-axis pass on either side.
#pragma once
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>
#include "engine_types.h"

namespace cupssgb {

enum Status : int {
  kOk = 0,
  kErrInvalid = -1,
  kErrCuda = -2,
  kErrUnsupported = -3,
  kErrState = -4,
  kErrParse = -5,
  kErrLimit = -6,
};

struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& msg) : std::runtime_error(msg), code(c) {}
};

struct HostPres {
  float pre = 0.f;
  int q2n = 0, iqx = 0, iqy = 0, iqz = 0, invq = 0;
};

struct HostTerm {
  std::vector<int> product;     // field indices, any order (multiset)
  std::vector<HostPres> pres;
};

struct HostField {
  bool dynamic = false;
  std::vector<HostPres> implicit;
  std::vector<HostTerm> terms;
  bool noisy = false;
  HostPres noise;
};

class Solver {
 public:
  Solver(int sx, int sy, int sz, float dx, float dy, float dz, float dt);
  ~Solver();
  Solver(const Solver&) = delete;
  Solver& operator=(const Solver&) = delete;

  int add_field(bool dynamic);
  void set_implicit(int f, const std::vector<HostPres>& p);
  int add_term(int f, const std::vector<int>& product, const std::vector<HostPres>& p);
  void set_term_pres(int f, int t, const std::vector<HostPres>& p);
  void set_noise(int f, bool on, const HostPres& amp);
  void set_seed(uint64_t s);
  void set_dt(float dt);

  void prepare();
  bool prepared() const { return prepared_; }
  // Scheduling priority of the solver's work: 0 the default, higher levels have their
  // kernels' CTAs scheduled first when several streams compete (clamped to the device's
  // range).  Callable at any time: later work goes to a stream of that priority, ordered
  // after everything queued before.
  void set_stream_priority(int level);
  // m: batch member (0 for a single system).  Returns true when the copy of a host
  // source runs asynchronously (page-locked memory, input stream), false otherwise.
  bool set_real(int f, const float* src, bool src_on_device, int m = 0);
  void advance(int nsteps);
  void get_real(int f, float* dst, bool dst_on_device, int m = 0);
  void get_fourier(int f, float2* dst, bool dst_on_device, int m = 0);
  // Output path of writeOut (src/field.cpp:350-402): copies the real values of field f
  // into host memory without holding up later work on the solver's stream.  The field is
  // materialised on the solver's stream into a device staging buffer of its own; the
  // device-to-host copy then runs on a separate output stream, and `done` (if not null) is
  // recorded there once the host copy is complete.  host_dst should be page-locked for the
  // copy to be asynchronous.  Each field has two staging buffers, used in turn; a snapshot
  // first waits until the copy of the one before the previous has left its buffer.
  void snapshot_real(int f, float* host_dst, cudaEvent_t done);

  // ---- batches: n independent systems of this structure and grid in one solver ----
  // set_members(n) before prepare turns the solver into a batch.  Member 0 starts as the
  // system given by the add_* calls and members 1..n-1 as copies of it; each member can
  // then get its own prefactor values (same monomials), noise amplitude and seed.  Every
  // step launch covers all members (blockIdx.z = member); a member's noise counter is
  // its own step count, so its trajectory does not depend on the rest of the batch.
  // Steps are replayed from CUDA graphs of kGraphSteps, 4 and 1 steps (single systems
  // too); a single system captures them at prepare, so advance() replays from its first
  // call on.
  void set_members(int n);
  int members() const { return nmem_; }
  bool batched() const { return batch_; }
  void set_member_term_pres(int m, int f, int t, const std::vector<HostPres>& p);
  void set_member_implicit(int m, int f, const std::vector<HostPres>& p);
  void set_member_noise(int m, int f, const HostPres& amp);
  void set_member_seed(int m, uint64_t seed);
  void set_member_active(int m, bool on);     // inactive members are skipped by every launch
  void reset_member(int m);                   // zero states and copies, step count 0
  long long member_step(int m);
  std::string tune_report() const;            // JSON: autotuned launch shapes per phase
  // Device bytes prepare() would allocate for a batch of `members` (no GPU needed).
  size_t estimate_bytes(int members);
  bool idle();                                // all queued work on the stream has finished
  static constexpr int kGraphSteps = 16;
  void get_real_pairs_device(int f, float2* dst);   // reference float2 layout (x, 0)
  // Materialisation points for callbacks (src/field.cpp:48-86), all device pointers in
  // the reference's layouts, ordered on the solver's stream:
  void advance_phase(int phase);                    // 0: non-dynamic, 1: dynamic (+ step count)
  void get_dealiased_pairs_device(int f, float2* dst);
  void set_fourier_device(int f, const float2* full);          // also re-derives the dealiased copy
  void set_real_pairs_device(int f, const float2* real, const float2* dealiased);
  void synchronize();
  // Kernel timing: when on, every launch of advance() is bracketed by CUDA events on
  // the solver's stream and its duration is accumulated per kernel kind.
  void set_kernel_timing(bool on);
  std::string kernel_report();   // JSON {kind: {"launches": n, "ms": t}}
  double time_advance(int nsteps);   // advance + CUDA-event elapsed ms on the stream
  // CUDA sources of the specialised turnaround kernels (one per non-empty phase);
  // needs no GPU (the plan is built if prepare has not run).
  std::vector<std::string> generated_sources();
  void set_use_jit(bool on) { use_jit_ = on; }
  bool use_jit() const { return use_jit_; }

  int sx() const { return sx_; }
  int sy() const { return sy_; }
  int sz() const { return sz_; }
  int dim() const { return dim_; }
  size_t npoints() const { return (size_t)sx_ * sy_ * sz_; }
  int nfields() const { return (int)fields_.size(); }
  long long step_count() const { return step_; }
  long long launches() const { return launches_; }
  cudaStream_t stream() const { return stream_; }
  size_t device_bytes() const { return dev_bytes_; }
  const HostField& field(int f) const { return fields_.at(f); }
  bool needs_alias(int f) const { return alias_order_.at(f) > 1; }
  int alias_order(int f) const { return alias_order_.at(f); }

 private:
  friend class MultiStep;   // engine_multi.cpp: fused launches over several batched solvers
  struct Phase {
    int id = 0;                              // 0: non-dynamic, 1: dynamic
    std::vector<int> fields;                 // fields updated in this phase
    std::vector<std::vector<int>> products;  // sorted multisets (size >= 2), channel by channel
    std::vector<int> prod_add;               // per product: added into the previous one's channel
    int nchan = 0;                           // product channels (sums of products) of the turnaround
    std::vector<int> chan_buf;               // per channel: the product whose buffer holds it (its last)
    std::vector<std::vector<std::pair<int, int>>> groups;   // merged terms (field, term) per channel
    std::vector<int> xin;                    // fields feeding the row pass
    std::vector<float2*> prodbuf;
    std::vector<int> term_slot;              // per (field, term) flattened: product slot or -1
    std::vector<int> jit_sig;                // structure of the last generated update program
    std::string jit_src;
    int tuned_w = 0;                         // autotuned turnaround tile width (0: pick_w's rule)
    int tuned_warps = 0;                     // resident-warp target of its registers (0: the solver's)
    int tuned_split = -1;                    // 512/1024-point lines: 1 split form, 0 four-step, -1 rule
    bool tune_cached = false;                // the shape came from the tune cache
    int tune_pdl = -1;                       // cached programmatic-dependent-launch choice (-1: none)
    double tune_best_ms = 0.0;               // the tuned shape's time per phase run
    std::vector<std::pair<std::string, double>> tune_ms;   // candidate -> ms per phase run
  };

  void check(cudaError_t e, const char* what);
  void* dalloc(size_t bytes, bool zero = true);
  void build_plan();
  // Distinct products of a phase, their channels and the terms' slots.  With `merge`,
  // product terms of one field with identical prefactor lists (for every batch member)
  // whose products no other term of the phase uses share one channel: the row pass sums
  // their real-space products before one forward transform, and the update applies the
  // prefactors once (KPZ's 0.5*lambda*iqxh^2 + 0.5*lambda*iqyh^2).
  void plan_products(Phase& P, bool merge);
  bool merges_hold() const;   // every merged group still has equal prefactors
  // After prefactor changes: if a merged group's terms now differ, the solver drops
  // merging (products keep their buffers; kernels and graphs are rebuilt).
  void check_merges();
  void run_phase(Phase& ph);
  // the row pass of a phase with products (its products from the dealiased channels)
  void row_params(const Phase& P, XParams& x) const;
  void fill_turn(const Phase& P, LineParams& p, int& nslots, bool& any_chan,
                 const std::vector<HostField>* fields = nullptr) const;
  const std::string& turn_source(Phase& P, const LineParams& p, int L, int nl);
  void fill_line_common(LineParams& p, int L, int geo, int mode) const;
  // other: CTAs of the launch along its second grid axis (0: no SM-coverage rule);
  // split: the lines use the split FFT form
  int pick_w(int L, int nl, int nslots, int other = 0, bool split = false) const;
  int turn_rows() const { return dim_ == 3 ? std::max(sy_ / 2, 1) : 1; }
  // the phase's turnaround runs the generated kernel with lines in the split FFT form
  bool phase_split(const Phase& P) const;
  int phase_warps(const Phase& P) const { return P.tuned_warps > 0 ? P.tuned_warps : turn_warps_; }
  // turnaround tile width of a phase: the tuned one, else the rule (and CUPSSGB_TURN_W)
  int phase_turn_w(const Phase& P, int nslots) const;
  int turn_len() const { return dim_ == 3 ? sz_ : sy_; }
  // autotuner: cache key of a phase, its value string, and applying a cached value
  std::string tune_key(const Phase& P);
  std::string tune_value(const Phase& P, double ms) const;
  bool apply_tune_value(Phase& P, const std::string& v, int wmax_rule);
  // lkeep > 0: inverse-pass input positions with |n| >= lkeep along the line are zero
  void line_fwd_inv(int geo, int mode, const float2* in, float2* out, int xlimit, bool batch = false,
                    int lkeep = 0, bool pdl = false);
  // real values of field f (member m) into dst (the real scratch array when null)
  void to_real_scratch(int f, int m, float* dst = nullptr);
  // 3D: phases whose products are one channel's power run the xy-plane pass (plane.cuh)
  // in place of a row pass and two y passes; decided at prepare (plane_)
  bool plane_phase(const Phase& P) const;
  bool decide_plane() const;
  void leave_plane_mode();                       // back to the row-pass form (see set_real_pairs_device)
  // keeps the row-pass channels current when the plane pass is switched off
  void sync_row_channels();
  void channelz_from_state(int f, float2* dst);  // masked state / N, z-inverted (plane-pass input)
  void step_once(uint32_t off, bool tick);
  // batches
  void check_member(int m) const;
  void check_same_monomials(const std::vector<HostPres>& a, const std::vector<HostPres>& b) const;
  void upload_member_values();
  void autotune();
  void zero_dynamic_buffers();
  void invalidate_graphs();
  // chunk index c: kGraphChunks[c] steps; parity: the ping-pong parity the graph starts at
  void capture_graph(int c, int parity);
  void capture_all_graphs();
  void run_graph(int c);
  void row_pass_simple(int in_mode, const void* in, int out_mode, void* out, float scale);
  void forward_lines(float2* st);
  void channel_from_state(int f, float2* dst);
  void mark_begin();
  void mark_end(const char* kind);
  void flush_timing();

  int sx_, sy_, sz_, dim_, Lx_;
  float dx_, dy_, dz_, dt_;
  float stepq_[3];
  uint64_t seed_ = 0x243F6A8885A308D3ull;
  std::vector<HostField> fields_;
  std::vector<int> alias_order_;
  // chan_wide_[f]: the dealiased channel of f may hold content beyond its dealias limit
  // (a real-space callback wrote it), so the row pass reads every column of it
  std::vector<char> chan_wide_;
  bool prepared_ = false;
  bool use_jit_ = true;
  int turn_w_ = 0;            // 0: automatic tile width
  int turn_warps_ = 16;       // resident warps per SM the generated turnaround's registers are sized for
  bool tuning_ = false;       // autotune in progress: run the width-generic generated kernel
  bool pdl_ = true;           // step kernels use programmatic dependent launch
  int pdl_env_ = -1;          // CUPSSGB_PDL (0/1), -1: tuned
  double pdl_ms_[2] = {0.0, 0.0};   // ms per step of a 16-step graph without / with it (0: not timed)
  bool plane_ok_ = false;     // every product phase can run the xy-plane pass (decide_plane)
  bool plane_ = false;        // 3D products by the xy-plane pass: chosen by the tuner among plane_ok_
  int plane_c_ = 0;           // CTAs per plane of the plane pass (0: the shape's default)
  int plane_env_ = -1;        // CUPSSGB_PLANE: 0 never the plane pass, 1 always where it applies, unset: tuned
  long long step_ = 0;
  long long launches_ = 0;
  size_t dev_bytes_ = 0;
  // batches
  int nmem_ = 1;
  bool merge_off_ = false;     // product merging dropped (a merged group diverged) or CUPSSGB_MERGE=0
  bool merge_check_ = false;   // prefactors changed since the merges were last checked
  int plan_epoch_ = 0;         // incremented when the phases are re-planned after prepare
  int stream_level_ = 0;   // set_stream_priority before prepare
  // one stream per priority in use (index: levels above the default), stream_ is one of them
  static constexpr int kMaxLevels = 8;
  cudaStream_t level_streams_[kMaxLevels] = {};
  int level_index_ = 0;
  cudaEvent_t level_ev_ = nullptr;
  int mspan_ = 1;   // members covered by step launches: 1 + the last active slot
  bool batch_ = false;
  size_t half_ = 0;                              // elements of one member's spectrum
  std::vector<std::vector<HostField>> mfields_;  // per member (values only differ)
  std::vector<MemberK> members_h_;
  MemberK* members_d_ = nullptr;
  float* mvals_d_[2] = {nullptr, nullptr};
  bool mvals_dirty_ = false;
  uint32_t step_off_ = 0;                        // step offset of the launches being issued
  static constexpr int kGraphChunks[3] = {kGraphSteps, 4, 1};
  cudaGraphExec_t graph_[3][2] = {};   // by chunk and by the ping-pong parity it starts at
  long long graph_launches_[3] = {};   // kernels per replay of each chunk

  cudaStream_t stream_ = nullptr;
  float2* tw_ = nullptr;
  std::vector<float2*> state_[2];
  std::vector<int> par_;
  std::vector<float2*> chan_;    // row-pass input (x spectrum, y/z positional)
  std::vector<float2*> chanz_;   // 3D: z-inverse output (the plane pass's input, or the y-inverse's)
  float* scratch_real_ = nullptr;
  float2* scratch_spec_ = nullptr;
  float2* scratch_full_ = nullptr;   // reference-layout full spectrum, allocated on first use
  // output path (snapshot_real), created on first use
  cudaStream_t out_stream_ = nullptr;
  std::vector<float*> out_stage_;          // per field, two: staging copies of the real values
  std::vector<cudaEvent_t> out_ready_;     // per staging buffer: written (solver stream)
  std::vector<cudaEvent_t> out_free_;      // per staging buffer: read out (output stream)
  std::vector<int> out_next_;              // per field: the staging buffer of its next snapshot
  // input path (set_real from page-locked host memory), created on first use: the copy
  // runs on its own stream into one of two staging buffers, so that it overlaps the
  // solver stream's work queued before it
  cudaStream_t up_stream_ = nullptr;
  float* up_stage_[2] = {nullptr, nullptr};
  cudaEvent_t up_ready_[2] = {nullptr, nullptr};   // staging copy written (input stream)
  cudaEvent_t up_free_[2] = {nullptr, nullptr};    // staging copy read (solver stream)
  int up_next_ = 0;
  std::vector<void*> allocs_;
  Phase phases_[2];              // 0: non-dynamic, 1: dynamic
  // kernel timing
  bool timing_ = false;
  std::vector<cudaEvent_t> ev_pool_;
  size_t ev_used_ = 0;
  std::vector<std::pair<std::string, size_t>> ev_marks_;   // kind, index of begin event
  std::vector<std::pair<std::string, std::pair<long long, double>>> ktimes_;
};

}  // namespace cupssgb
