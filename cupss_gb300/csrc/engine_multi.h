// Fused stepping of several batched solvers of one system structure on different grids.
#pragma once
#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "engine.h"

namespace cupssgb {

// Batched solvers ("grid classes") of one system structure on different 1D/2D grids,
// stepped together: every kernel of a step is one launch over all of them.  The fused
// turnaround and row pass are generated per set of classes (jit_generate_multi): each
// class's body is specialised to its grid, owns a contiguous range of blockIdx.x and sees
// its own members at blockIdx.z, so per-member data and noise are exactly those of the
// class's own launches: a member's trajectory is the one it has in its own solver, to
// rounding (the fused row pass is compiled by NVRTC, the solver's own by nvcc).
// Steps are replayed from CUDA graphs of 16, 4 and 1 steps.  The classes keep their
// buffers, member tables and set/get calls; stepping runs on this object's stream, which
// waits for the classes' streams before each advance (and they for it after).
class MultiStep {
 public:
  // "" when the solvers can be stepped fused, else the reason they cannot.  With
  // need_prepared false, unprepared solvers have their plans built (no GPU needed).
  static std::string unsupported(const std::vector<Solver*>& s, bool need_prepared = true);
  // Source of the fused kernels of phase ph (0 non-dynamic, 1 dynamic; "" when the phase
  // has no fields): needs no GPU.
  static std::string generated_source(const std::vector<Solver*>& s, int ph);
  explicit MultiStep(const std::vector<Solver*>& s);
  ~MultiStep();
  MultiStep(const MultiStep&) = delete;
  MultiStep& operator=(const MultiStep&) = delete;
  void advance(int nsteps);
  long long launches() const { return launches_; }
  std::string describe() const;   // JSON: per class grid, tile width, CTAs; the form chosen
  // Times the fused launches against every class stepping alone on its own stream
  // (their own tuned graphs, running concurrently), 16 steps each after 16 warm-up steps,
  // on the solvers' current buffers, and steps with the faster form from then on.  The
  // buffers are zeroed and every member is back at step 0 afterwards, as after prepare,
  // so call it before setting fields.  The choice is cached in the tune cache (key: GPU,
  // grids, member spans, kernel sources) and taken from there the next time.
  void choose();
  bool fused() const { return fused_; }

 private:
  struct PhaseK {
    bool active = false, has_row = false;
    cudaKernel_t turn = nullptr, row = nullptr;
    int turn_threads = 0;   // threads of a fused turnaround CTA: W_c * M_c for every class c
    size_t turn_smem = 0, row_smem = 0;
    dim3 turn_grid, row_grid;
    std::vector<int> turn_w, turn_tiles, row_blocks;
  };
  // Launch shapes of phase ph and (src != nullptr) the source of its fused kernels;
  // "" when every class fits them, else the reason.
  static std::string plan_phase(const std::vector<Solver*>& s, int ph, PhaseK& K, std::string* src);
  static void check(cudaError_t e, const char* what);
  void build();
  void launch_phase(int ph, uint32_t off);
  void step_once(uint32_t off, bool tick);
  void capture(int c, int parity);

  void restart();      // zero buffers, members at step 0 (after timing)
  void invalidate();   // drop the captured graphs (after the launch mode changed)
  std::string choice_key() const;

  std::vector<Solver*> s_;
  PhaseK ph_[2];
  uint64_t src_hash_ = 0;   // of the fused kernels' sources
  bool fused_ = true;       // false: every class steps on its own stream
  bool pdl_ = false;        // the fused launches use programmatic dependent launch
  bool choice_cached_ = false, chosen_ = false;
  double ms_fused_ = -1.0, ms_grouped_ = -1.0;   // per step, from choose() (fused: the better launch mode)
  double ms_fused_pdl_[2] = {-1.0, -1.0};        // fused, without / with programmatic dependent launch
  cudaStream_t stream_ = nullptr;
  cudaEvent_t ev_ = nullptr;
  std::vector<cudaEvent_t> class_ev_;
  cudaGraphExec_t graph_[3][2] = {};
  std::vector<int> graph_span_;   // the classes' member spans the graphs were captured with
  std::vector<int> epoch_;        // the classes' plan epochs the fused kernels were built for
  long long graph_launches_[3] = {};
  long long launches_ = 0;
  // parameter blocks of the fused launches (27 KB and 4 KB), built per launch
  std::unique_ptr<MultiTurnParams> mt_;
  std::unique_ptr<MultiRowParams> mr_;
};

}  // namespace cupssgb
