// ensemble: many independent solves of one system advanced together.
//
// No counterpart in the reference (its evolver runs one system per object).  The
// system is declared once, with the evolver's calls and string equations; each
// member then picks its grid, time step, seed and parameter values.  prepare()
// groups members that share a grid, time step and equation structure into batch
// solvers (one set of launches per step for the whole group, replayed from CUDA
// graphs, each group on its own stream so groups overlap on the GPU).  A member's
// result is the same as that of an evolver with the same system, values, seed and
// initial fields (tests/test_gpu_batch.py).
#ifndef CUPSS_GB300_ENSEMBLE_H
#define CUPSS_GB300_ENSEMBLE_H

#include <string>

class ensemble {
 public:
  ensemble();
  ~ensemble();
  ensemble(const ensemble&) = delete;
  ensemble& operator=(const ensemble&) = delete;

  // The system, as on an evolver (addParameter gives the default value).
  int createField(const std::string& name, bool dynamic);
  int addParameter(const std::string& name, float value);
  int addEquation(const std::string& equation);
  int addNoise(const std::string& field, const std::string& amplitude);

  // A member: grid (2^a or 3*2^a per axis), cell sizes, time step and noise seed.  Returns the
  // member index.  Parameters not set per member keep their defaults.
  int addMember(int sx, int sy, int sz, float dx, float dy, float dz, float dt, unsigned long long seed);
  int setMemberParameter(int member, const std::string& name, float value);

  // Parses every member's system, builds and autotunes the batch solvers.  Fields start
  // at zero; setReal gives initial conditions (sx*sy*sz floats, the evolver's layout).
  void prepare();
  int setReal(int member, const std::string& field, const float* host_real);
  // nsteps time steps of every member; returns when done.  Members are grouped by grid
  // (and cell size, time step); the groups step concurrently on their own streams, or,
  // when every group is a 1D/2D grid of the same system structure (up to 8 groups), each
  // kernel of a step may be one launch over all groups (fused()).  prepare times both
  // forms and keeps the faster (CUPSSGB_FUSE=1 / 0 forces fused / separate).
  int advance(int nsteps);
  int getReal(int member, const std::string& field, float* host_real);

  int members() const;
  int groups() const;
  long long deviceBytes() const;
  long long launches() const;
  bool fused() const;
  // JSON {"groups": [per group: grid, members, autotuned launch shapes], "fused": the fused
  // launches per grid class, the form chosen and both forms' ms per step, or null with
  // "why_not_fused"}.
  std::string describe() const;

 private:
  struct Impl;
  Impl* impl_;
};

#endif  // CUPSS_GB300_ENSEMBLE_H
