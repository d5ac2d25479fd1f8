// server: a request loop that runs many solves on one GPU with continuous batching.
//
// No counterpart in the reference.  Systems are declared once (the evolver's calls);
// requests then name a system, a grid, a time step, a step count, a seed, parameter
// values and initial fields.  A scheduler thread admits requests into slots of
// batch solvers ("pools", one per system structure, grid and time step) while device
// memory stays within an HBM budget, advances every pool with active members in
// chunks of steps (pools on their own streams, so their work overlaps on the GPU),
// retires finished members (result copied to host memory, slot freed) and admits
// waiting requests into freed slots between chunks.  A request's result does not
// depend on what else runs: it equals an evolver solve with the same inputs.
#ifndef CUPSS_GB300_SERVER_H
#define CUPSS_GB300_SERVER_H

#include <map>
#include <string>
#include <vector>

class server {
 public:
  // hbm_budget: device bytes all pools may hold; max_slots: members per pool;
  // max_chunk: most steps a pool runs before new requests can join it.
  explicit server(double hbm_budget = 150e9, int max_slots = 32, int max_chunk = 256);
  ~server();
  server(const server&) = delete;
  server& operator=(const server&) = delete;

  // System declarations (before the first submit that uses the system).
  int addSystem();
  int createField(int system, const std::string& name, bool dynamic);
  int addParameter(int system, const std::string& name, float value);
  int addEquation(int system, const std::string& equation);
  int addNoise(int system, const std::string& field, const std::string& amplitude);
  int setOutputField(int system, const std::string& field);   // returned by result(); default: first

  // Queues a solve; returns its id.  init: field name -> sx*sy*sz floats (copied);
  // fields not given start at zero.  Thread-safe.
  long long submit(int system, int sx, int sy, int sz, float dx, float dy, float dz, float dt, long long nsteps,
                   unsigned long long seed, const std::map<std::string, float>& params,
                   const std::map<std::string, const float*>& init);
  // Creates (and prepares) a pool for this system, grid and time step ahead of time.
  void warm(int system, int sx, int sy, int sz, float dx, float dy, float dz, float dt);
  // Waits up to timeout seconds (< 0: forever); true when the request is done.
  bool wait(long long id, double timeout);
  // The output field of a finished request (sx*sy*sz floats).  Throws if not done.
  void result(long long id, float* host_out);
  // Seconds since the server started: submitted, admitted to a slot, finished.
  void times(long long id, double* submitted, double* admitted, double* finished);
  // JSON: pools, device bytes, requests done / running / queued.
  std::string stats();

 private:
  struct Impl;
  Impl* impl_;
};

#endif  // CUPSS_GB300_SERVER_H
