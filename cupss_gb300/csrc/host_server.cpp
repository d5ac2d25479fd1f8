// server: continuous batching of independent solves (see include/cupss/server.h).
//
// One scheduler thread owns every pool (a batch solver with a fixed number of member
// slots) and runs this loop:
//   1. admit: waiting requests, oldest first, go into a free slot of a pool with their
//      key (system structure, grid, cells, dt); a new pool is created when none has a
//      free slot and the HBM budget allows it (idle pools are freed to make room);
//      admission = reset the slot, load values, seed and initial fields, activate;
//   2. launch: every idle pool with active members advances by a chunk of
//      min(max_chunk, fewest steps left among its members) steps, asynchronously on
//      its own stream -- pools overlap on the GPU;
//   3. retire: when a pool's chunk has finished, members with no steps left have their
//      output field copied to host memory, their slot is deactivated and the request
//      is done; the loop goes back to 1 so freed slots are refilled at once.
// Requests submitted meanwhile wait in the queue; nothing ever waits on a GPU
// without a timeout except the short synchronous copies of admission and retirement.
#include "../../include/cupss/server.h"

#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <sstream>
#include <stdexcept>
#include <thread>
#include <tuple>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/cupss_gb300.h"
#include "host_common.h"
#include "host_ir.h"

using cupssgb_host::IrField;
using cupssgb_host::ok;
using cupssgb_host::SystemOp;

namespace {
using Clock = std::chrono::steady_clock;

struct Sys {
  std::vector<SystemOp> ops;
  std::vector<std::string> fields, params;
  int out = 0;
  bool used = false;
};

struct Request {
  long long id = 0;
  int sys = 0;
  int sx = 1, sy = 1, sz = 1;
  float dx = 1, dy = 1, dz = 1, dt = 0.01f;
  long long nsteps = 0, left = 0;
  unsigned long long seed = 0;
  std::vector<IrField> ir;
  std::string key;
  std::vector<std::pair<int, std::vector<float>>> init;
  double t_submit = -1, t_admit = -1, t_finish = -1;
  int pool = -1, slot = -1;
  std::vector<float> result;
  bool done = false;
  std::string error;
};

struct Pool {
  std::string key;
  int sys = 0, sx = 1, sy = 1, sz = 1;
  cupssgb_solver* s = nullptr;
  std::vector<Request*> slots;    // running request or null
  long long inflight = 0;         // steps of the chunk running now (0: idle)
  long long bytes = 0;
  int active() const {
    int n = 0;
    for (const Request* r : slots) n += r != nullptr;
    return n;
  }
  int free_slots() const { return (int)slots.size() - active(); }
};
}  // namespace

struct server::Impl {
  double budget;
  int max_slots, max_chunk;
  int device = 0;
  Clock::time_point t0 = Clock::now();
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::vector<Sys> systems;
  std::map<long long, std::unique_ptr<Request>> reqs;
  std::deque<long long> queue;   // submitted, not admitted
  std::vector<Pool> pools;
  long long next_id = 1;
  long long used_bytes = 0;
  bool stop = false;
  std::thread worker;
  std::string fatal;   // error that stopped the scheduler

  double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
  Sys& sys(int i) {
    if (i < 0 || i >= (int)systems.size()) throw std::runtime_error("bad system id");
    return systems[i];
  }
  void declare(int i, const SystemOp& op) {
    std::lock_guard<std::mutex> lk(mu);
    Sys& S = sys(i);
    if (S.used) throw std::runtime_error("system already in use: declare it before submitting");
    S.ops.push_back(op);
  }

  void run();
  bool admit_one(Request& r);
  int new_pool(const Request& r);
  void free_idle_pool();
  void retire(Pool& p, int pi);
};

// --------------------------------------------------------------------------------------
// scheduler thread

int server::Impl::new_pool(const Request& r) {
  Pool p;
  p.key = r.key;
  p.sys = r.sys;
  p.sx = r.sx;
  p.sy = r.sy;
  p.sz = r.sz;
  p.s = cupssgb_host::create_solver(r.ir, r.sx, r.sy, r.sz, r.dx, r.dy, r.dz, r.dt);
  try {
    int cap = max_slots;
    long long b = cupssgb_solver_estimate_bytes(p.s, cap);
    while (cap > 1 && used_bytes + b > budget) b = cupssgb_solver_estimate_bytes(p.s, --cap);
    if (b < 0 || used_bytes + b > budget) {
      cupssgb_solver_destroy(p.s);
      return -1;
    }
    ok(cupssgb_solver_set_members(p.s, cap));
    for (int m = 0; m < cap; ++m) {
      cupssgb_host::set_member(p.s, m, r.ir, 0);
      ok(cupssgb_solver_set_member_active(p.s, m, 0));
    }
    ok(cupssgb_solver_prepare(p.s));
    p.bytes = cupssgb_solver_device_bytes(p.s);
    p.slots.assign(cap, nullptr);
  } catch (...) {
    cupssgb_solver_destroy(p.s);
    throw;
  }
  used_bytes += p.bytes;
  pools.push_back(p);
  return (int)pools.size() - 1;
}

void server::Impl::free_idle_pool() {
  for (size_t i = 0; i < pools.size(); ++i)
    if (pools[i].active() == 0 && pools[i].inflight == 0) {
      cupssgb_solver_destroy(pools[i].s);
      used_bytes -= pools[i].bytes;
      pools.erase(pools.begin() + i);
      // pool indices of running requests shift
      std::lock_guard<std::mutex> lk(mu);
      for (auto& kv : reqs)
        if (kv.second->pool > (int)i) kv.second->pool -= 1;
      return;
    }
}

bool server::Impl::admit_one(Request& r) {
  int pi = -1, slot = -1;
  for (size_t i = 0; i < pools.size() && pi < 0; ++i) {
    Pool& p = pools[i];
    if (p.key != r.key || p.inflight) continue;   // slots change only between chunks
    for (size_t k = 0; k < p.slots.size(); ++k)
      if (!p.slots[k]) {
        pi = (int)i;
        slot = (int)k;
        break;
      }
  }
  if (pi < 0) {
    // a busy pool of this key finishes its chunk soon; only grow when none exists
    for (const Pool& p : pools)
      if (p.key == r.key && p.inflight && p.free_slots() > 0) return false;
    pi = new_pool(r);
    while (pi < 0) {
      const size_t n = pools.size();
      free_idle_pool();
      if (pools.size() == n) return false;   // wait for memory
      pi = new_pool(r);
    }
    slot = 0;
  }
  Pool& p = pools[pi];
  ok(cupssgb_solver_reset_member(p.s, slot));
  cupssgb_host::set_member(p.s, slot, r.ir, r.seed);
  for (auto& fi : r.init) ok(cupssgb_solver_set_real_member(p.s, fi.first, slot, fi.second.data()));
  ok(cupssgb_solver_set_member_active(p.s, slot, 1));
  r.init.clear();
  r.left = r.nsteps;
  p.slots[slot] = &r;
  std::lock_guard<std::mutex> lk(mu);
  r.pool = pi;
  r.slot = slot;
  r.t_admit = now();
  return true;
}

void server::Impl::retire(Pool& p, int pi) {
  const long long chunk = p.inflight;
  p.inflight = 0;
  for (size_t k = 0; k < p.slots.size(); ++k) {
    if (!p.slots[k]) continue;
    Request& r = *p.slots[k];
    r.left -= chunk;
    if (r.left > 0) continue;
    r.result.resize((size_t)r.sx * r.sy * r.sz);
    ok(cupssgb_solver_get_real_member(p.s, systems[r.sys].out, (int)k, r.result.data()));
    ok(cupssgb_solver_set_member_active(p.s, (int)k, 0));
    p.slots[k] = nullptr;
    {
      std::lock_guard<std::mutex> lk(mu);
      r.t_finish = now();
      r.pool = -1;
      r.done = true;
    }
    cv_done.notify_all();
  }
  (void)pi;
}

void server::Impl::run() {
  cupssgb_set_device(device);
  try {
    while (true) {
      // 1. admit
      std::vector<Request*> waiting;
      {
        std::unique_lock<std::mutex> lk(mu);
        bool busy = false;
        for (const Pool& p : pools) busy = busy || p.inflight || p.active();
        if (!busy && queue.empty())
          cv_work.wait_for(lk, std::chrono::milliseconds(20), [&] { return stop || !queue.empty(); });
        if (stop) break;
        for (long long id : queue) waiting.push_back(reqs.at(id).get());
      }
      std::vector<long long> admitted;
      for (Request* r : waiting)
        if (admit_one(*r)) admitted.push_back(r->id);
      if (!admitted.empty()) {
        std::lock_guard<std::mutex> lk(mu);
        for (long long id : admitted)
          for (auto it = queue.begin(); it != queue.end(); ++it)
            if (*it == id) {
              queue.erase(it);
              break;
            }
      }
      // 2. launch idle pools with active members
      for (Pool& p : pools) {
        if (p.inflight || p.active() == 0) continue;
        long long chunk = max_chunk;
        for (const Request* r : p.slots)
          if (r) chunk = std::min(chunk, r->left);
        ok(cupssgb_solver_advance(p.s, (int)chunk));
        p.inflight = chunk;
      }
      // 3. retire finished chunks
      bool any = false;
      for (size_t i = 0; i < pools.size(); ++i) {
        Pool& p = pools[i];
        if (!p.inflight) continue;
        const int q = cupssgb_solver_query(p.s);
        if (q < 0) ok(q);
        if (q == 1) {
          retire(p, (int)i);
          any = true;
        }
      }
      if (!any) std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
  } catch (const std::exception& e) {
    std::lock_guard<std::mutex> lk(mu);
    fatal = e.what();
    for (auto& kv : reqs)
      if (!kv.second->done) {
        kv.second->error = fatal;
        kv.second->done = true;
      }
    cv_done.notify_all();
  }
}

// --------------------------------------------------------------------------------------
// public API

server::server(double hbm_budget, int max_slots, int max_chunk) : impl_(new Impl) {
  if (max_slots < 1 || max_chunk < 1) throw std::runtime_error("max_slots and max_chunk must be >= 1");
  impl_->budget = hbm_budget;
  impl_->max_slots = max_slots;
  impl_->max_chunk = max_chunk;
}

server::~server() {
  {
    std::lock_guard<std::mutex> lk(impl_->mu);
    impl_->stop = true;
  }
  impl_->cv_work.notify_all();
  if (impl_->worker.joinable()) impl_->worker.join();
  for (Pool& p : impl_->pools) cupssgb_solver_destroy(p.s);
  delete impl_;
}

int server::addSystem() {
  std::lock_guard<std::mutex> lk(impl_->mu);
  impl_->systems.push_back(Sys());
  return (int)impl_->systems.size() - 1;
}

int server::createField(int system, const std::string& name, bool dynamic) {
  {
    std::lock_guard<std::mutex> lk(impl_->mu);
    for (const std::string& f : impl_->sys(system).fields)
      if (f == name) throw std::runtime_error("field " + name + " declared twice");
  }
  impl_->declare(system, SystemOp{SystemOp::kField, name, "", 0.f, dynamic});
  std::lock_guard<std::mutex> lk(impl_->mu);
  impl_->sys(system).fields.push_back(name);
  return 0;
}

int server::addParameter(int system, const std::string& name, float value) {
  impl_->declare(system, SystemOp{SystemOp::kParameter, name, "", value, false});
  std::lock_guard<std::mutex> lk(impl_->mu);
  impl_->sys(system).params.push_back(name);
  return 0;
}

int server::addEquation(int system, const std::string& equation) {
  impl_->declare(system, SystemOp{SystemOp::kEquation, equation, "", 0.f, false});
  return 0;
}

int server::addNoise(int system, const std::string& field, const std::string& amplitude) {
  impl_->declare(system, SystemOp{SystemOp::kNoise, field, amplitude, 0.f, false});
  return 0;
}

int server::setOutputField(int system, const std::string& field) {
  std::lock_guard<std::mutex> lk(impl_->mu);
  Sys& S = impl_->sys(system);
  for (size_t i = 0; i < S.fields.size(); ++i)
    if (S.fields[i] == field) {
      S.out = (int)i;
      return 0;
    }
  throw std::runtime_error("unknown field " + field);
}

long long server::submit(int system, int sx, int sy, int sz, float dx, float dy, float dz, float dt, long long nsteps,
                         unsigned long long seed, const std::map<std::string, float>& params,
                         const std::map<std::string, const float*>& init) {
  if (nsteps < 1) throw std::runtime_error("nsteps must be >= 1");
  std::unique_ptr<Request> r(new Request);
  std::vector<SystemOp> ops;
  std::vector<std::string> fields, pnames;
  {
    std::lock_guard<std::mutex> lk(impl_->mu);
    if (!impl_->fatal.empty()) throw std::runtime_error("server stopped: " + impl_->fatal);
    Sys& S = impl_->sys(system);
    S.used = true;
    ops = S.ops;
    fields = S.fields;
    pnames = S.params;
  }
  for (const auto& kv : params) {
    bool known = false;
    for (const std::string& p : pnames) known = known || p == kv.first;
    if (!known) throw std::runtime_error("unknown parameter " + kv.first);
  }
  // parse on the caller's thread: errors surface here, not in the scheduler
  r->ir = cupssgb_host::parse_system(ops, params);
  std::ostringstream key;
  key << system << "|" << sx << "x" << sy << "x" << sz << "|" << dx << "," << dy << "," << dz << "|" << dt << "|"
      << cupssgb_host::structure_key(r->ir);
  r->key = key.str();
  r->sys = system;
  r->sx = sx;
  r->sy = sy;
  r->sz = sz;
  r->dx = dx;
  r->dy = dy;
  r->dz = dz;
  r->dt = dt;
  r->nsteps = nsteps;
  r->seed = seed;
  const size_t n = (size_t)sx * sy * sz;
  for (const auto& kv : init) {
    int fi = -1;
    for (size_t i = 0; i < fields.size(); ++i)
      if (fields[i] == kv.first) fi = (int)i;
    if (fi < 0) throw std::runtime_error("unknown field " + kv.first);
    r->init.push_back({fi, std::vector<float>(kv.second, kv.second + n)});
  }
  long long id;
  {
    std::lock_guard<std::mutex> lk(impl_->mu);
    id = impl_->next_id++;
    r->id = id;
    r->t_submit = impl_->now();
    impl_->reqs[id] = std::move(r);
    impl_->queue.push_back(id);
    if (!impl_->worker.joinable()) {
      cudaGetDevice(&impl_->device);
      impl_->worker = std::thread([this] { impl_->run(); });
    }
  }
  impl_->cv_work.notify_all();
  return id;
}

void server::warm(int system, int sx, int sy, int sz, float dx, float dy, float dz, float dt) {
  // a request of one step admitted and finished right away creates the pool
  const long long id = submit(system, sx, sy, sz, dx, dy, dz, dt, 1, 0, {}, {});
  if (!wait(id, -1.0)) throw std::runtime_error("warm-up request did not finish");
  std::lock_guard<std::mutex> lk(impl_->mu);
  if (!impl_->reqs.at(id)->error.empty()) throw std::runtime_error(impl_->reqs.at(id)->error);
  impl_->reqs.erase(id);
}

bool server::wait(long long id, double timeout) {
  std::unique_lock<std::mutex> lk(impl_->mu);
  auto it = impl_->reqs.find(id);
  if (it == impl_->reqs.end()) throw std::runtime_error("unknown request");
  Request* r = it->second.get();
  if (timeout < 0) {
    impl_->cv_done.wait(lk, [&] { return r->done; });
  } else {
    impl_->cv_done.wait_for(lk, std::chrono::duration<double>(timeout), [&] { return r->done; });
  }
  return r->done;
}

void server::result(long long id, float* host_out) {
  std::lock_guard<std::mutex> lk(impl_->mu);
  auto it = impl_->reqs.find(id);
  if (it == impl_->reqs.end()) throw std::runtime_error("unknown request");
  const Request& r = *it->second;
  if (!r.done) throw std::runtime_error("request not finished");
  if (!r.error.empty()) throw std::runtime_error(r.error);
  std::copy(r.result.begin(), r.result.end(), host_out);
}

void server::times(long long id, double* submitted, double* admitted, double* finished) {
  std::lock_guard<std::mutex> lk(impl_->mu);
  auto it = impl_->reqs.find(id);
  if (it == impl_->reqs.end()) throw std::runtime_error("unknown request");
  if (submitted) *submitted = it->second->t_submit;
  if (admitted) *admitted = it->second->t_admit;
  if (finished) *finished = it->second->t_finish;
}

std::string server::stats() {
  std::lock_guard<std::mutex> lk(impl_->mu);
  int done = 0, running = 0;
  for (const auto& kv : impl_->reqs) {
    if (kv.second->done) ++done;
    else if (kv.second->pool >= 0) ++running;
  }
  std::ostringstream os;
  os << "{\"pools\": " << impl_->pools.size() << ", \"device_bytes\": " << impl_->used_bytes
     << ", \"budget\": " << (long long)impl_->budget << ", \"done\": " << done << ", \"running\": " << running
     << ", \"queued\": " << impl_->queue.size() << ", \"error\": \"" << impl_->fatal << "\"}";
  return os.str();
}
