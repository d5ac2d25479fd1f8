// C-ABI entry points (declared in include/cupss_gb300.h).
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/cupss.h"
#include "../../include/cupss/ensemble.h"
#include "../../include/cupss/server.h"
#include "../../include/cupss_gb300.h"
#include "engine.h"
#include "engine_multi.h"
#include "host_common.h"
#include "jit.h"
#include "tune_cache.h"

struct cupssgb_solver {
  cupssgb::Solver* s;
};

struct cupssgb_evolver {
  evolver* e;
};

struct cupssgb_ensemble {
  ensemble* e;
};

struct cupssgb_server {
  server* s;
};

struct cupssgb_multi {
  cupssgb::MultiStep* m;
};

namespace {
thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

template <class F>
int guard(F&& fn) {
  try {
    g_last_error.clear();
    return fn();
  } catch (const cupssgb::Error& e) {
    return fail(e.code, e.what());
  } catch (const cupssgb_host::ParseError& e) {
    return fail(CUPSSGB_ERR_PARSE, e.what());
  } catch (const cupssgb_host::CapiError& e) {
    return fail(e.code, e.what());
  } catch (const std::exception& e) {
    return fail(CUPSSGB_ERR_INVALID, e.what());
  } catch (...) {
    return fail(CUPSSGB_ERR_INVALID, "unknown error");
  }
}

// Writes at most buflen-1 chars of r plus a NUL; returns the full length.
int copy_out(const std::string& r, char* buf, int buflen) {
  if (buf && buflen > 0) {
    const size_t n = std::min((size_t)buflen - 1, r.size());
    std::memcpy(buf, r.data(), n);
    buf[n] = 0;
  }
  return (int)r.size();
}

std::vector<cupssgb::HostPres> to_host(const cupssgb_pres* p, int n) {
  std::vector<cupssgb::HostPres> out;
  for (int i = 0; i < n; ++i) {
    cupssgb::HostPres h;
    h.pre = p[i].preFactor;
    h.q2n = p[i].q2n;
    h.iqx = p[i].iqx;
    h.iqy = p[i].iqy;
    h.iqz = p[i].iqz;
    h.invq = p[i].invq;
    out.push_back(h);
  }
  return out;
}

#define NEED(ptr)                                                     \
  if ((ptr) == nullptr) return fail(CUPSSGB_ERR_INVALID, #ptr " is NULL")

void json_pres(std::ostringstream& os, const pres& p) {
  char buf[160];
  std::snprintf(buf, sizeof(buf), "[%.9g, %d, %d, %d, %d, %d]", (double)p.preFactor, p.q2n, p.iqx, p.iqy,
                p.iqz, p.invq);
  os << buf;
}

field* find_field(evolver* e, const char* name) {
  if (!name) return nullptr;
  auto it = e->fieldsMap.find(name);
  return it == e->fieldsMap.end() ? nullptr : it->second;
}
}  // namespace

namespace cupssgb {
// Lets other translation units report through cupssgb_last_error().
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace cupssgb

extern "C" {

const char* cupssgb_last_error(void) { return g_last_error.c_str(); }
int cupssgb_version(void) { return 100; }

// ---------------- solver level ----------------
int cupssgb_solver_create(int sx, int sy, int sz, float dx, float dy, float dz, float dt,
                          cupssgb_solver** out) {
  NEED(out);
  return guard([&] {
    *out = new cupssgb_solver{new cupssgb::Solver(sx, sy, sz, dx, dy, dz, dt)};
    return 0;
  });
}

int cupssgb_solver_destroy(cupssgb_solver* s) {
  if (!s) return 0;
  return guard([&] {
    delete s->s;
    delete s;
    return 0;
  });
}

int cupssgb_solver_add_field(cupssgb_solver* s, int dynamic) {
  NEED(s);
  return guard([&] { return s->s->add_field(dynamic != 0); });
}

int cupssgb_solver_set_implicit(cupssgb_solver* s, int field, const cupssgb_pres* pres, int n) {
  NEED(s);
  if (n > 0 && !pres) return fail(CUPSSGB_ERR_INVALID, "pres is NULL");
  return guard([&] {
    s->s->set_implicit(field, to_host(pres, n));
    return 0;
  });
}

int cupssgb_solver_update_implicit(cupssgb_solver* s, int field, const cupssgb_pres* pres, int n) {
  return cupssgb_solver_set_implicit(s, field, pres, n);
}

int cupssgb_solver_add_term(cupssgb_solver* s, int field, const int* product, int n_product,
                            const cupssgb_pres* pres, int n_pres) {
  NEED(s);
  if ((n_product > 0 && !product) || !pres || n_pres <= 0 || n_product < 0)
    return fail(CUPSSGB_ERR_INVALID, "bad term arguments");
  return guard([&] {
    return s->s->add_term(field, std::vector<int>(product, product + n_product), to_host(pres, n_pres));
  });
}

int cupssgb_solver_set_term_pres(cupssgb_solver* s, int field, int term, const cupssgb_pres* pres, int n) {
  NEED(s);
  NEED(pres);
  return guard([&] {
    s->s->set_term_pres(field, term, to_host(pres, n));
    return 0;
  });
}

int cupssgb_solver_set_noise(cupssgb_solver* s, int field, const cupssgb_pres* amp) {
  NEED(s);
  return guard([&] {
    cupssgb::HostPres h;
    if (amp) h = to_host(amp, 1)[0];
    s->s->set_noise(field, amp != nullptr, h);
    return 0;
  });
}

int cupssgb_solver_set_seed(cupssgb_solver* s, unsigned long long seed) {
  NEED(s);
  s->s->set_seed(seed);
  return 0;
}

int cupssgb_solver_prepare(cupssgb_solver* s) {
  NEED(s);
  return guard([&] {
    s->s->prepare();
    return 0;
  });
}

int cupssgb_solver_set_real(cupssgb_solver* s, int field, const float* host_real) {
  NEED(s);
  NEED(host_real);
  return guard([&] {
    // a pageable source is copied before this returns (and errors surface here); a
    // page-locked one stays in flight on the input stream
    if (!s->s->set_real(field, host_real, false)) s->s->synchronize();
    return 0;
  });
}

int cupssgb_solver_set_real_device(cupssgb_solver* s, int field, const float* dev_real) {
  NEED(s);
  NEED(dev_real);
  return guard([&] {
    s->s->set_real(field, dev_real, true);
    return 0;
  });
}

int cupssgb_solver_advance(cupssgb_solver* s, int nsteps) {
  NEED(s);
  if (nsteps < 0) return fail(CUPSSGB_ERR_INVALID, "nsteps < 0");
  return guard([&] {
    s->s->advance(nsteps);
    return 0;
  });
}

int cupssgb_solver_get_real(cupssgb_solver* s, int field, float* host_real) {
  NEED(s);
  NEED(host_real);
  return guard([&] {
    s->s->get_real(field, host_real, false);
    return 0;
  });
}

int cupssgb_solver_get_real_device(cupssgb_solver* s, int field, float* dev_real) {
  NEED(s);
  NEED(dev_real);
  return guard([&] {
    s->s->get_real(field, dev_real, true);
    return 0;
  });
}

int cupssgb_solver_get_fourier(cupssgb_solver* s, int field, float* host_complex) {
  NEED(s);
  NEED(host_complex);
  return guard([&] {
    s->s->get_fourier(field, reinterpret_cast<float2*>(host_complex), false);
    return 0;
  });
}

int cupssgb_solver_get_fourier_device(cupssgb_solver* s, int field, float* dev_complex) {
  NEED(s);
  NEED(dev_complex);
  return guard([&] {
    s->s->get_fourier(field, reinterpret_cast<float2*>(dev_complex), true);
    return 0;
  });
}

int cupssgb_solver_advance_phase(cupssgb_solver* s, int phase) {
  NEED(s);
  return guard([&] {
    s->s->advance_phase(phase);
    return 0;
  });
}

int cupssgb_solver_get_real_pairs_device(cupssgb_solver* s, int field, float* dev_pairs) {
  NEED(s);
  NEED(dev_pairs);
  return guard([&] {
    s->s->get_real_pairs_device(field, reinterpret_cast<float2*>(dev_pairs));
    return 0;
  });
}

int cupssgb_solver_get_dealiased_pairs_device(cupssgb_solver* s, int field, float* dev_pairs) {
  NEED(s);
  NEED(dev_pairs);
  return guard([&] {
    s->s->get_dealiased_pairs_device(field, reinterpret_cast<float2*>(dev_pairs));
    return 0;
  });
}

int cupssgb_solver_set_fourier_device(cupssgb_solver* s, int field, const float* dev_complex) {
  NEED(s);
  NEED(dev_complex);
  return guard([&] {
    s->s->set_fourier_device(field, reinterpret_cast<const float2*>(dev_complex));
    return 0;
  });
}

int cupssgb_solver_set_real_pairs_device(cupssgb_solver* s, int field, const float* dev_pairs,
                                         const float* dev_dealiased_pairs) {
  NEED(s);
  NEED(dev_pairs);
  return guard([&] {
    s->s->set_real_pairs_device(field, reinterpret_cast<const float2*>(dev_pairs),
                                reinterpret_cast<const float2*>(dev_dealiased_pairs));
    return 0;
  });
}

int cupssgb_solver_synchronize(cupssgb_solver* s) {
  NEED(s);
  return guard([&] {
    s->s->synchronize();
    return 0;
  });
}

int cupssgb_solver_time_advance(cupssgb_solver* s, int nsteps, double* ms) {
  NEED(s);
  NEED(ms);
  return guard([&] {
    *ms = s->s->time_advance(nsteps);
    return 0;
  });
}

int cupssgb_solver_set_kernel_timing(cupssgb_solver* s, int on) {
  NEED(s);
  return guard([&] {
    s->s->set_kernel_timing(on != 0);
    return 0;
  });
}

int cupssgb_solver_kernel_report(cupssgb_solver* s, char* buf, int buflen) {
  NEED(s);
  std::string r;
  int rc = guard([&] {
    r = s->s->kernel_report();
    return 0;
  });
  if (rc != 0) return rc;
  if (buf && buflen > 0) {
    const size_t n = std::min((size_t)buflen - 1, r.size());
    std::memcpy(buf, r.data(), n);
    buf[n] = 0;
  }
  return (int)r.size();
}

int cupssgb_solver_generated_source(cupssgb_solver* s, int index, char* buf, int buflen) {
  NEED(s);
  std::string src;
  int rc = guard([&] {
    std::vector<std::string> v = s->s->generated_sources();
    if (index < 0 || index >= (int)v.size()) return fail(CUPSSGB_ERR_INVALID, "no such generated program");
    src = v[index];
    return 0;
  });
  if (rc != 0) return rc;
  if (buf && buflen > 0) {
    const size_t n = std::min((size_t)buflen - 1, src.size());
    std::memcpy(buf, src.data(), n);
    buf[n] = 0;
  }
  return (int)src.size();
}

int cupssgb_solver_set_generated_programs(cupssgb_solver* s, int on) {
  NEED(s);
  s->s->set_use_jit(on != 0);
  return 0;
}

int cupssgb_jit_check(const char* source, char* log, int loglen) {
  NEED(source);
  std::string msg;
  int rc = guard([&] {
    size_t bytes = 0;
    msg = cupssgb::jit_compile_only(source, &bytes);
    return msg.empty() ? (int)bytes : fail(CUPSSGB_ERR_CUDA, "NVRTC compilation failed");
  });
  if (log && loglen > 0) {
    const size_t n = std::min((size_t)loglen - 1, msg.size());
    std::memcpy(log, msg.data(), n);
    log[n] = 0;
  }
  return rc;
}

int cupssgb_host_alloc(long long bytes, void** out) {
  NEED(out);
  cudaError_t e = cudaMallocHost(out, (size_t)bytes);
  return e == cudaSuccess ? 0 : fail(CUPSSGB_ERR_CUDA, cudaGetErrorString(e));
}

int cupssgb_host_free(void* p) {
  cudaError_t e = cudaFreeHost(p);
  return e == cudaSuccess ? 0 : fail(CUPSSGB_ERR_CUDA, cudaGetErrorString(e));
}

int cupssgb_solver_snapshot_real(cupssgb_solver* s, int field, float* host_real, void* done_event) {
  NEED(s);
  return guard([&] {
    s->s->snapshot_real(field, host_real, (cudaEvent_t)done_event);
    return 0;
  });
}

int cupssgb_tune_cache_path(char* buf, int buflen) {
  return copy_out(cupssgb::tune_cache_path(), buf, buflen);
}

int cupssgb_tune_cache_lookup(const char* key, char* value, int buflen) {
  NEED(key);
  std::string v;
  if (!cupssgb::tune_cache_lookup(key, &v)) return fail(CUPSSGB_ERR_INVALID, std::string("no entry for ") + key);
  return copy_out(v, value, buflen);
}

int cupssgb_tune_cache_store(const char* key, const char* value) {
  NEED(key);
  NEED(value);
  if (!cupssgb::tune_cache_store(key, value)) return fail(CUPSSGB_ERR_INVALID, "tune cache not written");
  return 0;
}

namespace {
std::vector<cupssgb::Solver*> solvers_of(cupssgb_solver* const* solvers, int n) {
  if (!solvers || n < 1) throw cupssgb::Error(CUPSSGB_ERR_INVALID, "no solvers");
  std::vector<cupssgb::Solver*> v;
  for (int i = 0; i < n; ++i) {
    if (!solvers[i]) throw cupssgb::Error(CUPSSGB_ERR_INVALID, "null solver");
    v.push_back(solvers[i]->s);
  }
  return v;
}
}  // namespace

int cupssgb_multi_check(cupssgb_solver* const* solvers, int n, char* buf, int buflen) {
  return guard([&] {
    const std::string why = cupssgb::MultiStep::unsupported(solvers_of(solvers, n));
    copy_out(why, buf, buflen);
    return why.empty() ? 0 : fail(CUPSSGB_ERR_UNSUPPORTED, why);
  });
}

int cupssgb_multi_create(cupssgb_solver* const* solvers, int n, cupssgb_multi** out) {
  NEED(out);
  return guard([&] {
    *out = new cupssgb_multi{new cupssgb::MultiStep(solvers_of(solvers, n))};
    return 0;
  });
}

int cupssgb_multi_destroy(cupssgb_multi* m) {
  if (!m) return 0;
  return guard([&] {
    delete m->m;
    delete m;
    return 0;
  });
}

int cupssgb_multi_advance(cupssgb_multi* m, int nsteps) {
  NEED(m);
  return guard([&] {
    m->m->advance(nsteps);
    return 0;
  });
}

long long cupssgb_multi_launch_count(const cupssgb_multi* m) { return m ? m->m->launches() : -1; }

int cupssgb_multi_describe(const cupssgb_multi* m, char* buf, int buflen) {
  NEED(m);
  return copy_out(m->m->describe(), buf, buflen);
}

int cupssgb_solver_set_stream_priority(cupssgb_solver* s, int level) {
  NEED(s);
  return guard([&] {
    s->s->set_stream_priority(level);
    return 0;
  });
}

int cupssgb_multi_choose(cupssgb_multi* m) {
  NEED(m);
  return guard([&] {
    m->m->choose();
    return m->m->fused() ? 1 : 0;
  });
}

int cupssgb_multi_generated_source(cupssgb_solver* const* solvers, int n, int phase, char* buf, int buflen) {
  std::string src;
  const int rc = guard([&] {
    src = cupssgb::MultiStep::generated_source(solvers_of(solvers, n), phase);
    return 0;
  });
  if (rc != 0) return rc;
  return copy_out(src, buf, buflen);
}

int cupssgb_set_device(int device) {
  cudaError_t e = cudaSetDevice(device);
  return e == cudaSuccess ? 0 : fail(CUPSSGB_ERR_CUDA, cudaGetErrorString(e));
}

int cupssgb_device_info(char* buf, int buflen) {
  int n = 0, drv = 0, rt = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) {
    cudaGetLastError();
    n = 0;
  } else if (e != cudaSuccess) {
    return fail(CUPSSGB_ERR_CUDA, std::string("cudaGetDeviceCount: ") + cudaGetErrorString(e));
  }
  std::ostringstream os;
  for (int i = 0; i < n; ++i) {
    cudaDeviceProp pr;
    e = cudaGetDeviceProperties(&pr, i);
    if (e != cudaSuccess) return fail(CUPSSGB_ERR_CUDA, std::string("cudaGetDeviceProperties: ") + cudaGetErrorString(e));
    os << i << ": " << pr.name << ", " << pr.multiProcessorCount << " SMs, sm_" << pr.major << pr.minor << ", "
       << (pr.totalGlobalMem >> 20) << " MiB\n";
  }
  cudaDriverGetVersion(&drv);
  cudaRuntimeGetVersion(&rt);
  os << "driver " << drv / 1000 << "." << (drv % 1000) / 10 << ", runtime " << rt / 1000 << "." << (rt % 1000) / 10
     << "\n";
  copy_out(os.str(), buf, buflen);
  return n;
}

long long cupssgb_solver_step_count(const cupssgb_solver* s) { return s ? s->s->step_count() : -1; }
long long cupssgb_solver_launch_count(const cupssgb_solver* s) { return s ? s->s->launches() : -1; }
long long cupssgb_solver_device_bytes(const cupssgb_solver* s) {
  return s ? (long long)s->s->device_bytes() : -1;
}
void* cupssgb_solver_stream(const cupssgb_solver* s) { return s ? (void*)s->s->stream() : nullptr; }

// ---------------- evolver level ----------------
int cupssgb_evolver_create(int with_cuda, int sx, int sy, int sz, float dx, float dy, float dz, float dt,
                           int write_every, cupssgb_evolver** out) {
  NEED(out);
  if (sx < 1 || sy < 1 || sz < 1 || write_every < 1) return fail(CUPSSGB_ERR_INVALID, "bad sizes");
  return guard([&] {
    evolver* e;
    if (sy == 1 && sz == 1) e = new evolver(with_cuda != 0, sx, dx, dt, write_every);
    else if (sz == 1) e = new evolver(with_cuda != 0, sx, sy, dx, dy, dt, write_every);
    else e = new evolver(with_cuda != 0, sx, sy, sz, dx, dy, dz, dt, write_every);
    e->setThrowOnError(true);
    *out = new cupssgb_evolver{e};
    return 0;
  });
}

int cupssgb_evolver_destroy(cupssgb_evolver* e) {
  if (!e) return 0;
  return guard([&] {
    delete e->e;
    delete e;
    return 0;
  });
}

int cupssgb_evolver_create_field(cupssgb_evolver* e, const char* name, int dynamic) {
  NEED(e);
  NEED(name);
  return guard([&] {
    int r = e->e->createField(name, dynamic != 0);
    return r == 0 ? 0 : fail(CUPSSGB_ERR_INVALID, std::string("field exists: ") + name);
  });
}

int cupssgb_evolver_add_parameter(cupssgb_evolver* e, const char* name, float value) {
  NEED(e);
  NEED(name);
  return guard([&] {
    int r = e->e->_parser->insert_parameter(name, value);
    return r == 0 ? 0 : fail(CUPSSGB_ERR_INVALID, std::string("duplicate parameter ") + name);
  });
}

int cupssgb_evolver_add_equation(cupssgb_evolver* e, const char* equation) {
  NEED(e);
  NEED(equation);
  return guard([&] { return e->e->addEquation(equation); });
}

int cupssgb_evolver_add_noise(cupssgb_evolver* e, const char* field_name, const char* amplitude) {
  NEED(e);
  NEED(field_name);
  NEED(amplitude);
  return guard([&] {
    int r = e->e->addNoise(field_name, amplitude);
    return r == 0 ? 0 : fail(CUPSSGB_ERR_INVALID, std::string("no field ") + field_name);
  });
}

int cupssgb_evolver_update_parameter(cupssgb_evolver* e, const char* name, float value) {
  NEED(e);
  NEED(name);
  return guard([&] { return e->e->updateParameter(name, value); });
}

int cupssgb_evolver_set_output_field(cupssgb_evolver* e, const char* name, int output) {
  NEED(e);
  NEED(name);
  return guard([&] {
    if (!find_field(e->e, name)) return fail(CUPSSGB_ERR_INVALID, std::string("no field ") + name);
    e->e->setOutputField(name, output);
    return 0;
  });
}

int cupssgb_evolver_set_seed(cupssgb_evolver* e, unsigned long long seed) {
  NEED(e);
  e->e->setNoiseSeed(seed);
  return 0;
}

int cupssgb_evolver_set_real(cupssgb_evolver* e, const char* name, const float* host_real) {
  NEED(e);
  NEED(host_real);
  return guard([&] {
    field* f = find_field(e->e, name);
    if (!f) return fail(CUPSSGB_ERR_INVALID, std::string("no field ") + (name ? name : ""));
    const size_t n = (size_t)e->e->getSystemSizeX() * e->e->getSystemSizeY() * e->e->getSystemSizeZ();
    for (size_t i = 0; i < n; ++i) f->real_array[i].x = host_real[i];
    return 0;
  });
}

int cupssgb_evolver_prepare(cupssgb_evolver* e) {
  NEED(e);
  return guard([&] {
    e->e->prepareProblem();
    return 0;
  });
}

int cupssgb_evolver_advance(cupssgb_evolver* e, int nsteps) {
  NEED(e);
  if (nsteps < 0) return fail(CUPSSGB_ERR_INVALID, "nsteps < 0");
  return guard([&] { return e->e->advanceTimeSteps(nsteps); });
}

int cupssgb_evolver_write_out(cupssgb_evolver* e) {
  NEED(e);
  return guard([&] {
    e->e->writeOut();
    return 0;
  });
}

int cupssgb_evolver_flush_output(cupssgb_evolver* e) {
  NEED(e);
  return guard([&] {
    e->e->flushOutput();
    return 0;
  });
}

int cupssgb_evolver_create_from_file(cupssgb_evolver* e, const char* path) {
  NEED(e);
  NEED(path);
  return guard([&] {
    const int r = e->e->createFromFile(path);
    return r == 0 ? 0 : fail(CUPSSGB_ERR_PARSE, std::string("cannot read system file ") + path);
  });
}

#define CUPSSGB_INIT_CALL(call)                                                               \
  NEED(e);                                                                                    \
  NEED(name);                                                                                 \
  return guard([&] {                                                                          \
    if (!find_field(e->e, name)) return fail(CUPSSGB_ERR_INVALID, std::string("no field ") + name); \
    e->e->call;                                                                               \
    return 0;                                                                                 \
  })

int cupssgb_evolver_initialize_uniform(cupssgb_evolver* e, const char* name, float value) {
  CUPSSGB_INIT_CALL(initializeUniform(name, value));
}
int cupssgb_evolver_initialize_uniform_noise(cupssgb_evolver* e, const char* name, float amplitude) {
  CUPSSGB_INIT_CALL(initializeUniformNoise(name, amplitude));
}
int cupssgb_evolver_initialize_normal_noise(cupssgb_evolver* e, const char* name, float mean, float sigma) {
  CUPSSGB_INIT_CALL(initializeNormalNoise(name, mean, sigma));
}
int cupssgb_evolver_initialize_half_system(cupssgb_evolver* e, const char* name, float value1, float value2,
                                           float interface_width, int direction) {
  CUPSSGB_INIT_CALL(initializeHalfSystem(name, value1, value2, interface_width, direction));
}
int cupssgb_evolver_initialize_droplet(cupssgb_evolver* e, const char* name, float value_out, float value_in,
                                       float radius, float interface_width, int center_x, int center_y,
                                       int center_z) {
  CUPSSGB_INIT_CALL(initializeDroplet(name, value_out, value_in, radius, interface_width, center_x, center_y, center_z));
}
int cupssgb_evolver_add_droplet(cupssgb_evolver* e, const char* name, float value, float radius,
                                float interface_width, int center_x, int center_y, int center_z) {
  CUPSSGB_INIT_CALL(addDroplet(name, value, radius, interface_width, center_x, center_y, center_z));
}
int cupssgb_evolver_initialize_from_file(cupssgb_evolver* e, const char* name, const char* path, int skiprows,
                                         char delimiter) {
  NEED(path);
  CUPSSGB_INIT_CALL(initializeFromFile(name, path, skiprows, delimiter));
}
#undef CUPSSGB_INIT_CALL

int cupssgb_evolver_get_host_real(cupssgb_evolver* e, const char* name, float* host_real) {
  NEED(e);
  NEED(host_real);
  return guard([&] {
    field* f = find_field(e->e, name);
    if (!f) return fail(CUPSSGB_ERR_INVALID, std::string("no field ") + (name ? name : ""));
    const size_t n = (size_t)e->e->getSystemSizeX() * e->e->getSystemSizeY() * e->e->getSystemSizeZ();
    for (size_t i = 0; i < n; ++i) host_real[i] = f->real_array[i].x;
    return 0;
  });
}

int cupssgb_write_field_csv(const char* path, const char* name, const float* values, int sx, int sy, int sz,
                            int precision) {
  NEED(path);
  NEED(name);
  NEED(values);
  if (sx < 1 || sy < 1 || sz < 1 || precision < 0) return fail(CUPSSGB_ERR_INVALID, "bad sizes");
  return guard([&] {
    const int dim = (sy == 1 && sz == 1) ? 1 : (sz == 1 ? 2 : 3);
    const std::string err = cupssgb_host::write_field_csv(path, name, values, sx, sy, sz, dim, precision);
    return err.empty() ? 0 : fail(CUPSSGB_ERR_INVALID, err);
  });
}

int cupssgb_evolver_get_real(cupssgb_evolver* e, const char* name, float* host_real) {
  NEED(e);
  NEED(host_real);
  return guard([&] {
    const int idx = e->e->existsField(name ? name : "");
    if (idx < 0) return fail(CUPSSGB_ERR_INVALID, std::string("no field ") + (name ? name : ""));
    cupssgb_solver* s = e->e->solverHandle();
    if (!s) return fail(CUPSSGB_ERR_STATE, "prepareProblem has not been called");
    return cupssgb_solver_get_real(s, idx, host_real);
  });
}

int cupssgb_evolver_get_fourier(cupssgb_evolver* e, const char* name, float* host_complex) {
  NEED(e);
  NEED(host_complex);
  return guard([&] {
    const int idx = e->e->existsField(name ? name : "");
    if (idx < 0) return fail(CUPSSGB_ERR_INVALID, std::string("no field ") + (name ? name : ""));
    cupssgb_solver* s = e->e->solverHandle();
    if (!s) return fail(CUPSSGB_ERR_STATE, "prepareProblem has not been called");
    return cupssgb_solver_get_fourier(s, idx, host_complex);
  });
}

float cupssgb_evolver_get_parameter(cupssgb_evolver* e, const char* name) {
  if (!e || !name) return 0.f;
  float v = 0.f;
  guard([&] {
    v = e->e->getParameter(name);
    return 0;
  });
  return v;
}

int cupssgb_evolver_current_step(const cupssgb_evolver* e) {
  return e ? const_cast<evolver*>(e->e)->getCurrentTimestep() : -1;
}

int cupssgb_evolver_describe(const cupssgb_evolver* ce, char* buf, int buflen) {
  NEED(ce);
  evolver* e = ce->e;
  std::ostringstream os;
  os << "[";
  for (size_t i = 0; i < e->fields.size(); ++i) {
    field* f = e->fields[i];
    if (i) os << ", ";
    os << "{\"name\": \"" << f->name << "\", \"dynamic\": " << (f->dynamic ? "true" : "false")
       << ", \"implicit\": [";
    for (size_t j = 0; j < f->implicit.size(); ++j) {
      if (j) os << ", ";
      json_pres(os, f->implicit[j]);
    }
    os << "], \"terms\": [";
    for (size_t t = 0; t < f->terms.size(); ++t) {
      if (t) os << ", ";
      os << "{\"product\": [";
      for (size_t k = 0; k < f->terms[t]->product.size(); ++k) {
        if (k) os << ", ";
        os << "\"" << f->terms[t]->product[k]->name << "\"";
      }
      os << "], \"pres\": [";
      for (size_t k = 0; k < f->terms[t]->prefactors_h.size(); ++k) {
        if (k) os << ", ";
        json_pres(os, f->terms[t]->prefactors_h[k]);
      }
      os << "]}";
    }
    os << "], \"noisy\": " << (f->isNoisy ? "true" : "false") << ", \"noise\": ";
    json_pres(os, f->noise_amplitude);
    os << "}";
  }
  os << "]";
  const std::string s = os.str();
  if (buf && buflen > 0) {
    const size_t n = std::min((size_t)buflen - 1, s.size());
    std::memcpy(buf, s.data(), n);
    buf[n] = 0;
  }
  return (int)s.size();
}

cupssgb_solver* cupssgb_evolver_solver(cupssgb_evolver* e) { return e ? e->e->solverHandle() : nullptr; }

int cupssgb_evolver_set_callback(cupssgb_evolver* e, const char* name, int fourier, cupssgb_callback fn) {
  NEED(e);
  return guard([&] {
    field* f = find_field(e->e, name);
    if (!f) return fail(CUPSSGB_ERR_INVALID, std::string("no field ") + (name ? name : ""));
    auto cb = reinterpret_cast<void (*)(evolver*, float2*, int, int, int)>(fn);
    if (fourier) {
      f->hasCBFourier = fn != nullptr;
      f->callbackFourier = cb;
    } else {
      f->hasCB = fn != nullptr;
      f->callback = cb;
    }
    return 0;
  });
}

/* ---------------- batches ---------------- */

int cupssgb_solver_set_members(cupssgb_solver* s, int n) {
  NEED(s);
  return guard([&] {
    s->s->set_members(n);
    return 0;
  });
}

int cupssgb_solver_members(const cupssgb_solver* s) { return s ? s->s->members() : CUPSSGB_ERR_INVALID; }

int cupssgb_solver_set_member_term_pres(cupssgb_solver* s, int member, int field, int term, const cupssgb_pres* pres,
                                        int n) {
  NEED(s);
  if (n > 0) NEED(pres);
  return guard([&] {
    s->s->set_member_term_pres(member, field, term, to_host(pres, n));
    return 0;
  });
}

int cupssgb_solver_set_member_implicit(cupssgb_solver* s, int member, int field, const cupssgb_pres* pres, int n) {
  NEED(s);
  if (n > 0) NEED(pres);
  return guard([&] {
    s->s->set_member_implicit(member, field, to_host(pres, n));
    return 0;
  });
}

int cupssgb_solver_set_member_noise(cupssgb_solver* s, int member, int field, const cupssgb_pres* amp) {
  NEED(s);
  NEED(amp);
  return guard([&] {
    s->s->set_member_noise(member, field, to_host(amp, 1)[0]);
    return 0;
  });
}

int cupssgb_solver_set_member_seed(cupssgb_solver* s, int member, unsigned long long seed) {
  NEED(s);
  return guard([&] {
    s->s->set_member_seed(member, seed);
    return 0;
  });
}

int cupssgb_solver_set_member_active(cupssgb_solver* s, int member, int active) {
  NEED(s);
  return guard([&] {
    s->s->set_member_active(member, active != 0);
    return 0;
  });
}

int cupssgb_solver_reset_member(cupssgb_solver* s, int member) {
  NEED(s);
  return guard([&] {
    s->s->reset_member(member);
    return 0;
  });
}

long long cupssgb_solver_member_step(cupssgb_solver* s, int member) {
  if (!s) return fail(CUPSSGB_ERR_INVALID, "null handle");
  long long out = 0;
  const int rc = guard([&] {
    out = s->s->member_step(member);
    return 0;
  });
  return rc != 0 ? rc : out;
}

int cupssgb_solver_set_real_member(cupssgb_solver* s, int field, int member, const float* host_real) {
  NEED(s);
  NEED(host_real);
  return guard([&] {
    if (!s->s->set_real(field, host_real, false, member)) s->s->synchronize();
    return 0;
  });
}

int cupssgb_solver_set_real_member_device(cupssgb_solver* s, int field, int member, const float* dev_real) {
  NEED(s);
  NEED(dev_real);
  return guard([&] {
    s->s->set_real(field, dev_real, true, member);
    return 0;
  });
}

int cupssgb_solver_get_real_member(cupssgb_solver* s, int field, int member, float* host_real) {
  NEED(s);
  NEED(host_real);
  return guard([&] {
    s->s->get_real(field, host_real, false, member);
    return 0;
  });
}

int cupssgb_solver_get_real_member_device(cupssgb_solver* s, int field, int member, float* dev_real) {
  NEED(s);
  NEED(dev_real);
  return guard([&] {
    s->s->get_real(field, dev_real, true, member);
    return 0;
  });
}

int cupssgb_solver_tune_report(cupssgb_solver* s, char* buf, int buflen) {
  NEED(s);
  std::string r;
  const int rc = guard([&] {
    r = s->s->tune_report();
    return 0;
  });
  if (rc != 0) return rc;
  return copy_out(r, buf, buflen);
}

long long cupssgb_solver_estimate_bytes(cupssgb_solver* s, int members) {
  if (!s) return fail(CUPSSGB_ERR_INVALID, "null handle");
  long long out = 0;
  const int rc = guard([&] {
    out = (long long)s->s->estimate_bytes(members);
    return 0;
  });
  return rc != 0 ? rc : out;
}

int cupssgb_solver_query(cupssgb_solver* s) {
  NEED(s);
  return guard([&] { return s->s->idle() ? 1 : 0; });
}

/* ---------------- ensembles ---------------- */

int cupssgb_ensemble_create(cupssgb_ensemble** out) {
  NEED(out);
  return guard([&] {
    *out = new cupssgb_ensemble{new ensemble()};
    return 0;
  });
}

int cupssgb_ensemble_destroy(cupssgb_ensemble* e) {
  if (!e) return 0;
  return guard([&] {
    delete e->e;
    delete e;
    return 0;
  });
}

int cupssgb_ensemble_create_field(cupssgb_ensemble* e, const char* name, int dynamic) {
  NEED(e);
  NEED(name);
  return guard([&] { return e->e->createField(name, dynamic != 0); });
}

int cupssgb_ensemble_add_parameter(cupssgb_ensemble* e, const char* name, float value) {
  NEED(e);
  NEED(name);
  return guard([&] { return e->e->addParameter(name, value); });
}

int cupssgb_ensemble_add_equation(cupssgb_ensemble* e, const char* equation) {
  NEED(e);
  NEED(equation);
  return guard([&] { return e->e->addEquation(equation); });
}

int cupssgb_ensemble_add_noise(cupssgb_ensemble* e, const char* field, const char* amplitude) {
  NEED(e);
  NEED(field);
  NEED(amplitude);
  return guard([&] { return e->e->addNoise(field, amplitude); });
}

int cupssgb_ensemble_add_member(cupssgb_ensemble* e, int sx, int sy, int sz, float dx, float dy, float dz, float dt,
                                unsigned long long seed) {
  NEED(e);
  return guard([&] { return e->e->addMember(sx, sy, sz, dx, dy, dz, dt, seed); });
}

int cupssgb_ensemble_set_member_parameter(cupssgb_ensemble* e, int member, const char* name, float value) {
  NEED(e);
  NEED(name);
  return guard([&] { return e->e->setMemberParameter(member, name, value); });
}

int cupssgb_ensemble_prepare(cupssgb_ensemble* e) {
  NEED(e);
  return guard([&] {
    e->e->prepare();
    return 0;
  });
}

int cupssgb_ensemble_set_real(cupssgb_ensemble* e, int member, const char* field, const float* host_real) {
  NEED(e);
  NEED(field);
  NEED(host_real);
  return guard([&] { return e->e->setReal(member, field, host_real); });
}

int cupssgb_ensemble_advance(cupssgb_ensemble* e, int nsteps) {
  NEED(e);
  return guard([&] { return e->e->advance(nsteps); });
}

int cupssgb_ensemble_get_real(cupssgb_ensemble* e, int member, const char* field, float* host_real) {
  NEED(e);
  NEED(field);
  NEED(host_real);
  return guard([&] { return e->e->getReal(member, field, host_real); });
}

int cupssgb_ensemble_groups(const cupssgb_ensemble* e) { return e ? e->e->groups() : CUPSSGB_ERR_INVALID; }

long long cupssgb_ensemble_device_bytes(const cupssgb_ensemble* e) { return e ? e->e->deviceBytes() : 0; }

long long cupssgb_ensemble_launch_count(const cupssgb_ensemble* e) { return e ? e->e->launches() : 0; }

int cupssgb_ensemble_describe(const cupssgb_ensemble* e, char* buf, int buflen) {
  NEED(e);
  std::string r;
  const int rc = guard([&] {
    r = e->e->describe();
    return 0;
  });
  if (rc != 0) return rc;
  return copy_out(r, buf, buflen);
}

/* ---------------- server ---------------- */

int cupssgb_server_create(double hbm_budget, int max_slots, int max_chunk, cupssgb_server** out) {
  NEED(out);
  return guard([&] {
    *out = new cupssgb_server{new server(hbm_budget, max_slots, max_chunk)};
    return 0;
  });
}

int cupssgb_server_destroy(cupssgb_server* s) {
  if (!s) return 0;
  return guard([&] {
    delete s->s;
    delete s;
    return 0;
  });
}

int cupssgb_server_add_system(cupssgb_server* s) {
  NEED(s);
  return guard([&] { return s->s->addSystem(); });
}

int cupssgb_server_create_field(cupssgb_server* s, int system, const char* name, int dynamic) {
  NEED(s);
  NEED(name);
  return guard([&] { return s->s->createField(system, name, dynamic != 0); });
}

int cupssgb_server_add_parameter(cupssgb_server* s, int system, const char* name, float value) {
  NEED(s);
  NEED(name);
  return guard([&] { return s->s->addParameter(system, name, value); });
}

int cupssgb_server_add_equation(cupssgb_server* s, int system, const char* equation) {
  NEED(s);
  NEED(equation);
  return guard([&] { return s->s->addEquation(system, equation); });
}

int cupssgb_server_add_noise(cupssgb_server* s, int system, const char* field, const char* amplitude) {
  NEED(s);
  NEED(field);
  NEED(amplitude);
  return guard([&] { return s->s->addNoise(system, field, amplitude); });
}

int cupssgb_server_set_output_field(cupssgb_server* s, int system, const char* field) {
  NEED(s);
  NEED(field);
  return guard([&] { return s->s->setOutputField(system, field); });
}

long long cupssgb_server_submit(cupssgb_server* s, int system, int sx, int sy, int sz, float dx, float dy, float dz,
                                float dt, long long nsteps, unsigned long long seed, int nparams,
                                const char* const* names, const float* values, int ninit,
                                const char* const* fields, const float* const* arrays) {
  if (!s) return fail(CUPSSGB_ERR_INVALID, "null handle");
  if ((nparams > 0 && (!names || !values)) || (ninit > 0 && (!fields || !arrays)))
    return fail(CUPSSGB_ERR_INVALID, "null parameter or field array");
  long long id = 0;
  const int rc = guard([&] {
    std::map<std::string, float> params;
    for (int i = 0; i < nparams; ++i) params[names[i]] = values[i];
    std::map<std::string, const float*> init;
    for (int i = 0; i < ninit; ++i) init[fields[i]] = arrays[i];
    id = s->s->submit(system, sx, sy, sz, dx, dy, dz, dt, nsteps, seed, params, init);
    return 0;
  });
  return rc != 0 ? rc : id;
}

int cupssgb_server_warm(cupssgb_server* s, int system, int sx, int sy, int sz, float dx, float dy, float dz,
                        float dt) {
  NEED(s);
  return guard([&] {
    s->s->warm(system, sx, sy, sz, dx, dy, dz, dt);
    return 0;
  });
}

int cupssgb_server_wait(cupssgb_server* s, long long id, double timeout) {
  NEED(s);
  return guard([&] { return s->s->wait(id, timeout) ? 1 : 0; });
}

int cupssgb_server_result(cupssgb_server* s, long long id, float* host_out) {
  NEED(s);
  NEED(host_out);
  return guard([&] {
    s->s->result(id, host_out);
    return 0;
  });
}

int cupssgb_server_times(cupssgb_server* s, long long id, double* times3) {
  NEED(s);
  NEED(times3);
  return guard([&] {
    s->s->times(id, times3, times3 + 1, times3 + 2);
    return 0;
  });
}

int cupssgb_server_stats(cupssgb_server* s, char* buf, int buflen) {
  NEED(s);
  std::string r;
  const int rc = guard([&] {
    r = s->s->stats();
    return 0;
  });
  if (rc != 0) return rc;
  return copy_out(r, buf, buflen);
}

}  // extern "C"
