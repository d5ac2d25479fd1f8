// evolver: the public C++ API of cuPSS on top of the GB300 engine.
//
// Reference behaviour kept: constructors and launch dims (src/evolver.cpp:13-74),
// prepareProblem (data/ directory, parameter_list.txt.0, upload of the initial
// real fields; :81-126), the advanceTime contract (writeOut every writeEveryNSteps
// before the step; :199-226), createField/createTerm/addNoise/updateParameter
// (:141-196, :326-394) and printInformation (:237-324).  The step itself is
// delegated to the engine through the solver-level C-ABI (include/cupss_gb300.h).
#include <sys/stat.h>

#include <cmath>
#include <cstdlib>
#include <ctime>
#include <iomanip>
#include <iostream>
#include <stdexcept>

#include "../../include/cupss.h"
#include "../../include/cupss_gb300.h"
#include "host_common.h"

using cupssgb_host::ParseError;

namespace {
[[noreturn]] void fatal(const std::string& msg) {
  std::cout << msg << std::endl;
  std::exit(1);
}

std::vector<cupssgb_pres> to_c(const std::vector<pres>& v) {
  std::vector<cupssgb_pres> out;
  out.reserve(v.size());
  for (const pres& p : v) out.push_back({p.preFactor, p.q2n, p.iqx, p.iqy, p.iqz, p.invq});
  return out;
}
}  // namespace

#define CUPSS_GUARD(expr)                                    \
  do {                                                       \
    try {                                                    \
      expr;                                                  \
    } catch (const std::exception& ex) {                     \
      if (throw_errors_) throw;                              \
      fatal(std::string("ERROR: ") + ex.what());             \
    }                                                        \
  } while (0)

void evolver::common_constructor() {
  currentTime = 0.0f;
  currentTimeStep = 0;
  dtsqrt = std::sqrt(dt);
  writeParametersOnUpdate = true;
  writePrecision = 6;
  _parser = new parser(this);
  verbose = false;
  solver_ = nullptr;
  throw_errors_ = false;
  seed_set_ = false;
  seed_ = 0;
  writer_ = nullptr;
  if (sz == 1 && sy == 1) {
    dimension = 1;
    blocks = 1;
    threads_per_block = sx;
  } else if (sz == 1) {
    dimension = 2;
    threads_per_block = dim3(32, 32);
    blocks = dim3((sx + 31) / 32, (sy + 31) / 32);
  } else {
    dimension = 3;
    threads_per_block = dim3(16, 8, 8);
    blocks = dim3((sx + 15) / 16, (sy + 7) / 8, (sz + 7) / 8);
  }
}

evolver::~evolver() {
  if (writer_) {
    // every queued file is written before the device state goes away
    const std::string err = writer_->flush();
    delete writer_;
    writer_ = nullptr;
    if (!err.empty()) {
      std::cout << err << std::endl;
      if (!throw_errors_) std::exit(1);
    }
  }
  for (field* f : fields) delete f;
  delete _parser;
  if (solver_) cupssgb_solver_destroy(solver_);
}

evolver::evolver(bool _with_cuda, int _sx, float _dx, float _dt, int _ses)
    : sx(_sx), sy(1), sz(1), dx(_dx), dy(1.0f), dz(1.0f), writeEveryNSteps(_ses), dt(_dt) {
  std::srand(time(0));
  with_cuda = _with_cuda;
  common_constructor();
}

evolver::evolver(bool _with_cuda, int _sx, int _sy, float _dx, float _dy, float _dt, int _ses)
    : sx(_sx), sy(_sy), sz(1), dx(_dx), dy(_dy), dz(1.0f), writeEveryNSteps(_ses), dt(_dt) {
  std::srand(time(NULL));
  with_cuda = _with_cuda;
  common_constructor();
}

evolver::evolver(bool _with_cuda, int _sx, int _sy, int _sz, float _dx, float _dy, float _dz, float _dt,
                 int _ses)
    : sx(_sx), sy(_sy), sz(_sz), dx(_dx), dy(_dy), dz(_dz), writeEveryNSteps(_ses), dt(_dt) {
  std::srand(time(NULL));
  with_cuda = _with_cuda;
  common_constructor();
}

void evolver::setThrowOnError(bool on) { throw_errors_ = on; }
cupssgb_solver* evolver::solverHandle() { return solver_; }

void evolver::setNoiseSeed(unsigned long long seed) {
  seed_ = seed;
  seed_set_ = true;
  if (solver_) cupssgb_solver_set_seed(solver_, seed);
}

int evolver::createFromFile(const std::string& file) {
  int r = 0;
  CUPSS_GUARD(r = _parser->createFromFile(file));
  return r;
}

bool evolver::has_callbacks() const {
  for (field* f : fields)
    if (f->hasCB || f->hasCBFourier) return true;
  return false;
}

void evolver::build_solver() {
  cupssgb_solver* s = nullptr;
  if (cupssgb_solver_create(sx, sy, sz, dx, dy, dz, dt, &s) != 0)
    throw std::runtime_error(cupssgb_last_error());
  solver_ = s;
  for (field* f : fields)
    if (cupssgb_solver_add_field(s, f->dynamic ? 1 : 0) < 0) throw std::runtime_error(cupssgb_last_error());
  for (size_t i = 0; i < fields.size(); ++i) {
    field* f = fields[i];
    std::vector<cupssgb_pres> imp = to_c(f->implicit);
    if (cupssgb_solver_set_implicit(s, (int)i, imp.data(), (int)imp.size()) != 0)
      throw std::runtime_error(cupssgb_last_error());
    for (term* t : f->terms) {
      std::vector<int> prod;
      for (field* g : t->product) prod.push_back(existsField(g->name));
      std::vector<cupssgb_pres> pv = to_c(t->prefactors_h);
      if (cupssgb_solver_add_term(s, (int)i, prod.data(), (int)prod.size(), pv.data(), (int)pv.size()) < 0)
        throw std::runtime_error(cupssgb_last_error());
    }
    if (f->isNoisy) {
      const pres& a = f->noise_amplitude;
      cupssgb_pres c = {a.preFactor, a.q2n, a.iqx, a.iqy, a.iqz, a.invq};
      cupssgb_solver_set_noise(s, (int)i, &c);
    }
  }
  unsigned long long seed = seed_set_ ? seed_ : (unsigned long long)time(NULL);
  cupssgb_solver_set_seed(s, seed);
  if (cupssgb_solver_prepare(s) != 0) throw std::runtime_error(cupssgb_last_error());
  // dealiasing flags as term::prepareDevice sets them (src/term_init.cpp:117-127)
  for (field* f : fields)
    for (term* t : f->terms)
      if (t->product.size() >= 2)
        for (field* g : t->product) {
          g->needsaliasing = true;
          if (g->aliasing_order < (int)t->product.size()) g->aliasing_order = (int)t->product.size();
        }
}

void evolver::prepareProblem() {
  try {
    if (with_cuda && verbose) check_device();
    struct stat info;
    const std::string path = "data";
    if (stat(path.c_str(), &info) != 0) {
      if (verbose) std::cout << "data directory not found, creating it.\n";
      if (mkdir(path.c_str(), S_IRWXU | S_IRWXG | S_IROTH | S_IXOTH) == -1)
        fatal("Error creating data directory");
    } else if (info.st_mode & S_IFDIR) {
      if (verbose) std::cout << "data directory already found, might rewrite output data.\n";
    } else {
      fatal("Can't create data directory, is there a file called data?");
    }
    _parser->writeParamsToFile("data/parameter_list.txt.0");
    if (!solver_) build_solver();
    if (verbose) std::cout << "Uploading initial states to the device." << std::endl;
    const size_t n = (size_t)sx * sy * sz;
    std::vector<float> tmp(n);
    for (size_t i = 0; i < fields.size(); ++i) {
      for (size_t k = 0; k < n; ++k) tmp[k] = fields[i]->real_array[k].x;
      if (cupssgb_solver_set_real(solver_, (int)i, tmp.data()) != 0)
        throw std::runtime_error(cupssgb_last_error());
      fields[i]->system_p = this;
      fields[i]->isCUDA = with_cuda;
    }
  } catch (const std::exception& ex) {
    if (throw_errors_) throw;
    fatal(std::string("ERROR: ") + ex.what());
  }
}

void evolver::setOutputField(const std::string& name, int output) {
  for (field* f : fields)
    if (f->name == name) {
      f->outputToFile = output != 0;
      return;
    }
  std::cout << "setOutputField EROR: " << name << " not found." << std::endl;
}

int evolver::addParameter(const std::string& name, float value) {
  _parser->insert_parameter(name, value);
  return 0;
}

int evolver::addEquation(const std::string& equation) {
  if (solver_) {
    if (throw_errors_) throw std::runtime_error("addEquation after prepareProblem");
    fatal("ERROR: addEquation after prepareProblem is not supported");
  }
  CUPSS_GUARD(_parser->add_equation(equation));
  return 0;
}

int evolver::existsField(const std::string& name) {
  for (size_t i = 0; i < fields.size(); ++i)
    if (fields[i]->name == name) return (int)i;
  return -1;
}

int evolver::addNoise(const std::string& name, const std::string& equation) {
  if (existsField(name) == -1) {
    std::cout << "Adding noise to non existing field! (" << name << ")" << std::endl;
    return -1;
  }
  pres p;
  CUPSS_GUARD(p = _parser->add_noise(equation));
  fieldsMap[name]->isNoisy = true;
  fieldsMap[name]->noise_amplitude = p;
  if (solver_) {
    cupssgb_pres c = {p.preFactor, p.q2n, p.iqx, p.iqy, p.iqz, p.invq};
    cupssgb_solver_set_noise(solver_, existsField(name), &c);
  }
  return 0;
}

void evolver::addField(field* f) { fields.push_back(f); }

int evolver::createField(std::string name, bool dynamic) {
  for (field* f : fields)
    if (f->name == name) {
      std::cout << "Trying to create field with name that already exists" << std::endl;
      return 1;
    }
  if (solver_) {
    if (throw_errors_) throw std::runtime_error("createField after prepareProblem");
    fatal("ERROR: createField after prepareProblem is not supported");
  }
  field* f = new field(sx, sy, sz, dx, dy, dz);
  f->name = name;
  f->isCUDA = with_cuda;
  f->dynamic = dynamic;
  f->blocks = blocks;
  f->threads_per_block = threads_per_block;
  f->system_p = this;
  fields.push_back(f);
  fieldsMap[name] = f;
  fieldsReal[name] = f->real_array;
  fieldsFourier[name] = f->comp_array;
  return 0;
}

void evolver::sync_host_arrays() {
  for (field* f : fields) f->copyDeviceToHost();
}

namespace {
void cuda_or_die(cudaError_t e, bool throw_errors, const char* what) {
  if (e == cudaSuccess) return;
  const std::string msg = std::string(what) + ": " + cudaGetErrorString(e);
  if (throw_errors) throw std::runtime_error(msg);
  std::cerr << "CUDA Runtime Error" << std::endl << msg << std::endl;
  std::exit(1);
}
}  // namespace

// One time step with user callbacks (src/field.cpp:48-86).  The engine runs the two
// phases separately; after each phase every field of that phase that has callbacks is
// materialised in the reference's layouts, handed to the callback (device pointers in
// GPU mode, host pointers in RUN_CPU mode) and written back.
void evolver::run_callbacks_step() {
  const size_t n = (size_t)sx * sy * sz;
  auto ok = [&](int rc) {
    if (rc != 0) {
      if (throw_errors_) throw std::runtime_error(cupssgb_last_error());
      fatal(std::string("CUDA Runtime Error\n") + cupssgb_last_error());
    }
  };
  for (int phase = 0; phase < 2; ++phase) {
    ok(cupssgb_solver_advance_phase(solver_, phase));
    for (size_t i = 0; i < fields.size(); ++i) {
      field* f = fields[i];
      if ((int)f->dynamic != phase || !(f->hasCB || f->hasCBFourier)) continue;
      if (f->hasCBFourier) {
        if (f->callbackFourier == nullptr) {
          std::cout << "Wants to apply callback function in Fourier space but pointer to function is NULL"
                    << std::endl;
        } else {
          if (!f->comp_array_d)
            cuda_or_die(cudaMalloc((void**)&f->comp_array_d, n * sizeof(float2)), throw_errors_, "cudaMalloc");
          ok(cupssgb_solver_get_fourier_device(solver_, (int)i, reinterpret_cast<float*>(f->comp_array_d)));
          ok(cupssgb_solver_synchronize(solver_));
          if (with_cuda) {
            f->callbackFourier(this, f->comp_array_d, sx, sy, sz);
          } else {
            cuda_or_die(cudaMemcpy(f->comp_array, f->comp_array_d, n * sizeof(float2), cudaMemcpyDeviceToHost),
                        throw_errors_, "cudaMemcpy");
            f->callbackFourier(this, f->comp_array, sx, sy, sz);
            cuda_or_die(cudaMemcpy(f->comp_array_d, f->comp_array, n * sizeof(float2), cudaMemcpyHostToDevice),
                        throw_errors_, "cudaMemcpy");
          }
          cuda_or_die(cudaDeviceSynchronize(), throw_errors_, "Fourier callback");
          ok(cupssgb_solver_set_fourier_device(solver_, (int)i, reinterpret_cast<float*>(f->comp_array_d)));
        }
      }
      if (f->hasCB) {
        if (f->callback == nullptr) {
          std::cout << "Wants to apply callback function but pointer to function is NULL" << std::endl;
          continue;
        }
        if (!f->real_array_d)
          cuda_or_die(cudaMalloc((void**)&f->real_array_d, n * sizeof(float2)), throw_errors_, "cudaMalloc");
        if (f->needsaliasing && !f->real_dealiased_d)
          cuda_or_die(cudaMalloc((void**)&f->real_dealiased_d, n * sizeof(float2)), throw_errors_, "cudaMalloc");
        ok(cupssgb_solver_get_real_pairs_device(solver_, (int)i, reinterpret_cast<float*>(f->real_array_d)));
        if (f->needsaliasing)
          ok(cupssgb_solver_get_dealiased_pairs_device(solver_, (int)i,
                                                       reinterpret_cast<float*>(f->real_dealiased_d)));
        ok(cupssgb_solver_synchronize(solver_));
        if (with_cuda) {
          f->callback(this, f->real_array_d, sx, sy, sz);
          if (f->needsaliasing) f->callback(this, f->real_dealiased_d, sx, sy, sz);
        } else {
          if (f->needsaliasing && !f->real_dealiased) f->real_dealiased = new float2[n];
          cuda_or_die(cudaMemcpy(f->real_array, f->real_array_d, n * sizeof(float2), cudaMemcpyDeviceToHost),
                      throw_errors_, "cudaMemcpy");
          f->callback(this, f->real_array, sx, sy, sz);
          cuda_or_die(cudaMemcpy(f->real_array_d, f->real_array, n * sizeof(float2), cudaMemcpyHostToDevice),
                      throw_errors_, "cudaMemcpy");
          if (f->needsaliasing) {
            cuda_or_die(cudaMemcpy(f->real_dealiased, f->real_dealiased_d, n * sizeof(float2),
                                   cudaMemcpyDeviceToHost),
                        throw_errors_, "cudaMemcpy");
            f->callback(this, f->real_dealiased, sx, sy, sz);
            cuda_or_die(cudaMemcpy(f->real_dealiased_d, f->real_dealiased, n * sizeof(float2),
                                   cudaMemcpyHostToDevice),
                        throw_errors_, "cudaMemcpy");
          }
        }
        cuda_or_die(cudaDeviceSynchronize(), throw_errors_, "callback");
        ok(cupssgb_solver_set_real_pairs_device(solver_, (int)i, reinterpret_cast<float*>(f->real_array_d),
                                                f->needsaliasing ? reinterpret_cast<float*>(f->real_dealiased_d)
                                                                 : nullptr));
      }
    }
  }
}

int evolver::advanceTime() {
  if (!solver_) {
    if (throw_errors_) throw std::runtime_error("advanceTime before prepareProblem");
    fatal("ERROR: advanceTime before prepareProblem");
  }
  report_output_error();
  if (currentTimeStep % writeEveryNSteps == 0) writeOut();
  if (has_callbacks()) {
    run_callbacks_step();
  } else if (cupssgb_solver_advance(solver_, 1) != 0) {
    if (throw_errors_) throw std::runtime_error(cupssgb_last_error());
    fatal(std::string("CUDA Runtime Error\n") + cupssgb_last_error());
  }
  currentTime += dt;
  currentTimeStep += 1;
  // host-mirror mode: RUN_CPU callers read real_array / comp_array directly after
  // each step (e.g. examples/06_kpz/06_kpz.cpp:46-52)
  if (!with_cuda) sync_host_arrays();
  return 0;
}

int evolver::advanceTimeSteps(int n) {
  // Equivalent to n advanceTime() calls; consecutive steps without output are
  // queued in one call to the engine.
  if (!solver_) {
    if (throw_errors_) throw std::runtime_error("advanceTimeSteps before prepareProblem");
    fatal("ERROR: advanceTimeSteps before prepareProblem");
  }
  bool any_output = false;
  for (field* f : fields) any_output = any_output || f->outputToFile;
  if (!with_cuda || has_callbacks()) {
    for (int i = 0; i < n; ++i) advanceTime();
    return 0;
  }
  int done = 0;
  while (done < n) {
    if (any_output && currentTimeStep % writeEveryNSteps == 0) writeOut();
    int chunk = n - done;
    if (any_output) {
      const int to_next = writeEveryNSteps - (currentTimeStep % writeEveryNSteps);
      if (to_next < chunk) chunk = to_next;
    }
    if (cupssgb_solver_advance(solver_, chunk) != 0) {
      if (throw_errors_) throw std::runtime_error(cupssgb_last_error());
      fatal(std::string("CUDA Runtime Error\n") + cupssgb_last_error());
    }
    currentTimeStep += chunk;
    currentTime += dt * chunk;
    done += chunk;
  }
  return 0;
}

// GPU fields are copied out on the engine's output stream and written by the background
// writer, so the steps queued after this call run while the files are formatted; RUN_CPU
// fields (host arrays refreshed every step) are written here.  Same files, format and
// NaN rule as the reference (src/evolver.cpp:228-232, src/field.cpp:350-402).
void evolver::writeOut() {
  report_output_error();
  const size_t n = (size_t)sx * sy * sz;
  for (size_t i = 0; i < fields.size(); ++i) {
    field* f = fields[i];
    if (!f->outputToFile) continue;
    if (!with_cuda || !solver_) {
      f->writeToFile(currentTimeStep, dimension, writePrecision);
      continue;
    }
    if (!writer_) {
      int dev = 0;
      cudaGetDevice(&dev);
      writer_ = new cupssgb_host::OutputWriter(dev, n);
    }
    float* buf = nullptr;
    void* done = nullptr;
    int rc = writer_->acquire(&buf, &done);
    if (rc == 0) {
      rc = cupssgb_solver_snapshot_real(solver_, (int)i, buf, done);
      if (rc == 0)
        writer_->submit("data/" + f->name + ".csv." + std::to_string(currentTimeStep), f->name, sx, sy, sz,
                        dimension, writePrecision, buf, done);
      else
        writer_->release(buf, done);
    }
    if (rc != 0) {
      if (throw_errors_) throw std::runtime_error(cupssgb_last_error());
      fatal(std::string("ERROR: output of field ") + f->name + ": " + cupssgb_last_error());
    }
  }
}

void evolver::report_output_error() {
  if (!writer_) return;
  const std::string err = writer_->error();
  if (err.empty()) return;
  if (throw_errors_) throw std::runtime_error(err);
  fatal(err);
}

void evolver::flushOutput() {
  if (!writer_) return;
  const std::string err = writer_->flush();
  if (err.empty()) return;
  if (throw_errors_) throw std::runtime_error(err);
  fatal(err);
}

void evolver::setVerbose() { verbose = true; }
void evolver::unsetVerbose() { verbose = false; }

void evolver::printInformation() {
  std::cout << std::fixed << std::setprecision(3);
  std::cout << "Information on this evolver:" << std::endl;
  std::cout << dimension << "-dimensional system of size " << sx << "x" << sy << "x" << sz << std::endl;
  std::cout << "Physical size " << (float)sx * dx << "x" << (float)sy * dy << "x" << (float)sz * dz
            << " with cells of size " << dx << "x" << dy << "x" << dz << std::endl;
  std::cout << "There are " << fields.size() << " fields." << std::endl;
  for (size_t i = 0; i < fields.size(); ++i) {
    field* f = fields[i];
    std::cout << "Field " << i << ": " << f->name;
    std::cout << (f->dynamic ? " is dynamic." : " is not dynamic");
    std::cout << " and has " << f->terms.size() << " explicit terms";
    std::cout << " and " << f->implicit.size() << " implicit terms.";
    std::cout << " Runs on GPU: " << f->isCUDA;
    if (f->needsaliasing)
      std::cout << ". Will be dealiased for a nonlinearity of order " << f->aliasing_order;
    else
      std::cout << ". Will not be dealised.";
    std::cout << std::endl << "\t";
    if (f->dynamic) std::cout << "(d/dt)";
    std::cout << f->name;
    if (f->dynamic) std::cout << " = ";
    auto mono = [](const pres& p) {
      std::string s;
      if (p.iqx != 0) s += "(iqx)^(" + std::to_string(p.iqx) + ")";
      if (p.iqy != 0) s += "(iqy)^(" + std::to_string(p.iqy) + ")";
      if (p.iqz != 0) s += "(iqz)^(" + std::to_string(p.iqz) + ")";
      if (p.q2n != 0) s += "(q)^(" + std::to_string(2 * p.q2n) + ")";
      if (p.invq != 0) s += "(1/|q|)^(" + std::to_string(p.invq) + ")";
      return s;
    };
    if (!f->implicit.empty()) {
      std::string line = "[";
      for (const pres& p : f->implicit) {
        if (p.preFactor > 0.0f) line += "+";
        line += std::to_string(p.preFactor) + mono(p);
      }
      line += "]";
      if (f->dynamic) line += f->name;
      std::cout << line;
    }
    if (!f->dynamic) std::cout << " = ";
    for (size_t j = 0; j < f->terms.size(); ++j) {
      std::string line = (j != 0) ? " + [" : " [";
      const term* t = f->terms[j];
      for (size_t p = 0; p < t->prefactors_h.size(); ++p) {
        line += " + (" + std::to_string(t->prefactors_h[p].preFactor) + ")" + mono(t->prefactors_h[p]);
        if (p != t->prefactors_h.size() - 1) line += " + ";
      }
      line += "] (";
      for (const field* g : t->product) line += " " + g->name;
      line += " )";
      std::cout << line;
    }
    if (f->isNoisy) {
      std::cout << "+ sqrt[2*" << f->noise_amplitude.preFactor;
      if (f->noise_amplitude.q2n != 0) std::cout << "*q^" << f->noise_amplitude.q2n * 2;
      if (f->noise_amplitude.invq != 0) std::cout << "*1/|q|^" << f->noise_amplitude.invq;
      std::cout << "] x noise";
    }
    std::cout << std::endl << std::endl;
  }
}

int evolver::createTerm(const std::string& fname, const std::vector<pres>& prefactors,
                        const std::vector<std::string>& product) {
  const int idx = existsField(fname);
  if (idx == -1) {
    std::cout << "Field " << fname << " not found trying to create term" << std::endl;
    return 1;
  }
  term* t = new term(sx, sy, sz, dx, dy, dz);
  t->isCUDA = with_cuda;
  for (const std::string& pn : product)
    for (field* g : fields)
      if (g->name == pn) t->product.push_back(g);
  t->prefactors_h = prefactors;
  t->blocks = blocks;
  t->threads_per_block = threads_per_block;
  fields[idx]->terms.push_back(t);
  return 0;
}

void evolver::copyAllDataToHost() { sync_host_arrays(); }

int evolver::getSystemSizeX() { return sx; }
int evolver::getSystemSizeY() { return sy; }
int evolver::getSystemSizeZ() { return sz; }
float evolver::getSystemPhysicalSizeX() { return (float)sx * dx; }
float evolver::getSystemPhysicalSizeY() { return (float)sy * dy; }
float evolver::getSystemPhysicalSizeZ() { return (float)sz * dz; }
int evolver::getCurrentTimestep() { return currentTimeStep; }
float evolver::getCurrentTime() { return currentTime; }
bool evolver::getCuda() { return with_cuda; }

float evolver::getParameter(const std::string& name) {
  float v = 0.f;
  CUPSS_GUARD(v = _parser->getParameter(name));
  return v;
}

void evolver::push_parameters_to_solver() {
  if (!solver_) return;
  for (size_t i = 0; i < fields.size(); ++i) {
    field* f = fields[i];
    std::vector<cupssgb_pres> imp = to_c(f->implicit);
    cupssgb_solver_update_implicit(solver_, (int)i, imp.data(), (int)imp.size());
    for (size_t t = 0; t < f->terms.size(); ++t) {
      std::vector<cupssgb_pres> pv = to_c(f->terms[t]->prefactors_h);
      cupssgb_solver_set_term_pres(solver_, (int)i, (int)t, pv.data(), (int)pv.size());
    }
  }
}

int evolver::updateParameter(const std::string& name, float value) {
  CUPSS_GUARD(_parser->changeParameter(name, value));
  CUPSS_GUARD(for (field* f : fields) f->updateParameter(name, value));
  push_parameters_to_solver();
  if (writeParametersOnUpdate)
    _parser->writeParamsToFile("data/parameter_list.txt." + std::to_string(currentTimeStep));
  return 0;
}
