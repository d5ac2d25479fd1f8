// field and term: host-side holders of one field's arrays and IR.
// Reference behaviour restated: constructors and q-steps (src/field_init.cpp:191-213,
// src/term_init.cpp:103-119), writeToFile CSV format and NaN check
// (src/field.cpp:350-402), implicit/prefactor strings and updateParameter
// (src/field.cpp:408-441, src/term.cpp:27-46).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <iostream>

#include "../../include/cupss.h"
#include "../../include/cupss_gb300.h"

void field::common_constructor() {
  const size_t n = (size_t)sx * sy * sz;
  real_array = new float2[n];
  comp_array = new float2[n];
  for (size_t i = 0; i < n; ++i) {
    real_array[i] = make_float2(0.f, 0.f);
    comp_array[i] = make_float2(0.f, 0.f);
  }
  real_array_d = nullptr;
  comp_array_d = nullptr;
  real_dealiased = nullptr;
  real_dealiased_d = nullptr;
  needsaliasing = false;
  aliasing_order = 1;
  outputToFile = false;
  hasCB = false;
  callback = nullptr;
  hasCBFourier = false;
  callbackFourier = nullptr;
  isNoisy = false;
  noiseType = GaussianWhite;
  isCUDA = true;
  dynamic = false;
  integrator = EULER;
  system_p = nullptr;
}

field::field(int _sx, float _dx)
    : sx(_sx), sy(1), sz(1), dx(_dx), dy(1.0f), dz(1.0f),
      stepqx(2.0f * PI / (_dx * (float)_sx)), stepqy(2.0f * PI), stepqz(2.0f * PI) {
  common_constructor();
}

field::field(int _sx, int _sy, float _dx, float _dy)
    : sx(_sx), sy(_sy), sz(1), dx(_dx), dy(_dy), dz(1.0f),
      stepqx(2.0f * PI / (_dx * (float)_sx)), stepqy(2.0f * PI / (_dy * (float)_sy)), stepqz(2.0f * PI) {
  common_constructor();
}

field::field(int _sx, int _sy, int _sz, float _dx, float _dy, float _dz)
    : sx(_sx), sy(_sy), sz(_sz), dx(_dx), dy(_dy), dz(_dz),
      stepqx(2.0f * PI / (_dx * (float)_sx)), stepqy(2.0f * PI / (_dy * (float)_sy)),
      stepqz(2.0f * PI / (_dz * (float)_sz)) {
  common_constructor();
}

field::~field() {
  delete[] real_array;
  delete[] comp_array;
  delete[] real_dealiased;
  if (real_array_d) cudaFree(real_array_d);
  if (comp_array_d) cudaFree(comp_array_d);
  if (real_dealiased_d) cudaFree(real_dealiased_d);
  for (term* t : terms) delete t;
}

void field::copyHostToDevice() {
  const size_t n = (size_t)sx * sy * sz;
  if (real_array_d) cudaMemcpy(real_array_d, real_array, n * sizeof(float2), cudaMemcpyHostToDevice);
  if (comp_array_d) cudaMemcpy(comp_array_d, comp_array, n * sizeof(float2), cudaMemcpyHostToDevice);
}

void field::copyDeviceToHost() {
  if (system_p) {
    cupssgb_solver* s = system_p->solverHandle();
    if (s) {
      int idx = system_p->existsField(name);
      const size_t n = (size_t)sx * sy * sz;
      std::vector<float> tmp(n);
      if (cupssgb_solver_get_real(s, idx, tmp.data()) == 0)
        for (size_t i = 0; i < n; ++i) real_array[i] = make_float2(tmp[i], 0.f);
      cupssgb_solver_get_fourier(s, idx, reinterpret_cast<float*>(comp_array));
    }
  }
}

void field::writeToFile(int currentTimeStep, int dim, int writePrecision) {
  if (!outputToFile) return;
  if (isCUDA && system_p && system_p->solverHandle()) {
    const size_t n = (size_t)sx * sy * sz;
    std::vector<float> tmp(n);
    cupssgb_solver_get_real(system_p->solverHandle(), system_p->existsField(name), tmp.data());
    for (size_t i = 0; i < n; ++i) real_array[i] = make_float2(tmp[i], 0.f);
  }
  const std::string file_name = "data/" + name + ".csv." + std::to_string(currentTimeStep);
  FILE* fp = std::fopen(file_name.c_str(), "w+");
  if (fp == nullptr) {
    std::cout << "Error creating output file at timestep" << currentTimeStep << std::endl;
    std::exit(1);
  }
  std::string fmt = "%i, ";
  std::fprintf(fp, "x, ");
  if (dim == 2) {
    std::fprintf(fp, "y, ");
    fmt += "%i, ";
  }
  if (dim == 3) {
    std::fprintf(fp, "y, z, ");
    fmt += "%i, %i, ";
  }
  std::fprintf(fp, "%s\n", name.c_str());
  fmt += "%." + std::to_string(writePrecision) + "f\n";
  for (int k = 0; k < sz; ++k)
    for (int j = 0; j < sy; ++j)
      for (int i = 0; i < sx; ++i) {
        const size_t idx = (size_t)k * sx * sy + (size_t)j * sx + i;
        const float v = real_array[idx].x;
        if (std::isnan(v)) {
          std::cout << "NaN found in field " << name << std::endl;
          std::exit(1);
        }
        int w = 0;
        if (dim == 1) w = std::fprintf(fp, fmt.c_str(), i, v);
        if (dim == 2) w = std::fprintf(fp, fmt.c_str(), i, j, v);
        if (dim == 3) w = std::fprintf(fp, fmt.c_str(), i, j, k, v);
        if (w < 0) {
          std::cout << "Error writing data to output file " << file_name << std::endl;
          std::exit(1);
        }
      }
  std::fclose(fp);
}

float field::getStepqx() { return stepqx; }
float field::getStepqy() { return stepqy; }
float field::getStepqz() { return stepqz; }

int field::addImplicitString(const std::string& s) {
  implicit_prefactor_strings.push_back(s);
  return 0;
}

void field::printImplicitString() {
  for (const std::string& s : implicit_prefactor_strings) std::cout << s << std::endl;
  for (const auto& kv : usedParameters) std::cout << kv.first << " " << kv.second << std::endl;
}

int field::updateParameter(const std::string& pname, float) {
  // Re-derive the pres of every string that mentions the parameter
  // (src/field.cpp:422-441); the evolver pushes the new pres to the engine.
  if (usedParameters[pname])
    system_p->_parser->recalculateImplicits(implicit_prefactor_strings, implicit, dynamic ? 1 : 0);
  for (term* t : terms)
    if (t->usedParameters[pname])
      system_p->_parser->recalculateImplicits(t->prefactor_strings, t->prefactors_h, 0);
  return 0;
}

// ---------------------------------------------------------------------------------
void term::common_constructor() {
  isCUDA = true;
  multiply_by_i_pre = 0;
}

term::term(int _sx, float _dx)
    : sx(_sx), sy(1), sz(1), dx(_dx), dy(1.0f), dz(1.0f), stepqx(2.0f * PI / (_dx * (float)_sx)),
      stepqy(2.0f * PI), stepqz(2.0f * PI) {
  common_constructor();
}

term::term(int _sx, int _sy, float _dx, float _dy)
    : sx(_sx), sy(_sy), sz(1), dx(_dx), dy(_dy), dz(1.0f), stepqx(2.0f * PI / (_dx * (float)_sx)),
      stepqy(2.0f * PI / (_dy * (float)_sy)), stepqz(2.0f * PI) {
  common_constructor();
}

term::term(int _sx, int _sy, int _sz, float _dx, float _dy, float _dz)
    : sx(_sx), sy(_sy), sz(_sz), dx(_dx), dy(_dy), dz(_dz), stepqx(2.0f * PI / (_dx * (float)_sx)),
      stepqy(2.0f * PI / (_dy * (float)_sy)), stepqz(2.0f * PI / (_dz * (float)_sz)) {
  common_constructor();
}

term::~term() {}

int term::setPrefactorString(const std::vector<std::string>& s) {
  prefactor_strings.insert(prefactor_strings.end(), s.begin(), s.end());
  return 0;
}

void term::printPrefactorString() {
  for (const std::string& s : prefactor_strings) std::cout << s << std::endl;
  for (const auto& kv : usedParameters) std::cout << kv.first << " " << kv.second << std::endl;
}
