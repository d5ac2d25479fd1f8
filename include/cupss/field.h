// field: one scalar field of a cuPSS system (reference interface:
// inc/cupss/field.h:21-145).  The public data members user code reads or writes
// (host arrays, callbacks, output flag, IR lists) keep their names and meaning.
// Device arrays real_array_d / comp_array_d are the reference's float2 layouts;
// this implementation materialises them for fields with callbacks (they are
// nullptr otherwise, because the engine keeps its own packed spectral state).
#ifndef CUPSS_GB300_FIELD_H
#define CUPSS_GB300_FIELD_H

#include <map>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "defines.h"

class term;
struct pres;
class evolver;

class field {
 private:
  const int sx, sy, sz;
  const float dx, dy, dz;
  const float stepqx, stepqy, stepqz;
  std::vector<std::string> implicit_prefactor_strings;

 public:
  field(int, float);
  field(int, int, float, float);
  field(int, int, int, float, float, float);
  ~field();
  void common_constructor();

  std::string name;
  std::map<std::string, int> usedParameters;  // only implicits
  bool isCUDA;
  bool outputToFile;
  evolver* system_p;
  bool dynamic;
  int integrator;

  // Noise
  bool isNoisy;
  NoiseType noiseType;

  // real_* : real space, comp_* : Fourier space, *_d : device pointers
  float2* real_array;
  float2* comp_array;
  float2* real_array_d;
  float2* comp_array_d;

  bool needsaliasing;
  int aliasing_order;
  float2* real_dealiased;      // host copy handed to callbacks in RUN_CPU mode
  float2* real_dealiased_d;

  std::vector<term*> terms;
  std::vector<pres> implicit;

  pres noise_amplitude;

  // callback functions (called with device pointers in GPU mode)
  bool hasCB;
  void (*callback)(evolver*, float2*, int, int, int);
  bool hasCBFourier;
  void (*callbackFourier)(evolver*, float2*, int, int, int);

  dim3 threads_per_block;
  dim3 blocks;

  void copyHostToDevice();
  void copyDeviceToHost();
  void writeToFile(int, int, int);

  float getStepqx();
  float getStepqy();
  float getStepqz();

  int addImplicitString(const std::string&);
  void printImplicitString();
  const std::vector<std::string>& implicitStrings() const { return implicit_prefactor_strings; }
  int updateParameter(const std::string&, float);
};

#endif  // CUPSS_GB300_FIELD_H
