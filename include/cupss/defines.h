// Shared types of the cuPSS C++ API.  The members, order and defaults of these
// types are the reference's interface (inc/cupss/defines.h:1-62) and are kept
// identical so that user code and the pres IR stay binary/source compatible.
#ifndef CUPSS_GB300_DEFINES_H
#define CUPSS_GB300_DEFINES_H

#include <cuda_runtime.h>

#include <iostream>
#include <map>
#include <string>
#include <vector>

struct system_constants {
  int sx, sy, sz;
  float dx, dy, dz;
  float dt;
  int writeEveryNSteps;
};

// One q-monomial of an equation: preFactor * q^(2 q2n) * (iqx)^iqx * (iqy)^iqy *
// (iqz)^iqz * |q|^-invq.
struct pres {
  float preFactor = 0.0f;
  int q2n = 0;
  int iqx = 0;
  int iqy = 0;
  int iqz = 0;
  int invq = 0;
};

struct full_term {
  std::vector<pres> prefactors;
  std::vector<std::string> fields;
};

#define PI 3.1415926535f

enum DeviceToRunOn { RUN_CPU, RUN_GPU };
enum integrators { EULER, RK2, RK4 };
enum NoiseType { GaussianWhite };

#endif
