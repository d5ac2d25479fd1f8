// Host-side initial conditions written into field::real_array (fieldsReal).
// Same formulas and error behaviour as the reference (src/initializers.cpp:14-267).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <ctime>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <string>

#include "../../include/cupss.h"

namespace {
// The reference prints the message and exits with status 1; an evolver driven through
// the C-ABI (setThrowOnError) throws instead.
[[noreturn]] void init_error(bool throw_errors, const std::string& msg) {
  if (throw_errors) throw std::runtime_error(msg);
  std::cout << msg << std::endl;
  std::exit(1);
}
void require_field(evolver* e, bool throw_errors, const std::string& name, const char* what) {
  if (e->existsField(name) < 0) init_error(throw_errors, std::string("ERROR in ") + what + ", " + name + " not found");
}
}  // namespace

void evolver::initializeUniform(std::string f, float value) {
  require_field(this, throw_errors_, f, "initialize uniform");
  float2* a = fieldsMap[f]->real_array;
  const size_t n = (size_t)sx * sy * sz;
  for (size_t i = 0; i < n; ++i) a[i].x = value;
}

void evolver::initializeUniformNoise(std::string f, float value) {
  require_field(this, throw_errors_, f, "initialize uniform");
  std::srand(time(0));
  float2* a = fieldsMap[f]->real_array;
  const size_t n = (size_t)sx * sy * sz;
  for (size_t i = 0; i < n; ++i) a[i].x = value * 0.01f * (float)(std::rand() % 200 - 100);
}

void evolver::initializeNormalNoise(std::string f, float mean, float sigma) {
  require_field(this, throw_errors_, f, "initialize uniform");
  std::srand(time(0));
  float2* a = fieldsMap[f]->real_array;
  const size_t n = (size_t)sx * sy * sz;
  // Box-Muller on pairs of points, as the reference (src/initializers.cpp:77-94)
  for (size_t i = 0; i + 1 < n + 1; i += 2) {
    const float v1 = 0.01 * (float)(std::rand() % 100 + 1);
    const float v2 = 0.01 * (float)(std::rand() % 100 + 1);
    a[i].x = sigma * sigma * std::sqrt(-2.0 * std::log(v1)) * std::cos(2.0 * PI * v2) + mean;
    if (i + 1 < n) a[i + 1].x = sigma * sigma * std::sqrt(-2.0 * std::log(v1)) * std::sin(2.0 * PI * v2) + mean;
  }
}

void evolver::initializeHalfSystem(std::string f, float val1, float val2, float xi, int direction) {
  require_field(this, throw_errors_, f, "initialize half system");
  if (xi <= 0.0) {
    init_error(throw_errors_, "ERROR in initialize, interface width cannot be 0 or negative");
  }
  if (direction < 1 || direction > 3) {
    init_error(throw_errors_, "ERROR in initialize, direction can be 1, 2 or 3 for x, y, z, respectively");
  }
  std::srand(time(0));
  const int rev = direction == 1 ? sx : (direction == 2 ? sy : sz);
  float2* a = fieldsMap[f]->real_array;
  for (int k = 0; k < sz; ++k)
    for (int j = 0; j < sy; ++j)
      for (int i = 0; i < sx; ++i) {
        const int ref = direction == 1 ? i : (direction == 2 ? j : k);
        const size_t idx = (size_t)k * sx * sy + (size_t)j * sx + i;
        a[idx].x = val1 + (val2 - val1) * 0.5 * (1.0 + std::tanh((ref - rev / 2) / (std::sqrt(2) * xi)));
      }
}

void evolver::initializeDroplet(std::string f, float val1, float val2, float radius, float xi, int p_x,
                                int p_y, int p_z) {
  require_field(this, throw_errors_, f, "initialize droplet");
  if (xi <= 0.0 || radius <= 0.0) {
    init_error(throw_errors_, "ERROR in initialize, droplet radius and interface width cannot be 0 or negative");
  }
  const int x0 = p_x % sx, y0 = p_y % sy, z0 = p_z % sz;
  std::srand(time(0));
  float2* a = fieldsMap[f]->real_array;
  for (int k = 0; k < sz; ++k)
    for (int j = 0; j < sy; ++j)
      for (int i = 0; i < sx; ++i) {
        const float xd = i - x0, yd = j - y0, zd = k - z0;
        const float rc = std::sqrt(xd * xd + yd * yd + zd * zd);
        const size_t idx = (size_t)k * sx * sy + (size_t)j * sx + i;
        a[idx].x = val1 + (val2 - val1) * 0.5 * (1.0 + std::tanh((rc - radius) / (std::sqrt(2) * xi)));
      }
}

void evolver::addDroplet(std::string f, float val, float radius, float xi, int p_x, int p_y, int p_z) {
  require_field(this, throw_errors_, f, "initialize droplet");
  if (xi <= 0.0 || radius <= 0.0) {
    init_error(throw_errors_, "ERROR in initialize, droplet radius and interface width cannot be 0 or negative");
  }
  const int x0 = p_x % sx, y0 = p_y % sy, z0 = p_z % sz;
  std::srand(time(0));
  float2* a = fieldsMap[f]->real_array;
  for (int k = 0; k < sz; ++k)
    for (int j = 0; j < sy; ++j)
      for (int i = 0; i < sx; ++i) {
        const float xd = i - x0, yd = j - y0, zd = k - z0;
        const float rc = std::sqrt(xd * xd + yd * yd + zd * zd);
        const size_t idx = (size_t)k * sx * sy + (size_t)j * sx + i;
        a[idx].x += val * 0.5 * (1.0 + std::tanh((radius - rc) / (std::sqrt(2) * xi)));
      }
}

void evolver::initializeFromFile(std::string f, std::string file, int skiprows, char delimiter) {
  require_field(this, throw_errors_, f, "initialize droplet");
  FILE* chk = std::fopen(file.c_str(), "r");
  if (chk == nullptr) {
    init_error(throw_errors_, "Initial file: " + file + " not found. Doing nothing");
  }
  std::fclose(chk);
  std::ifstream in(file.c_str());
  std::string posx, posy = "0", posz = "0", value;
  for (int i = 0; i < skiprows; ++i) std::getline(in, posx);
  const size_t n = (size_t)sx * sy * sz;
  float2* a = fieldsMap[f]->real_array;
  for (size_t i = 0; i < n; ++i) {
    if (!std::getline(in, posx, delimiter)) {
      init_error(throw_errors_, "Incompatible number of lines on file " + file + ", only " + std::to_string(i + 1) +
                                    " found for a system size of " + std::to_string(n));
    }
    if (dimension > 1) std::getline(in, posy, delimiter);
    if (dimension > 2) std::getline(in, posz, delimiter);
    std::getline(in, value);
    const int px = std::stoi(posx), py = std::stoi(posy), pz = std::stoi(posz);
    a[(size_t)pz * sx * sy + (size_t)py * sx + px].x = std::stof(value);
  }
}
