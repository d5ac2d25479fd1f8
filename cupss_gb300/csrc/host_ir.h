// System description shared by the batched forms (ensemble, server): the calls that
// declare a system on an evolver, replayed per member with that member's parameter
// values, and the parser's IR that results.
#pragma once
#include <map>
#include <string>
#include <vector>

#include "../../include/cupss_gb300.h"

namespace cupssgb_host {

// One declaration call: createField / addParameter / addEquation / addNoise.
struct SystemOp {
  enum Kind { kField, kParameter, kEquation, kNoise } kind;
  std::string a, b;     // field or parameter name / equation / noise amplitude
  float value = 0.f;    // parameter default
  bool dynamic = false;
};

struct IrTerm {
  std::vector<int> product;
  std::vector<cupssgb_pres> pres;
};

struct IrField {
  std::string name;
  bool dynamic = false;
  std::vector<cupssgb_pres> implicit;
  std::vector<IrTerm> terms;
  bool noisy = false;
  cupssgb_pres noise{};
};

// Parses the system with the library's parser (the evolver's, src/parser.cpp
// semantics) using `values` for the parameters it names (others keep their
// defaults).  Throws ParseError / std::runtime_error.
std::vector<IrField> parse_system(const std::vector<SystemOp>& ops, const std::map<std::string, float>& values);

// Everything of the IR except the numerical prefactor values: members with equal
// keys (and grids) can share one batch solver.
std::string structure_key(const std::vector<IrField>& ir);

// Creates a solver for `ir` (not prepared).  Throws on failure.
cupssgb_solver* create_solver(const std::vector<IrField>& ir, int sx, int sy, int sz, float dx, float dy, float dz,
                              float dt);
// Gives batch member m the values of `ir` (same structure as the solver's) and seed.
void set_member(cupssgb_solver* s, int m, const std::vector<IrField>& ir, unsigned long long seed);

// Throws CapiError with cupssgb_last_error() if rc < 0.
void ok(int rc);

}  // namespace cupssgb_host
