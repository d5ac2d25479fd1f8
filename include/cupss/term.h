// term: one explicit RHS group of a field -- product of fields times a sum of
// q-monomials (reference interface: inc/cupss/term.h:14-70).  The engine executes
// it; this class keeps the IR for printInformation and updateParameter.
#ifndef CUPSS_GB300_TERM_H
#define CUPSS_GB300_TERM_H

#include <map>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "defines.h"

class field;

class term {
 private:
  const int sx, sy, sz;
  const float dx, dy, dz;
  const float stepqx, stepqy, stepqz;

 public:
  term(int, float);
  term(int, int, float, float);
  term(int, int, int, float, float, float);
  ~term();
  void common_constructor();

  bool isCUDA;

  pres prefactors;
  std::vector<pres> prefactors_h;

  std::vector<field*> product;
  int multiply_by_i_pre;

  dim3 threads_per_block;
  dim3 blocks;

  // dynamic update of parameters
  std::map<std::string, int> usedParameters;
  std::vector<std::string> prefactor_strings;
  int setPrefactorString(const std::vector<std::string>&);
  void printPrefactorString();
};

#endif  // CUPSS_GB300_TERM_H
