// evolver: system container and public API of cuPSS (reference interface:
// inc/cupss/evolver.h:14-86).  Same public members and methods; the time step runs
// on the GB300 engine behind the C-ABI in cupss_gb300.h.
#ifndef CUPSS_GB300_EVOLVER_H
#define CUPSS_GB300_EVOLVER_H

#include <map>
#include <string>
#include <vector>

#include "defines.h"

class field;
class parser;
struct pres;
struct cupssgb_solver;
namespace cupssgb_host {
class OutputWriter;
}

class evolver {
 private:
  const int sx, sy, sz;
  const float dx, dy, dz;
  const int writeEveryNSteps;
  bool with_cuda;
  float currentTime;
  int currentTimeStep;
  bool verbose;
  // GB300 engine state
  cupssgb_solver* solver_;
  bool throw_errors_;
  bool seed_set_;
  unsigned long long seed_;
  void build_solver();
  void push_parameters_to_solver();
  void sync_host_arrays();
  void run_callbacks_step();
  bool has_callbacks() const;
  cupssgb_host::OutputWriter* writer_;   // writes writeOut's files in the background
  void report_output_error();

 public:
  int dimension;
  dim3 threads_per_block;
  dim3 blocks;
  float dt;
  float dtsqrt;
  std::vector<field*> fields;
  parser* _parser;
  evolver(bool, int, float, float, int);
  evolver(bool, int, int, float, float, float, int);
  evolver(bool, int, int, int, float, float, float, float, int);
  ~evolver();
  void common_constructor();

  // Direct access to fields
  std::map<std::string, field*> fieldsMap;
  std::map<std::string, float2*> fieldsReal;
  std::map<std::string, float2*> fieldsFourier;

  // Getters
  int getSystemSizeX();
  int getSystemSizeY();
  int getSystemSizeZ();
  float getSystemPhysicalSizeX();
  float getSystemPhysicalSizeY();
  float getSystemPhysicalSizeZ();
  int getCurrentTimestep();
  float getCurrentTime();
  bool getCuda();
  float getParameter(const std::string&);
  void printInformation();
  void setVerbose();
  void unsetVerbose();

  // System declaration functions
  void addField(field*);
  int createField(std::string, bool);
  int createTerm(const std::string&, const std::vector<pres>&, const std::vector<std::string>&);
  int addParameter(const std::string&, float);
  int addEquation(const std::string&);
  int addNoise(const std::string&, const std::string&);
  int createFromFile(const std::string&);
  int existsField(const std::string&);

  // Dynamics functions
  int advanceTime();
  void writeOut();
  void copyAllDataToHost();
  void setOutputField(const std::string&, int);
  int updateParameter(const std::string&, float);
  int writePrecision;
  bool writeParametersOnUpdate;

  // Initializing functions
  void prepareProblem();

  void initializeUniform(std::string field, float value);
  void initializeUniformNoise(std::string field, float amplitude);
  void initializeNormalNoise(std::string field, float mean, float sigma);
  void initializeHalfSystem(std::string field, float value1, float value2, float interface_width,
                            int direction);
  void initializeDroplet(std::string field, float value_out, float value_in, float radius,
                         float interface_width, int center_x, int center_y, int center_z);
  void addDroplet(std::string field, float value, float radius, float interface_width, int center_x,
                  int center_y, int center_z);
  void initializeFromFile(std::string field, std::string file, int skiprows, char delimiter);

  // Additions of this implementation (no counterpart in the reference).
  // Seed of the Fourier-space noise; without it the seed comes from time(NULL) like
  // the reference's cuRAND seeding (src/field_init.cpp:137).
  void setNoiseSeed(unsigned long long seed);
  // Run-many-steps entry: equivalent to n calls of advanceTime().
  int advanceTimeSteps(int n);
  // Parse/state errors throw std::runtime_error instead of printing and exiting.
  void setThrowOnError(bool on);
  // writeOut queues its files; a background thread writes them while the steps go on.
  // Waits until every queued file is written (the destructor does too).  A file that
  // could not be written, or a NaN in a field, is reported here or at the next writeOut
  // or advanceTime, the reference's way (message, exit status 1) unless errors throw.
  void flushOutput();
  cupssgb_solver* solverHandle();
};

#endif  // CUPSS_GB300_EVOLVER_H
