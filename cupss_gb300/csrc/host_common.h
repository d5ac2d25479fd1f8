// Internal helpers shared by the drop-in host classes.
#pragma once
#include <cstddef>
#include <stdexcept>
#include <string>

namespace cupssgb_host {

// Fatal parse / usage error.  The public C++ API reports it the way the reference
// does (message on stdout, exit status 1) unless evolver::setThrowOnError(true).
struct ParseError : std::runtime_error {
  explicit ParseError(const std::string& m) : std::runtime_error(m) {}
};

// A failed C-ABI call made by a host class, with its status code.
struct CapiError : std::runtime_error {
  int code;
  CapiError(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// Writes one field file in the reference's CSV format (src/field.cpp:350-402); returns ""
// or the error message (a NaN value, a file that cannot be written).
std::string write_field_csv(const std::string& path, const std::string& name, const float* values, int sx, int sy,
                            int sz, int dim, int precision);

// Background writer of writeOut's field files.  acquire() hands out a page-locked host
// buffer of npoints floats and a CUDA event; the caller queues the device-to-host copy
// into the buffer (recording the event when it completes) and submit()s the file, or
// gives both back with release().  A worker thread waits for each event, writes the
// file and recycles the buffer.  At most kMaxPending files are in flight; acquire()
// waits for the oldest beyond that.  flush() waits until every queued file is written;
// it and error() return the first failure not yet returned ("" if none).
class OutputWriter {
 public:
  static constexpr int kMaxPending = 3;
  OutputWriter(int device, size_t npoints);
  ~OutputWriter();   // writes the files still queued
  OutputWriter(const OutputWriter&) = delete;
  OutputWriter& operator=(const OutputWriter&) = delete;
  int acquire(float** buf, void** done_event);
  void submit(const std::string& path, const std::string& name, int sx, int sy, int sz, int dim, int precision,
              float* buf, void* done_event);
  void release(float* buf, void* done_event);
  std::string flush();
  std::string error();

 private:
  struct Impl;
  Impl* impl_;
};

}  // namespace cupssgb_host
