// Internal helpers shared by the drop-in host classes.
#pragma once
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

}  // namespace cupssgb_host
