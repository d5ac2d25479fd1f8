// check_error / check_device of the drop-in API (inc/cupss/cu_utils.h:6-7 in the
// reference).  Both keep the reference's contract -- a failed CUDA status or a machine
// without a GPU ends the program with status 1 -- on top of this library's status-code
// query cupssgb_device_info.
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "../../include/cupss.h"
#include "../../include/cupss_gb300.h"

void check_error(cudaError_t err) {
  if (err == cudaSuccess) return;
  std::fprintf(stderr, "cupss: CUDA call failed (%s): %s\n", cudaGetErrorName(err), cudaGetErrorString(err));
  std::exit(1);
}

void check_device() {
  std::vector<char> text(4096);
  const int n = cupssgb_device_info(text.data(), (int)text.size());
  if (n < 0) {
    std::fprintf(stderr, "cupss: device query failed: %s\n", cupssgb_last_error());
    std::exit(1);
  }
  if (n == 0) {
    std::fprintf(stderr, "cupss: a GPU run was asked for but no CUDA device is visible\n");
    std::exit(1);
  }
  std::printf("cupss: %d CUDA device%s\n%s", n, n == 1 ? "" : "s", text.data());
}
