// CUDA status helpers (reference: inc/cupss/cu_utils.h, src/cu_utils.cpp:4-37).
#ifndef CUPSS_GB300_CU_UTILS_H
#define CUPSS_GB300_CU_UTILS_H

#include "defines.h"

// Prints the CUDA error string and exits with status 1 if err != cudaSuccess.
void check_error(cudaError_t err);
// Prints the visible devices and the driver/runtime versions.
void check_device();

#endif
