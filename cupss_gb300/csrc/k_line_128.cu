#include "k_line_inst.cuh"
CUPSSGB_LINE_INST(128)
