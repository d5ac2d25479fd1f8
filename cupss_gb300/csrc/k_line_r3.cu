// Line lengths 3 * 2^a (y and z axes of grids such as 96^3 or 192^3).
#include "k_line_inst.cuh"
CUPSSGB_LINE_INST(6)
CUPSSGB_LINE_INST(12)
CUPSSGB_LINE_INST(24)
CUPSSGB_LINE_INST(48)
CUPSSGB_LINE_INST(96)
CUPSSGB_LINE_INST(192)
