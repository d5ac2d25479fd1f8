/* Umbrella header of the GB300-native cuPSS drop-in (same include set as the
 * reference's inc/cupss.h:1-6). */
#include "cupss/defines.h"
#include "cupss/cu_utils.h"
#include "cupss/evolver.h"
#include "cupss/field.h"
#include "cupss/term.h"
#include "cupss/parser.h"
