/*
 * s2let_lm.h: the per-module header name of the S2LET C API
 * (include/s2let/s2let_lm.h of S2LET 2.2.7: s2let_lm_power (the random-flm test helpers are not provided)).
 * The declarations, with the reference's names, signatures and layouts, are
 * in s2let_gpu.h and are implemented by libs2let_gpu.so.
 */
#ifndef S2LET_LM
#define S2LET_LM
#include "../s2let_gpu.h"
#endif
