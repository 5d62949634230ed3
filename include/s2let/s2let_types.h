/*
 * s2let_types.h: the per-module header name of the S2LET C API
 * (include/s2let/s2let_types.h of S2LET 2.2.7: s2let_parameters_t, the sampling and wavelet-kind enums, S2LET_COMPLEX).
 * The declarations, with the reference's names, signatures and layouts, are
 * in s2let_gpu.h and are implemented by libs2let_gpu.so.
 */
#ifndef S2LET_TYPES
#define S2LET_TYPES
#include "../s2let_gpu.h"
#endif
