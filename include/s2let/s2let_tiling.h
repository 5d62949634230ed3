/*
 * s2let_tiling.h: the per-module header name of the S2LET C API
 * (include/s2let/s2let_tiling.h of S2LET 2.2.7: the harmonic tilings and their identity checks).
 * The declarations, with the reference's names, signatures and layouts, are
 * in s2let_gpu.h and are implemented by libs2let_gpu.so.
 */
#ifndef S2LET_TILING
#define S2LET_TILING
#include "../s2let_gpu.h"
#endif
