/*
 * s2let_mw.h: the per-module header name of the S2LET C API
 * (include/s2let/s2let_mw.h of S2LET 2.2.7: plain MW spherical-harmonic transforms and power).
 * The declarations, with the reference's names, signatures and layouts, are
 * in s2let_gpu.h and are implemented by libs2let_gpu.so.
 */
#ifndef S2LET_MW
#define S2LET_MW
#include "../s2let_gpu.h"
#endif
