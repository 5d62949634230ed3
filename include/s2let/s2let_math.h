/*
 * s2let_math.h: the per-module header name of the S2LET C API
 * (include/s2let/s2let_math.h of S2LET 2.2.7: kappa quadrature, binomial coefficients, s2let_spin_normalization).
 * The declarations, with the reference's names, signatures and layouts, are
 * in s2let_gpu.h and are implemented by libs2let_gpu.so.
 */
#ifndef S2LET_MATH
#define S2LET_MATH
#include "../s2let_gpu.h"
#endif
