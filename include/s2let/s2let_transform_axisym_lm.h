/*
 * s2let_transform_axisym_lm.h: the per-module header name of the S2LET C API
 * (include/s2let/s2let_transform_axisym_lm.h of S2LET 2.2.7: axisymmetric wavelets in harmonic space).
 * The declarations, with the reference's names, signatures and layouts, are
 * in s2let_gpu.h and are implemented by libs2let_gpu.so.
 */
#ifndef S2LET_transform_AXISYM_LM
#define S2LET_transform_AXISYM_LM
#include "../s2let_gpu.h"
#endif
