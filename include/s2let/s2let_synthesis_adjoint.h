/*
 * s2let_synthesis_adjoint.h: the per-module header name of the S2LET C API
 * (include/s2let/s2let_synthesis_adjoint.h of S2LET 2.2.7: the exact adjoints of the synthesis).
 * The declarations, with the reference's names, signatures and layouts, are
 * in s2let_gpu.h and are implemented by libs2let_gpu.so.
 */
#ifndef S2LET_SYNTHESIS_ADJOINT
#define S2LET_SYNTHESIS_ADJOINT
#include "../s2let_gpu.h"
#endif
