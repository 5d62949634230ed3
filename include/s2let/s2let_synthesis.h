/*
 * s2let_synthesis.h: the per-module header name of the S2LET C API
 * (include/s2let/s2let_synthesis.h of S2LET 2.2.7: lmn2lm, wav2lm, wav2px and their _real and _manual forms).
 * The declarations, with the reference's names, signatures and layouts, are
 * in s2let_gpu.h and are implemented by libs2let_gpu.so.
 */
#ifndef S2LET_SYNTHESIS
#define S2LET_SYNTHESIS
#include "../s2let_gpu.h"
#endif
