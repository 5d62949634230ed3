/*
 * s2let_fits.h: the per-module header name of the S2LET C API
 * (include/s2let/s2let_fits.h of S2LET 2.2.7: FITS I/O of MW / MWSS maps (written without cfitsio)).
 * The declarations, with the reference's names, signatures and layouts, are
 * in s2let_gpu.h and are implemented by libs2let_gpu.so.
 */
#ifndef S2LET_FITS
#define S2LET_FITS
#include "../s2let_gpu.h"
#endif
