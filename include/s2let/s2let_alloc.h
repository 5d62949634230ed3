/*
 * s2let_alloc.h: the per-module header name of the S2LET C API
 * (include/s2let/s2let_alloc.h of S2LET 2.2.7: s2let_allocate_* (calloc'ed host buffers)).
 * The declarations, with the reference's names, signatures and layouts, are
 * in s2let_gpu.h and are implemented by libs2let_gpu.so.
 */
#ifndef S2LET_ALLOC
#define S2LET_ALLOC
#include "../s2let_gpu.h"
#endif
