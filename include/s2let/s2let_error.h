/*
 * s2let_error.h: the error macros of the S2LET C API
 * (include/s2let/s2let_error.h of S2LET 2.2.7), for callers that use them in
 * their own code.  libs2let_gpu.so itself never exits: it records a status
 * (s2let_gpu_last_error) unless S2LET_GPU_ABORT_ON_ERROR=1 is set.
 */
#ifndef S2LET_ERROR
#define S2LET_ERROR
#include <stdio.h>
#include <stdlib.h>
#include "../s2let_gpu.h"

/* prints the message and where it happened, then ends the process */
#define S2LET_ERROR_GENERIC(comment)                                              \
  {                                                                               \
    printf("ERROR: %s.\n", comment);                                             \
    printf("ERROR: Occurred in function <%s> of file %s on line %d.\n", __func__, \
           __FILE__, __LINE__);                                                   \
    exit(1);                                                                      \
  }

#define S2LET_ERROR_MEM_ALLOC_CHECK(pointer)                                      \
  if ((pointer) == NULL) {                                                        \
    S2LET_ERROR_GENERIC("Memory allocation failed")                               \
  }
#endif
