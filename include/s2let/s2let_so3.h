/*
 * s2let_so3.h: the SO3 configuration helpers of the S2LET C API
 * (include/s2let/s2let_so3.h of S2LET 2.2.7).  libs2let_gpu.so carries its own
 * Wigner transforms and needs no SO3 library; these helpers fill an SO3
 * library's so3_parameters_t for callers that use SO3 themselves, and are
 * defined only when <so3/so3.h> can be included.
 */
#ifndef S2LET_SO3
#define S2LET_SO3
#include "../s2let_gpu.h"

#if defined(__has_include)
#if __has_include(<so3/so3.h>)
#include <so3/so3.h>
#define S2LET_SO3_N_ORDER SO3_N_ORDER_NEGATIVE_FIRST
#define S2LET_SO3_STORAGE SO3_STORAGE_COMPACT

/* the SO3 layout S2LET's wavelet coefficients use: compact storage, n
 * negative first, n of the parity that N selects (odd N: even n) */
static inline void fill_so3_parameters(so3_parameters_t *so3_parameters, const s2let_parameters_t *parameters) {
  so3_parameters->verbosity = parameters->verbosity;
  so3_parameters->L = parameters->L;
  so3_parameters->N = parameters->N;
  so3_parameters->sampling_scheme = (so3_sampling_t)parameters->sampling_scheme;
  so3_parameters->n_order = S2LET_SO3_N_ORDER;
  so3_parameters->storage = S2LET_SO3_STORAGE;
  so3_parameters->dl_method = parameters->dl_method;
  so3_parameters->reality = parameters->reality;
  so3_parameters->steerable = 0;
  so3_parameters->L0 = 0;
  so3_parameters->n_mode = (parameters->N % 2) ? SO3_N_MODE_EVEN : SO3_N_MODE_ODD;
}
#endif
#endif
#endif
