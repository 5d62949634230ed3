/* ORACLE / TEST INFRASTRUCTURE ONLY: multi-transform entry points shared by the
 * SSHT and SO3 restatements (several spins evaluated in one sweep over l). */
#ifndef ORACLE_INTERNAL_H
#define ORACLE_INTERNAL_H
#include <complex.h>

/* f[j] is double* when real[j] != 0 (spin must be 0), else complex double*.
 * ss = 0: MW sampling, ss = 1: MWSS sampling. */
void oracle_ssht_inverse_multi(void **f, const complex double **flm, const int *spin,
                               const int *real, int njob, int L, int ss);
void oracle_ssht_forward_multi(complex double **flm, const void **f, const int *spin,
                               const int *real, int njob, int L, int ss);
void oracle_ssht_adjoint_inverse_multi(complex double **flm, const void **f, const int *spin,
                                       const int *real, int njob, int L, int ss);
void oracle_ssht_adjoint_forward_multi(void **f, const complex double **flm, const int *spin,
                                       const int *real, int njob, int L, int ss);
#endif
