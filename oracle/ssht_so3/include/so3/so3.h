/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * The subset of the SO3 C API (Wigner transforms on the rotation group with
 * McEwen-Wiaux sampling) that the reference S2LET sources call.  SO3 is an
 * external dependency of the reference (conanfile.txt:2 pins
 * astro-informatics-so3 >= 1.3.4), absent from the reference tree.  Names,
 * struct fields and argument orders follow the reference call sites
 * (include/s2let/s2let_so3.h:24-42, src/c/s2let_analysis.c:67-76,348,432,
 * src/c/s2let_synthesis.c:361,444, src/c/s2let_analysis_adjoint.c:371,460,
 * src/c/s2let_synthesis_adjoint.c:352,441, test/c/test_adjoint.c:395-459).
 * Implementations (so3.c) are written from the SO3 sampling theorem
 * (McEwen, Buttner, Leistedt, Peiris & Wiaux 2015):
 *   f(a,b,g) = sum_{l,m,n} (2l+1)/(8 pi^2) flmn D^{l*}_{mn}(a,b,g),
 *   D^l_{mn}(a,b,g) = e^{-i m a} d^l_{mn}(b) e^{-i n g},
 *   a_p = 2 pi p/(2L-1), b_t = pi(2t+1)/(2L-1), g_k = 2 pi k/(2N-1),
 *   sample index k*L*(2L-1) + t*(2L-1) + p.
 * Storage: SO3_STORAGE_COMPACT keeps l >= |n| only; SO3_N_ORDER_NEGATIVE_FIRST
 * orders the n-blocks -N+1..N-1; real signals keep n >= 0 only.
 */
#ifndef ORACLE_SO3_H
#define ORACLE_SO3_H

#include <complex.h>
#include <stdio.h>
#include <stdlib.h>

#include <ssht/ssht.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum { SO3_SAMPLING_MW = 0, SO3_SAMPLING_MW_SS, SO3_SAMPLING_SIZE } so3_sampling_t;
typedef enum { SO3_N_ORDER_ZERO_FIRST = 0, SO3_N_ORDER_NEGATIVE_FIRST, SO3_N_ORDER_SIZE } so3_n_order_t;
typedef enum { SO3_STORAGE_PADDED = 0, SO3_STORAGE_COMPACT, SO3_STORAGE_SIZE } so3_storage_t;
typedef enum {
  SO3_N_MODE_ALL = 0,
  SO3_N_MODE_EVEN,
  SO3_N_MODE_ODD,
  SO3_N_MODE_MAXIMUM,
  SO3_N_MODE_L,
  SO3_N_MODE_SIZE
} so3_n_mode_t;

typedef struct {
  int verbosity;
  int reality;
  int L0;
  int L;
  int N;
  so3_sampling_t sampling_scheme;
  so3_n_order_t n_order;
  so3_storage_t storage;
  so3_n_mode_t n_mode;
  ssht_dl_method_t dl_method;
  int steerable;
} so3_parameters_t;

#define SO3_ERROR_GENERIC(comment)                                                             \
  {                                                                                            \
    printf("ERROR: %s.\n", comment);                                                           \
    exit(1);                                                                                   \
  }
#define SO3_ERROR_MEM_ALLOC_CHECK(pointer)                                                     \
  if ((pointer) == NULL) {                                                                     \
    SO3_ERROR_GENERIC("Memory allocation failed")                                              \
  }

void so3_sampling_elmn2ind(int *ind, int el, int m, int n, const so3_parameters_t *parameters);
void so3_sampling_elmn2ind_real(int *ind, int el, int m, int n,
                                const so3_parameters_t *parameters);
int so3_sampling_flmn_size(const so3_parameters_t *parameters);
int so3_sampling_f_size(const so3_parameters_t *parameters);
int so3_sampling_ngamma(const so3_parameters_t *parameters);
int so3_sampling_nalpha(const so3_parameters_t *parameters);
int so3_sampling_nbeta(const so3_parameters_t *parameters);

void so3_core_inverse_direct(complex double *f, const complex double *flmn,
                             const so3_parameters_t *parameters);
void so3_core_inverse_via_ssht(complex double *f, const complex double *flmn,
                               const so3_parameters_t *parameters);
void so3_core_forward_direct(complex double *flmn, const complex double *f,
                             const so3_parameters_t *parameters);
void so3_core_forward_via_ssht(complex double *flmn, const complex double *f,
                               const so3_parameters_t *parameters);
void so3_core_inverse_direct_real(double *f, const complex double *flmn,
                                  const so3_parameters_t *parameters);
void so3_core_inverse_via_ssht_real(double *f, const complex double *flmn,
                                    const so3_parameters_t *parameters);
void so3_core_forward_direct_real(complex double *flmn, const double *f,
                                  const so3_parameters_t *parameters);
void so3_core_forward_via_ssht_real(complex double *flmn, const double *f,
                                    const so3_parameters_t *parameters);

void so3_adjoint_inverse_direct(complex double *flmn, const complex double *f,
                                const so3_parameters_t *parameters);
void so3_adjoint_forward_direct(complex double *f, const complex double *flmn,
                                const so3_parameters_t *parameters);
void so3_adjoint_inverse_direct_real(complex double *flmn, const double *f,
                                     const so3_parameters_t *parameters);
void so3_adjoint_forward_direct_real(double *f, const complex double *flmn,
                                     const so3_parameters_t *parameters);

#ifdef __cplusplus
}
#endif
#endif
