/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * The subset of the SSHT C API (spin spherical-harmonic transforms on
 * McEwen-Wiaux sampling) that the reference S2LET sources call.  SSHT is an
 * external dependency of the reference (conanfile.txt:3 pins ssht >= 1.5.2) and
 * is not present in the reference tree; the names and argument orders below are
 * those used at the reference call sites (e.g. src/c/s2let_analysis.c:324,471,
 * src/c/s2let_analysis_adjoint.c:336,506, src/c/s2let_synthesis.c:335,489).
 * The implementations (oracle/ssht_so3/ssht.c) are written from the published
 * MW sampling theorem (McEwen & Wiaux 2011), not from SSHT's source.
 *
 * Conventions:
 *   sY_lm(theta,phi) = (-1)^s sqrt((2l+1)/4pi) e^{i m phi} d^l_{m,-s}(theta)
 *   (Condon-Shortley phase), theta_t = pi(2t+1)/(2L-1), phi_p = 2 pi p/(2L-1),
 *   map index t*(2L-1)+p, harmonic index l^2+l+m (MW; MWSS further below).
 */
#ifndef ORACLE_SSHT_H
#define ORACLE_SSHT_H

#include <complex.h>
#include <stdio.h>
#include <stdlib.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum { SSHT_DL_RISBO = 0, SSHT_DL_TRAPANI = 1 } ssht_dl_method_t;

static inline void ssht_sampling_elm2ind(int *ind, int el, int m) { *ind = el * el + el + m; }
static inline void ssht_sampling_ind2elm(int *el, int *m, int ind) {
  int l = 0;
  while ((l + 1) * (l + 1) <= ind) ++l;
  *el = l;
  *m = ind - l * l - l;
}
static inline int ssht_sampling_mw_ntheta(int L) { return L; }
static inline int ssht_sampling_mw_nphi(int L) { return 2 * L - 1; }
static inline int ssht_sampling_mw_ss_ntheta(int L) { return L + 1; }
static inline int ssht_sampling_mw_ss_nphi(int L) { return 2 * L; }

/* Forward (pixels -> flm), exact for band-limited signals. */
void ssht_core_mw_forward_sov_conv_sym(complex double *flm, const complex double *f, int L,
                                       int spin, ssht_dl_method_t dl_method, int verbosity);
void ssht_core_mw_forward_sov_conv_sym_real(complex double *flm, const double *f, int L,
                                            ssht_dl_method_t dl_method, int verbosity);
/* Inverse (flm -> pixels). */
void ssht_core_mw_inverse_sov_sym(complex double *f, const complex double *flm, int L, int spin,
                                  ssht_dl_method_t dl_method, int verbosity);
void ssht_core_mw_inverse_sov_sym_real(double *f, const complex double *flm, int L,
                                       ssht_dl_method_t dl_method, int verbosity);
/* Adjoint of the inverse (pixels -> flm) and of the forward (flm -> pixels). */
void ssht_adjoint_mw_inverse_sov_sym(complex double *flm, const complex double *f, int L,
                                     int spin, ssht_dl_method_t dl_method, int verbosity);
void ssht_adjoint_mw_inverse_sov_sym_real(complex double *flm, const double *f, int L,
                                          ssht_dl_method_t dl_method, int verbosity);
void ssht_adjoint_mw_forward_sov_sym(complex double *f, const complex double *flm, int L,
                                     int spin, ssht_dl_method_t dl_method, int verbosity);
void ssht_adjoint_mw_forward_sov_sym_real(double *f, const complex double *flm, int L,
                                          ssht_dl_method_t dl_method, int verbosity);

/* MW symmetric sampling (MWSS): theta_t = pi t/L, t = 0..L (both poles),
 * phi_p = 2 pi p/(2L), map index t*2L+p. */
void ssht_core_mw_forward_sov_conv_sym_ss(complex double *flm, const complex double *f, int L,
                                          int spin, ssht_dl_method_t dl_method, int verbosity);
void ssht_core_mw_forward_sov_conv_sym_ss_real(complex double *flm, const double *f, int L,
                                               ssht_dl_method_t dl_method, int verbosity);
void ssht_core_mw_inverse_sov_sym_ss(complex double *f, const complex double *flm, int L,
                                     int spin, ssht_dl_method_t dl_method, int verbosity);
void ssht_core_mw_inverse_sov_sym_ss_real(double *f, const complex double *flm, int L,
                                          ssht_dl_method_t dl_method, int verbosity);
void ssht_adjoint_mw_inverse_sov_sym_ss(complex double *flm, const complex double *f, int L,
                                        int spin, ssht_dl_method_t dl_method, int verbosity);
void ssht_adjoint_mw_inverse_sov_sym_ss_real(complex double *flm, const double *f, int L,
                                             ssht_dl_method_t dl_method, int verbosity);
void ssht_adjoint_mw_forward_sov_sym_ss(complex double *f, const complex double *flm, int L,
                                        int spin, ssht_dl_method_t dl_method, int verbosity);
void ssht_adjoint_mw_forward_sov_sym_ss_real(double *f, const complex double *flm, int L,
                                             ssht_dl_method_t dl_method, int verbosity);

/* Wigner d at pi/2 for one l: D[mp*(l+1)+m] = d^l_{mp,m}(pi/2), 0 <= mp,m <= l. */
void oracle_delta_quadrant(double *D, int l);
/* Wigner d^l_{mn}(theta) for l = max(|m|,|n|)..L-1 by three-term recursion in l. */
void oracle_wigner_d_column(double *out, int L, int m, int n, double theta);

#ifdef __cplusplus
}
#endif
#endif
