/*
 * s2let_gpu.h — C ABI of libs2let_gpu.so, a GB300 (sm_103a) implementation of
 * S2LET's scale-discretised wavelet transforms on McEwen–Wiaux sampling (MW
 * and its symmetric variant MWSS).
 *
 * Drop-in boundary.  Every s2let_* function below has the name, argument list,
 * argument meaning and coefficient layout of the reference C API
 * (the include/s2let headers of S2LET 2.2.7), so that a caller of the reference relinks
 * against this library unchanged.  Each declaration cites the reference
 * declaration it replaces.  Buffers are HOST memory, allocated by the caller
 * (e.g. with the s2let_allocate_* helpers); complex arrays are interleaved
 * (re, im) doubles, as C99 `double complex` and C++ `std::complex<double>` lay
 * them out.  Calls are synchronous.
 *
 * Errors.  The reference prints and calls exit(1) on an invalid sampling scheme
 * (include/s2let/s2let_error.h:13-27) and validates nothing else.  This library
 * never exits the host process: an invalid argument or a CUDA failure leaves
 * the outputs untouched, records a status readable with s2let_gpu_last_error()
 * / s2let_gpu_last_error_string(), and prints one line to stderr.  Setting the
 * environment variable S2LET_GPU_ABORT_ON_ERROR=1 restores the reference's
 * exit(1) behaviour.
 *
 * Sampling.  The directional transforms (px2wav / wav2px, lm2wav / wav2lm and
 * their adjoints) follow parameters->sampling_scheme as the reference does:
 * S2LET_SAMPLING_MW (L rings of 2L-1 samples) or S2LET_SAMPLING_MW_SS (L+1
 * rings of 2L samples, both poles), for the signal, the scaling map and the
 * SO3 wavelet maps alike.  Any other value is S2LET_GPU_ERR_UNSUPPORTED (the
 * reference's "Sampling scheme not supported.").  The axisymmetric pixel-space
 * transforms, the manual-tiling entry points and s2let_mw_* use MW whatever the
 * parameters say, as in the reference.
 *
 * Extensions (no reference counterpart) are prefixed s2let_gpu_: precision
 * selection, device-pointer batched entry points on a caller stream, and the
 * status query.
 */
#ifndef S2LET_GPU_H
#define S2LET_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
#include <complex>
#define S2LET_COMPLEX(TYPE) std::complex<TYPE>
extern "C" {
#else
#include <complex.h>
#define S2LET_COMPLEX(TYPE) TYPE complex
#endif

/* ------------------------------------------------------------------------ */
/* Types (layout identical to include/s2let/s2let_types.h:18-137)           */
/* ------------------------------------------------------------------------ */

/* Wigner recursion selector of SSHT; accepted and ignored (results are the
 * same linear map either way).  Where SSHT's own header is installed it
 * provides the type, as in the reference's headers; otherwise an int-sized
 * enum of the same values is declared here.  Define S2LET_GPU_NO_SSHT_TYPES
 * to supply the type yourself. */
#if !defined(S2LET_GPU_NO_SSHT_TYPES) && defined(__has_include)
#if __has_include(<ssht/ssht.h>)
#include <ssht/ssht.h>
#define S2LET_GPU_NO_SSHT_TYPES
#endif
#endif
#ifndef S2LET_GPU_NO_SSHT_TYPES
typedef enum { SSHT_DL_RISBO = 0, SSHT_DL_TRAPANI = 1 } ssht_dl_method_t;
#endif

/* include/s2let/s2let_types.h:18-38 */
typedef enum {
  S2LET_SAMPLING_MW,
  S2LET_SAMPLING_MW_SS,
  S2LET_SAMPLING_SIZE
} s2let_sampling_t;

/* include/s2let/s2let_types.h:56-137 — field order and types must not change. */
typedef struct {
  int verbosity;
  int reality;
  int upsample;
  double B;
  int L;
  int J_min;
  int N;
  int spin;
  int original_spin;
  s2let_sampling_t sampling_scheme;
  ssht_dl_method_t dl_method;
} s2let_parameters_t;

/* ------------------------------------------------------------------------ */
/* Tiling (host FP64; src/c/s2let_tiling.c)                                 */
/* ------------------------------------------------------------------------ */

void s2let_switch_wavtype(int typenum);                                   /* s2let_tiling.h:14 */
int s2let_bandlimit(int j, const s2let_parameters_t *parameters);          /* s2let_tiling.h:16 */
int s2let_L0(int j, const s2let_parameters_t *parameters);                 /* s2let_tiling.h:18 */
int s2let_j_max(const s2let_parameters_t *parameters);                     /* s2let_tiling.h:20 */
void s2let_tiling_axisym_allocate(double **kappa, double **kappa0,
                                  const s2let_parameters_t *parameters);    /* s2let_tiling.h:22 */
void s2let_tiling_axisym(double *kappa, double *kappa0,
                         const s2let_parameters_t *parameters);             /* s2let_tiling.h:24 */
void s2let_tiling_direction_allocate(S2LET_COMPLEX(double) **s_elm,
                                     const s2let_parameters_t *parameters); /* s2let_tiling.h:26 */
void s2let_tiling_direction(S2LET_COMPLEX(double) *s_elm,
                            const s2let_parameters_t *parameters);          /* s2let_tiling.h:28 */
void s2let_tiling_wavelet_allocate(S2LET_COMPLEX(double) **psi, double **phi,
                                   const s2let_parameters_t *parameters);   /* s2let_tiling.h:30 */
void s2let_tiling_wavelet(S2LET_COMPLEX(double) *psi, double *phi,
                          const s2let_parameters_t *parameters);            /* s2let_tiling.h:32 */
double s2let_tiling_axisym_check_identity(double *kappa, double *kappa0,
                                          const s2let_parameters_t *parameters);  /* s2let_tiling.h:34 */
double s2let_tiling_direction_check_identity(S2LET_COMPLEX(double) *s_elm,
                                             const s2let_parameters_t *parameters); /* s2let_tiling.h:36 */
double s2let_tiling_wavelet_check_identity(S2LET_COMPLEX(double) *psi, double *phi,
                                           const s2let_parameters_t *parameters);   /* s2let_tiling.h:38 */

/* math helpers (include/s2let/s2let_math.h) */
double s2let_math_kappa0_quadtrap_s2dw(double a, double b, int n, double B);
double s2let_math_kappa0_quadtrap_needlet(double a, double b, int n);
double s2let_math_spline_scalingfct(double x, double y);
unsigned long binomial_coefficient(int n, int k, int exact);

/* ------------------------------------------------------------------------ */
/* Sizes and allocation (src/c/s2let_helper.c, src/c/s2let_alloc.c)        */
/* ------------------------------------------------------------------------ */

int s2let_n_phi(const s2let_parameters_t *parameters);      /* s2let_helper.h:8  */
int s2let_n_theta(const s2let_parameters_t *parameters);    /* s2let_helper.h:9  */
int s2let_n_px(const s2let_parameters_t *parameters);       /* s2let_helper.h:10 */
int s2let_n_lm(const s2let_parameters_t *parameters);       /* s2let_helper.h:12 */
int s2let_n_lm_scal(const s2let_parameters_t *parameters);  /* s2let_helper.h:14 */
int s2let_n_lmn_wav(const s2let_parameters_t *parameters);  /* s2let_helper.h:15 */
int s2let_n_gamma(const s2let_parameters_t *parameters);    /* s2let_helper.h:17 */
int s2let_n_scal(const s2let_parameters_t *parameters);     /* s2let_helper.h:18 */
int s2let_n_wav(const s2let_parameters_t *parameters);      /* s2let_helper.h:19 */
int s2let_n_wav_j(int j, const s2let_parameters_t *parameters); /* s2let_helper.h:21 */

void s2let_allocate_mw(S2LET_COMPLEX(double) **f, int L);              /* s2let_alloc.h:16 */
void s2let_allocate_mw_real(double **f, int L);                        /* s2let_alloc.h:17 */
void s2let_allocate_mwss(S2LET_COMPLEX(double) **f, int L);            /* s2let_alloc.h:19 */
void s2let_allocate_mwss_real(double **f, int L);                      /* s2let_alloc.h:20 */
void s2let_allocate_lm(S2LET_COMPLEX(double) **flm, int L);            /* s2let_alloc.h:24 */
void s2let_allocate_lmn_f_wav(S2LET_COMPLEX(double) **f_wav_lmn, S2LET_COMPLEX(double) **f_scal_lm,
                              const s2let_parameters_t *parameters);   /* s2let_alloc.h:28 */
void s2let_allocate_f_wav(S2LET_COMPLEX(double) **f_wav, S2LET_COMPLEX(double) **f_scal,
                          const s2let_parameters_t *parameters);       /* s2let_alloc.h:35 */
void s2let_allocate_f_wav_real(double **f_wav, double **f_scal,
                               const s2let_parameters_t *parameters);  /* s2let_alloc.h:40 */
void s2let_allocate_f_wav_manual(S2LET_COMPLEX(double) **f_wav, S2LET_COMPLEX(double) **f_scal,
                                 int *wav_bandlimits, int scal_bandlimit, int N, int J,
                                 const s2let_parameters_t *parameters); /* s2let_alloc.h:45 */

/* ------------------------------------------------------------------------ */
/* Directional analysis (src/c/s2let_analysis.c; s2let_analysis.h:16-77)   */
/* ------------------------------------------------------------------------ */

void s2let_analysis_lm2lmn(S2LET_COMPLEX(double) *f_wav_lmn, S2LET_COMPLEX(double) *f_scal_lm,
                           const S2LET_COMPLEX(double) *flm, const S2LET_COMPLEX(double) *wav_lm,
                           const double *scal_l, const s2let_parameters_t *parameters); /* s2let_analysis.h:16 */
void s2let_analysis_lm2lmn_real(S2LET_COMPLEX(double) *f_wav_lmn, S2LET_COMPLEX(double) *f_scal_lm,
                                const S2LET_COMPLEX(double) *flm, const S2LET_COMPLEX(double) *wav_lm,
                                const double *scal_l, const s2let_parameters_t *parameters); /* s2let_analysis.h:26 */
void s2let_analysis_lm2wav_manual(S2LET_COMPLEX(double) *f_wav, S2LET_COMPLEX(double) *f_scal,
                                  const S2LET_COMPLEX(double) *flm, const double *scal_l,
                                  const S2LET_COMPLEX(double) *wav_lm, const int scal_bandlimit,
                                  const int *wav_bandlimits, int J, int L, int spin, int N); /* s2let_analysis.h:36 */
void s2let_analysis_lm2wav(S2LET_COMPLEX(double) *f_wav, S2LET_COMPLEX(double) *f_scal,
                           const S2LET_COMPLEX(double) *flm,
                           const s2let_parameters_t *parameters);                /* s2let_analysis.h:49 */
void s2let_analysis_lm2wav_real(double *f_wav, double *f_scal, const S2LET_COMPLEX(double) *flm,
                                const s2let_parameters_t *parameters);           /* s2let_analysis.h:57 */
void s2let_analysis_px2wav(S2LET_COMPLEX(double) *f_wav, S2LET_COMPLEX(double) *f_scal,
                           const S2LET_COMPLEX(double) *f,
                           const s2let_parameters_t *parameters);                /* s2let_analysis.h:65 */
void s2let_analysis_px2wav_real(double *f_wav, double *f_scal, const double *f,
                                const s2let_parameters_t *parameters);           /* s2let_analysis.h:73 */

/* ------------------------------------------------------------------------ */
/* Directional synthesis (src/c/s2let_synthesis.c; s2let_synthesis.h:16-77) */
/* ------------------------------------------------------------------------ */

void s2let_synthesis_lmn2lm(S2LET_COMPLEX(double) *flm, const S2LET_COMPLEX(double) *f_wav_lmn,
                            const S2LET_COMPLEX(double) *f_scal_lm, const S2LET_COMPLEX(double) *wav_lm,
                            const double *scal_l, const s2let_parameters_t *parameters); /* s2let_synthesis.h:16 */
void s2let_synthesis_lmn2lm_real(S2LET_COMPLEX(double) *flm, const S2LET_COMPLEX(double) *f_wav_lmn,
                                 const S2LET_COMPLEX(double) *f_scal_lm,
                                 const S2LET_COMPLEX(double) *wav_lm, const double *scal_l,
                                 const s2let_parameters_t *parameters);          /* s2let_synthesis.h:26 */
void s2let_synthesis_wav2lm_manual(S2LET_COMPLEX(double) *flm, const S2LET_COMPLEX(double) *f_wav,
                                   const S2LET_COMPLEX(double) *f_scal, const double *scal_l,
                                   const S2LET_COMPLEX(double) *wav_lm, const int scal_bandlimit,
                                   const int *wav_bandlimits, int J, int L, int spin, int N); /* s2let_synthesis.h:36 */
void s2let_synthesis_wav2lm(S2LET_COMPLEX(double) *flm, const S2LET_COMPLEX(double) *f_wav,
                            const S2LET_COMPLEX(double) *f_scal,
                            const s2let_parameters_t *parameters);               /* s2let_synthesis.h:49 */
void s2let_synthesis_wav2lm_real(S2LET_COMPLEX(double) *flm, const double *f_wav,
                                 const double *f_scal, const s2let_parameters_t *parameters); /* s2let_synthesis.h:57 */
void s2let_synthesis_wav2px(S2LET_COMPLEX(double) *f, const S2LET_COMPLEX(double) *f_wav,
                            const S2LET_COMPLEX(double) *f_scal,
                            const s2let_parameters_t *parameters);               /* s2let_synthesis.h:65 */
void s2let_synthesis_wav2px_real(double *f, const double *f_wav, const double *f_scal,
                                 const s2let_parameters_t *parameters);          /* s2let_synthesis.h:73 */

/* ------------------------------------------------------------------------ */
/* Adjoints (src/c/s2let_analysis_adjoint.c, src/c/s2let_synthesis_adjoint.c) */
/* ------------------------------------------------------------------------ */

void s2let_analysis_adjoint_lmn2lm(S2LET_COMPLEX(double) *flm, const S2LET_COMPLEX(double) *f_wav_lmn,
                                   const S2LET_COMPLEX(double) *f_scal_lm,
                                   const S2LET_COMPLEX(double) *wav_lm, const double *scal_l,
                                   const s2let_parameters_t *parameters);        /* s2let_analysis_adjoint.h:31 */
void s2let_analysis_adjoint_lmn2lm_real(S2LET_COMPLEX(double) *flm,
                                        const S2LET_COMPLEX(double) *f_wav_lmn,
                                        const S2LET_COMPLEX(double) *f_scal_lm,
                                        const S2LET_COMPLEX(double) *wav_lm, const double *scal_l,
                                        const s2let_parameters_t *parameters);   /* s2let_analysis_adjoint.h:58 */
void s2let_analysis_adjoint_wav2lm_manual(S2LET_COMPLEX(double) *flm, const S2LET_COMPLEX(double) *f_wav,
                                          const S2LET_COMPLEX(double) *f_scal, const double *scal_l,
                                          const S2LET_COMPLEX(double) *wav_lm,
                                          const int scal_bandlimit, const int *wav_bandlimits,
                                          int J, int L, int spin, int N);        /* s2let_analysis_adjoint.h:96 */
void s2let_analysis_adjoint_wav2lm(S2LET_COMPLEX(double) *flm, const S2LET_COMPLEX(double) *f_wav,
                                   const S2LET_COMPLEX(double) *f_scal,
                                   const s2let_parameters_t *parameters);        /* s2let_analysis_adjoint.h:125 */
void s2let_analysis_adjoint_wav2lm_real(S2LET_COMPLEX(double) *flm, const double *f_wav,
                                        const double *f_scal,
                                        const s2let_parameters_t *parameters);   /* s2let_analysis_adjoint.h:147 */
void s2let_analysis_adjoint_wav2px(S2LET_COMPLEX(double) *f, const S2LET_COMPLEX(double) *f_wav,
                                   const S2LET_COMPLEX(double) *f_scal,
                                   const s2let_parameters_t *parameters);        /* s2let_analysis_adjoint.h:168 */
void s2let_analysis_adjoint_wav2px_real(double *f, const double *f_wav, const double *f_scal,
                                        const s2let_parameters_t *parameters);   /* s2let_analysis_adjoint.h:188 */

void s2let_synthesis_adjoint_lm2lmn(S2LET_COMPLEX(double) *f_wav_lmn, S2LET_COMPLEX(double) *f_scal_lm,
                                    const S2LET_COMPLEX(double) *flm,
                                    const S2LET_COMPLEX(double) *wav_lm, const double *scal_l,
                                    const s2let_parameters_t *parameters);       /* s2let_synthesis_adjoint.h:29 */
void s2let_synthesis_adjoint_lm2lmn_real(S2LET_COMPLEX(double) *f_wav_lmn,
                                         S2LET_COMPLEX(double) *f_scal_lm,
                                         const S2LET_COMPLEX(double) *flm,
                                         const S2LET_COMPLEX(double) *wav_lm, const double *scal_l,
                                         const s2let_parameters_t *parameters);  /* s2let_synthesis_adjoint.h:56 */
void s2let_synthesis_adjoint_lm2wav_manual(S2LET_COMPLEX(double) *f_wav, S2LET_COMPLEX(double) *f_scal,
                                           const S2LET_COMPLEX(double) *flm, const double *scal_l,
                                           const S2LET_COMPLEX(double) *wav_lm,
                                           const int scal_bandlimit, const int *wav_bandlimits,
                                           int J, int L, int spin, int N);       /* s2let_synthesis_adjoint.h:94 */
void s2let_synthesis_adjoint_lm2wav(S2LET_COMPLEX(double) *f_wav, S2LET_COMPLEX(double) *f_scal,
                                    const S2LET_COMPLEX(double) *flm,
                                    const s2let_parameters_t *parameters);       /* s2let_synthesis_adjoint.h:124 */
void s2let_synthesis_adjoint_lm2wav_real(double *f_wav, double *f_scal,
                                         const S2LET_COMPLEX(double) *flm,
                                         const s2let_parameters_t *parameters);  /* s2let_synthesis_adjoint.h:147 */
void s2let_synthesis_adjoint_px2wav(S2LET_COMPLEX(double) *f_wav, S2LET_COMPLEX(double) *f_scal,
                                    const S2LET_COMPLEX(double) *f,
                                    const s2let_parameters_t *parameters);       /* s2let_synthesis_adjoint.h:170 */
void s2let_synthesis_adjoint_px2wav_real(double *f_wav, double *f_scal, const double *f,
                                         const s2let_parameters_t *parameters);  /* s2let_synthesis_adjoint.h:193 */

/* ------------------------------------------------------------------------ */
/* Axisymmetric wavelets (src/c/s2let_transform_axisym_lm.c, _mw.c)         */
/* ------------------------------------------------------------------------ */

void s2let_transform_axisym_lm_allocate_f_wav(S2LET_COMPLEX(double) **f_wav_lm,
                                              S2LET_COMPLEX(double) **f_scal_lm,
                                              const s2let_parameters_t *parameters); /* s2let_transform_axisym_lm.h:14 */
void s2let_transform_axisym_lm_allocate_f_wav_multires(S2LET_COMPLEX(double) **f_wav_lm,
                                                       S2LET_COMPLEX(double) **f_scal_lm,
                                                       const s2let_parameters_t *parameters); /* s2let_transform_axisym_lm.h:19 */
void s2let_transform_axisym_lm_allocate_wav(double **wav_lm, double **scal_lm,
                                            const s2let_parameters_t *parameters); /* s2let_transform_axisym_lm.h:24 */
void s2let_transform_axisym_lm_wav(double *wav_lm, double *scal_lm,
                                   const s2let_parameters_t *parameters);          /* s2let_transform_axisym_lm.h:25 */
void s2let_transform_axisym_lm_wav_analysis(S2LET_COMPLEX(double) *f_wav_lm,
                                            S2LET_COMPLEX(double) *f_scal_lm,
                                            const S2LET_COMPLEX(double) *flm, const double *wav_lm,
                                            const double *scal_lm,
                                            const s2let_parameters_t *parameters);   /* s2let_transform_axisym_lm.h:27 */
void s2let_transform_axisym_lm_wav_synthesis(S2LET_COMPLEX(double) *flm,
                                             const S2LET_COMPLEX(double) *f_wav_lm,
                                             const S2LET_COMPLEX(double) *f_scal_lm,
                                             const double *wav_lm, const double *scal_lm,
                                             const s2let_parameters_t *parameters);  /* s2let_transform_axisym_lm.h:34 */
void s2let_transform_axisym_lm_wav_analysis_multires(S2LET_COMPLEX(double) *f_wav_lm,
                                                     S2LET_COMPLEX(double) *f_scal_lm,
                                                     const S2LET_COMPLEX(double) *flm,
                                                     const double *wav_lm, const double *scal_lm,
                                                     const s2let_parameters_t *parameters); /* s2let_transform_axisym_lm.h:42 */
void s2let_transform_axisym_lm_wav_synthesis_multires(S2LET_COMPLEX(double) *flm,
                                                      const S2LET_COMPLEX(double) *f_wav_lm,
                                                      const S2LET_COMPLEX(double) *f_scal_lm,
                                                      const double *wav_lm, const double *scal_lm,
                                                      const s2let_parameters_t *parameters); /* s2let_transform_axisym_lm.h:49 */

void s2let_transform_axisym_allocate_mw_f_wav(S2LET_COMPLEX(double) **f_wav, S2LET_COMPLEX(double) **f_scal,
                                              const s2let_parameters_t *parameters); /* s2let_transform_axisym_mw.h:13 */
void s2let_transform_axisym_allocate_mw_f_wav_multires(S2LET_COMPLEX(double) **f_wav,
                                                       S2LET_COMPLEX(double) **f_scal,
                                                       const s2let_parameters_t *parameters); /* s2let_transform_axisym_mw.h:14 */
void s2let_transform_axisym_allocate_mw_f_wav_real(double **f_wav, double **f_scal,
                                                   const s2let_parameters_t *parameters); /* s2let_transform_axisym_mw.h:15 */
void s2let_transform_axisym_allocate_mw_f_wav_multires_real(double **f_wav, double **f_scal,
                                                            const s2let_parameters_t *parameters); /* s2let_transform_axisym_mw.h:16 */
void s2let_transform_axisym_wav_analysis_mw(S2LET_COMPLEX(double) *f_wav, S2LET_COMPLEX(double) *f_scal,
                                            const S2LET_COMPLEX(double) *f,
                                            const s2let_parameters_t *parameters); /* s2let_transform_axisym_mw.h:18 */
void s2let_transform_axisym_wav_analysis_adjoint_mw(S2LET_COMPLEX(double) *f,
                                                    const S2LET_COMPLEX(double) *f_wav,
                                                    const S2LET_COMPLEX(double) *f_scal,
                                                    const s2let_parameters_t *parameters); /* s2let_transform_axisym_mw.h:19 */
void s2let_transform_axisym_wav_synthesis_mw(S2LET_COMPLEX(double) *f, const S2LET_COMPLEX(double) *f_wav,
                                             const S2LET_COMPLEX(double) *f_scal,
                                             const s2let_parameters_t *parameters); /* s2let_transform_axisym_mw.h:20 */
void s2let_transform_axisym_wav_synthesis_adjoint_mw(S2LET_COMPLEX(double) *f_wav,
                                                     S2LET_COMPLEX(double) *f_scal,
                                                     const S2LET_COMPLEX(double) *f,
                                                     const s2let_parameters_t *parameters); /* s2let_transform_axisym_mw.h:21 */
void s2let_transform_axisym_wav_analysis_mw_multires(S2LET_COMPLEX(double) *f_wav,
                                                     S2LET_COMPLEX(double) *f_scal,
                                                     const S2LET_COMPLEX(double) *f,
                                                     const s2let_parameters_t *parameters); /* s2let_transform_axisym_mw.h:23 */
void s2let_transform_axisym_wav_analysis_adjoint_mw_multires(S2LET_COMPLEX(double) *f,
                                                             const S2LET_COMPLEX(double) *f_wav,
                                                             const S2LET_COMPLEX(double) *f_scal,
                                                             const s2let_parameters_t *parameters); /* s2let_transform_axisym_mw.h:24 */
void s2let_transform_axisym_wav_synthesis_mw_multires(S2LET_COMPLEX(double) *f,
                                                      const S2LET_COMPLEX(double) *f_wav,
                                                      const S2LET_COMPLEX(double) *f_scal,
                                                      const s2let_parameters_t *parameters); /* s2let_transform_axisym_mw.h:25 */
void s2let_transform_axisym_wav_synthesis_adjoint_mw_multires(S2LET_COMPLEX(double) *f_wav,
                                                              S2LET_COMPLEX(double) *f_scal,
                                                              const S2LET_COMPLEX(double) *f,
                                                              const s2let_parameters_t *parameters); /* s2let_transform_axisym_mw.h:26 */
void s2let_transform_axisym_wav_analysis_mw_real(double *f_wav, double *f_scal, const double *f,
                                                 const s2let_parameters_t *parameters); /* s2let_transform_axisym_mw.h:28 */
void s2let_transform_axisym_wav_analysis_adjoint_mw_real(double *f, const double *f_wav,
                                                         const double *f_scal,
                                                         const s2let_parameters_t *parameters); /* s2let_transform_axisym_mw.h:29 */
void s2let_transform_axisym_wav_synthesis_mw_real(double *f, const double *f_wav, const double *f_scal,
                                                  const s2let_parameters_t *parameters); /* s2let_transform_axisym_mw.h:30 */
void s2let_transform_axisym_wav_synthesis_adjoint_mw_real(double *f_wav, double *f_scal, const double *f,
                                                          const s2let_parameters_t *parameters); /* s2let_transform_axisym_mw.h:31 */
void s2let_transform_axisym_wav_analysis_mw_multires_real(double *f_wav, double *f_scal,
                                                          const double *f,
                                                          const s2let_parameters_t *parameters); /* s2let_transform_axisym_mw.h:33 */
void s2let_transform_axisym_wav_analysis_adjoint_mw_multires_real(double *f, const double *f_wav,
                                                                  const double *f_scal,
                                                                  const s2let_parameters_t *parameters); /* s2let_transform_axisym_mw.h:34 */
void s2let_transform_axisym_wav_synthesis_mw_multires_real(double *f, const double *f_wav,
                                                           const double *f_scal,
                                                           const s2let_parameters_t *parameters); /* s2let_transform_axisym_mw.h:35 */
void s2let_transform_axisym_wav_synthesis_adjoint_mw_multires_real(double *f_wav, double *f_scal,
                                                                   const double *f,
                                                                   const s2let_parameters_t *parameters); /* s2let_transform_axisym_mw.h:36 */
void s2let_transform_axisym_wav_hardthreshold_real(double *g_wav, const double *threshold,
                                                   const s2let_parameters_t *parameters); /* s2let_transform_axisym_mw.h:38 */
void s2let_transform_axisym_wav_hardthreshold_multires_real(double *g_wav, const double *threshold,
                                                            const s2let_parameters_t *parameters); /* s2let_transform_axisym_mw.h:39 */
/* No counterpart in the reference.  The hard threshold above (multires = 0:
 * _real, 1: _multires_real) with no device allocation: staging lives in one
 * 8 MiB static device array shared by every call, so calls that overlap on the
 * GPU (two host threads at once) race.  Requests above 8 MiB (maps + 2 x 256 B
 * of scale tables) return S2LET_GPU_ERR_INVALID.  Returns the status. */
int s2let_gpu_axisym_wav_hardthreshold_real_noalloc(double *g_wav, const double *threshold,
                                                    const s2let_parameters_t *parameters, int multires);

/* ------------------------------------------------------------------------ */
/* Plain MW spherical-harmonic transforms (src/c/s2let_mw.c; s2let_mw.h)    */
/* ------------------------------------------------------------------------ */

void s2let_mw_map2alm_real(S2LET_COMPLEX(double) *flm, const double *f, int L);          /* s2let_mw.h:15 */
void s2let_mw_alm2map_real(double *f, const S2LET_COMPLEX(double) *flm, int L);          /* s2let_mw.h:16 */
void s2let_mw_alm2map(S2LET_COMPLEX(double) *f, const S2LET_COMPLEX(double) *flm, int L, int spin); /* s2let_mw.h:17 */
void s2let_mw_map2alm(S2LET_COMPLEX(double) *flm, const S2LET_COMPLEX(double) *f, int L, int spin); /* s2let_mw.h:18 */
double s2let_mw_power(S2LET_COMPLEX(double) *flm, int L);                                /* s2let_mw.h:21 */
double s2let_mw_power_real(double *flm, int L);                                          /* s2let_mw.h:22 */
double s2let_lm_power(S2LET_COMPLEX(double) *flm, int L);                                /* s2let_lm.h:14 */

/* ------------------------------------------------------------------------ */
/* FITS I/O of MW / MWSS maps (src/c/s2let_fits.c; s2let_fits.h), host code   */
/* without cfitsio: an empty primary HDU and one binary table BINTABLE with    */
/* the map column(s) and the keyword L (and MWSS = 1).  Readers accept 8-byte */
/* (D) or 4-byte (E) float columns.  Writers refuse an existing file unless   */
/* its name starts with '!', as cfitsio does.  Errors set the status.         */
/* ------------------------------------------------------------------------ */
int s2let_fits_hpx_read_nside(char *filename);                                            /* s2let_fits.h:18 */
int s2let_fits_mw_read_bandlimit(char *filename);                                         /* s2let_fits.h:26 */
void s2let_fits_mw_read_map(double *f, char *file, int L);                                /* s2let_fits.h:36 */
void s2let_fits_mwss_read_map(double *f, char *file, int L);                              /* s2let_fits.h:46 */
void s2let_fits_mw_write_map(char *file, double *f, int L);                               /* s2let_fits.h:56 */
void s2let_fits_mwss_write_map(char *file, double *f, int L);                             /* s2let_fits.h:66 */
void s2let_fits_mw_read_spin_maps(double *fQ, double *fU, char *file, int L);             /* s2let_fits.h:76 */
void s2let_fits_mwss_read_spin_maps(double *fQ, double *fU, char *file, int L);           /* s2let_fits.h:86 */
void s2let_fits_mw_write_spin_maps(char *file, double *fQ, double *fU, int L);            /* s2let_fits.h:96 */
void s2let_fits_mwss_write_spin_maps(char *file, double *fQ, double *fU, int L);          /* s2let_fits.h:106 */

/* ------------------------------------------------------------------------ */
/* GB300 extensions (no reference counterpart)                              */
/* ------------------------------------------------------------------------ */

enum {
  S2LET_GPU_OK = 0,
  S2LET_GPU_ERR_INVALID = 1,     /* bad parameter (L<1, N<1, B<=1, |spin|>=L, ...) */
  S2LET_GPU_ERR_UNSUPPORTED = 2, /* e.g. an unknown sampling scheme, more than 16 directions per scale */
  S2LET_GPU_ERR_CUDA = 3,        /* a CUDA runtime call failed */
  S2LET_GPU_ERR_NOMEM = 4,       /* device or host allocation failed */
  S2LET_GPU_ERR_NO_DEVICE = 5    /* no usable CUDA device */
};

/* Status of the last call made on this thread (0 = success). */
int s2let_gpu_last_error(void);
const char *s2let_gpu_last_error_string(void);

/* Arithmetic used by subsequent calls of this thread.
 *   0 = FP64 throughout (default);
 *   1 = split precision (within 1e-10 of the FP64 path): on stored Wigner
 *       tables the Legendre/Wigner contraction of batches of two maps or
 *       more runs on the tensor cores (bf16 digit slices, FP32 accumulation,
 *       FP64 combination); one-map calls (s2let_gpu_set_df_max_maps) and
 *       band-limits below 128 contract in double-float arithmetic on the FP32
 *       pipe; recomputed tables regenerate and contract in double-float; ring
 *       and gamma DFTs in double-float. */
int s2let_gpu_set_precision(int mode);
int s2let_gpu_get_precision(void);

/* Double-float copies of the stored Wigner tables for the double-float
 * contractions of the split-precision path (1 = default): built on first use,
 * the same size as the FP64 tables, skipped when they would leave less than
 * 4 GiB of device memory free; 0 = split the FP64 values as they are read
 * (slower, no extra memory).  Process-wide; copies are freed by
 * s2let_gpu_release_plans.  Returns the status. */
int s2let_gpu_set_split_tables(int on);
int s2let_gpu_get_split_tables(void);

/* Split precision on stored tables: batches of at most `maps` maps (0-4,
 * default 1, initially S2LET_GPU_DF_MAX_MAPS when set) contract in
 * double-float on the FP64 tables (8 bytes per table entry streamed, two
 * scales of one band-limit in one pass) instead of on the tensor cores (14
 * bytes per entry); 0 keeps every batch on the tensor cores.  Process-wide.
 * Returns the status. */
int s2let_gpu_set_df_max_maps(int maps);
int s2let_gpu_get_df_max_maps(void);

/* Wigner tables used by plans built afterwards on this thread.
 *   0 = auto (default): stored D and Q tables while a plan's tables fit 60 % of
 *       the free device memory (S2LET_GPU_TABLE_BUDGET_GB overrides), else the
 *       largest band-limits recomputed;
 *   1 = stored tables always;
 *   2 = recomputed always: the kernels regenerate the Wigner d values from
 *       double-double checkpoints every 64 degrees (≈ 1/50 of the memory) and
 *       apply the forward quadrature as a separate operator (FP64, or
 *       double-float at split precision).
 * Returns the status. */
int s2let_gpu_set_table_mode(int mode);
int s2let_gpu_get_table_mode(void);

/* Adjoints of the plain MW transforms (host buffers): the adjoint of
 * s2let_mw_map2alm maps flm to pixels, the adjoint of s2let_mw_alm2map maps
 * pixels to flm.  These are the SSHT adjoints the reference calls internally
 * (ssht_adjoint_mw_forward_sov_sym / ssht_adjoint_mw_inverse_sov_sym at
 * src/c/s2let_analysis_adjoint.c:506 and src/c/s2let_synthesis_adjoint.c:480). */
void s2let_gpu_mw_adjoint_map2alm(S2LET_COMPLEX(double) *f, const S2LET_COMPLEX(double) *flm, int L,
                                  int spin);
void s2let_gpu_mw_adjoint_alm2map(S2LET_COMPLEX(double) *flm, const S2LET_COMPLEX(double) *f, int L,
                                  int spin);

/* The SSHT transforms the wavelet transforms call, on either sampling (host
 * buffers; f is double* when real != 0, then spin must be 0):
 *   dir 0  forward, pixels -> flm    ssht_core_mw_forward_sov_conv_sym[_ss][_real]  (src/c/s2let_analysis.c:471-474)
 *   dir 1  inverse, flm -> pixels    ssht_core_mw_inverse_sov_sym[_ss][_real]       (src/c/s2let_synthesis.c:489-492)
 *   dir 2  adjoint of the forward    ssht_adjoint_mw_forward_sov_sym[_ss][_real]    (src/c/s2let_analysis_adjoint.c:505-509)
 *   dir 3  adjoint of the inverse    ssht_adjoint_mw_inverse_sov_sym[_ss][_real]    (src/c/s2let_synthesis_adjoint.c:479-483)
 * sampling_scheme: S2LET_SAMPLING_MW or S2LET_SAMPLING_MW_SS.  Returns the status. */
int s2let_gpu_sht(int dir, int sampling_scheme, int L, int spin, int real, void *f, void *flm);

/* Drops cached plans (Wigner tables, FFT chirps) and frees their device memory. */
void s2let_gpu_release_plans(void);
/* Bytes of device memory currently held by cached plans. */
size_t s2let_gpu_plan_bytes(void);

/* Heterogeneous batches: map k has its own parameters params[k] (band-limit,
 * N, spin, B, J_min, upsample, sampling) and reality real[k] (nonzero: a real
 * map, double buffers; else complex).  f[k], f_wav[k], f_scal[k] are DEVICE
 * pointers to one map's buffers of the reference's layout (s2let_n_px /
 * s2let_n_wav / s2let_n_scal of params[k]); work is enqueued on `stream`.
 * Maps with equal parameters run as one batch.  use_graph != 0 with a
 * non-default stream: the first call with a given set of parameters and
 * pointers runs eagerly and builds the plans, the second captures the whole
 * launch sequence into a CUDA graph, later calls replay the graph (one launch).
 * s2let_gpu_release_plans() drops the graphs.  Returns the status. */
int s2let_gpu_px2wav_multi(void *const *f_wav, void *const *f_scal, void *const *f,
                           const s2let_parameters_t *params, const int *real, int nmaps, int use_graph,
                           void *stream);
int s2let_gpu_wav2px_multi(void *const *f, void *const *f_wav, void *const *f_scal,
                           const s2let_parameters_t *params, const int *real, int nmaps, int use_graph,
                           void *stream);

/*
 * Host-pointer batches: the drop-in functions above for `nbatch` maps in one
 * call (HOST buffers, map b at b * s2let_n_px / s2let_n_wav / s2let_n_scal
 * elements, synchronous).  Up to 32 maps run as one device batch
 * (S2LET_GPU_HOST_PASS overrides), so the Wigner tables are streamed once for
 * all of them, and f_wav crosses the bus on a second stream in pieces (one
 * scale of a group of up to 8 maps) overlapped with the transforms: the
 * analysis copies each piece out as soon as it is written, largest scales
 * first; the synthesis starts each group's kernels as soon as its piece is in.
 * Returns the status.
 */
int s2let_gpu_analysis_px2wav_real_host_batch(double *f_wav, double *f_scal, const double *f, int nbatch,
                                              const s2let_parameters_t *parameters);
int s2let_gpu_synthesis_wav2px_real_host_batch(double *f, const double *f_wav, const double *f_scal,
                                               int nbatch, const s2let_parameters_t *parameters);
int s2let_gpu_analysis_px2wav_host_batch(void *f_wav, void *f_scal, const void *f, int nbatch,
                                         const s2let_parameters_t *parameters);
int s2let_gpu_synthesis_wav2px_host_batch(void *f, const void *f_wav, const void *f_scal, int nbatch,
                                          const s2let_parameters_t *parameters);

/*
 * Batched device-pointer entry points.  All pointers are DEVICE pointers; `stream`
 * is a cudaStream_t (NULL = default stream).  `nbatch` maps share one parameter
 * set; map b starts at b*stride of each array, strides being the single-map sizes
 * (s2let_n_px, s2let_n_wav, s2let_n_scal elements).  Asynchronous with respect to
 * the host; the status covers launch-time errors.  Real-signal layouts as the
 * _real host functions.
 */
int s2let_gpu_analysis_px2wav_real_batch(double *f_wav, double *f_scal, const double *f, int nbatch,
                                         const s2let_parameters_t *parameters, void *stream);
int s2let_gpu_synthesis_wav2px_real_batch(double *f, const double *f_wav, const double *f_scal,
                                          int nbatch, const s2let_parameters_t *parameters,
                                          void *stream);
int s2let_gpu_analysis_px2wav_batch(void *f_wav, void *f_scal, const void *f, int nbatch,
                                    const s2let_parameters_t *parameters, void *stream);
int s2let_gpu_synthesis_wav2px_batch(void *f, const void *f_wav, const void *f_scal, int nbatch,
                                     const s2let_parameters_t *parameters, void *stream);
/* Exact adjoints (backward of the autograd op), same conventions. */
int s2let_gpu_analysis_adjoint_wav2px_real_batch(double *f, const double *f_wav, const double *f_scal,
                                                 int nbatch, const s2let_parameters_t *parameters,
                                                 void *stream);
int s2let_gpu_synthesis_adjoint_px2wav_real_batch(double *f_wav, double *f_scal, const double *f,
                                                  int nbatch, const s2let_parameters_t *parameters,
                                                  void *stream);
int s2let_gpu_analysis_adjoint_wav2px_batch(void *f, const void *f_wav, const void *f_scal,
                                            int nbatch, const s2let_parameters_t *parameters,
                                            void *stream);
int s2let_gpu_synthesis_adjoint_px2wav_batch(void *f_wav, void *f_scal, const void *f, int nbatch,
                                             const s2let_parameters_t *parameters, void *stream);

/*
 * FP32 storage (configurations that keep maps and wavelet coefficients in
 * single precision).  The batched device-pointer entry points above with
 * `float` maps, f_wav and f_scal (complex signals as interleaved float
 * pairs), the same strides in elements.  Inputs are widened to FP64 on the
 * device, the transforms run as in the FP64-storage path at the precision set
 * by s2let_gpu_set_precision, and outputs are rounded to FP32 (so the results
 * are the FP64-storage results rounded, about 6e-8 relative).  Only the used
 * part of each f_wav row is read or written.  Device scratch: the FP64 copies
 * of the batch.  Asynchronous on `stream`; returns the status.  No counterpart
 * in the reference (its transforms take double arrays only).
 */
int s2let_gpu_analysis_px2wav_real_batch_f32(float *f_wav, float *f_scal, const float *f, int nbatch,
                                             const s2let_parameters_t *parameters, void *stream);
int s2let_gpu_synthesis_wav2px_real_batch_f32(float *f, const float *f_wav, const float *f_scal, int nbatch,
                                              const s2let_parameters_t *parameters, void *stream);
int s2let_gpu_analysis_px2wav_batch_f32(void *f_wav, void *f_scal, const void *f, int nbatch,
                                        const s2let_parameters_t *parameters, void *stream);
int s2let_gpu_synthesis_wav2px_batch_f32(void *f, const void *f_wav, const void *f_scal, int nbatch,
                                         const s2let_parameters_t *parameters, void *stream);
int s2let_gpu_analysis_adjoint_wav2px_real_batch_f32(float *f, const float *f_wav, const float *f_scal,
                                                     int nbatch, const s2let_parameters_t *parameters,
                                                     void *stream);
int s2let_gpu_synthesis_adjoint_px2wav_real_batch_f32(float *f_wav, float *f_scal, const float *f, int nbatch,
                                                      const s2let_parameters_t *parameters, void *stream);
int s2let_gpu_analysis_adjoint_wav2px_batch_f32(void *f, const void *f_wav, const void *f_scal, int nbatch,
                                                const s2let_parameters_t *parameters, void *stream);
int s2let_gpu_synthesis_adjoint_px2wav_batch_f32(void *f_wav, void *f_scal, const void *f, int nbatch,
                                                 const s2let_parameters_t *parameters, void *stream);
/* s2let_gpu_px2wav_multi / s2let_gpu_wav2px_multi with FP32 storage: every
 * map's f, f_wav and f_scal are float arrays (device pointers), widened into
 * FP64 batch scratch and rounded back, inside the CUDA graph when use_graph. */
int s2let_gpu_px2wav_multi_f32(void *const *f_wav, void *const *f_scal, void *const *f,
                               const s2let_parameters_t *params, const int *real, int nmaps, int use_graph,
                               void *stream);
int s2let_gpu_wav2px_multi_f32(void *const *f, void *const *f_wav, void *const *f_scal,
                               const s2let_parameters_t *params, const int *real, int nmaps, int use_graph,
                               void *stream);

/* Reads and clears the device-side fault flag of the split-precision
 * tensor-core contraction: non-zero when one of its bounded waits expired since
 * the last call (the affected outputs are invalid).  0 when all went well. */
int s2let_gpu_device_fault(void);

/* One device per process.  Plans, Wigner tables, streams and kernel
 * attributes are cached for the device that was current at the first compute
 * call of the process; every later call made while another device is current
 * fails with S2LET_GPU_ERR_UNSUPPORTED (use one process per GPU, as the
 * multi-GPU benchmark does).  s2let_gpu_bind_device(d) names that device ahead
 * of the first call: it returns S2LET_GPU_OK if the library is unbound or
 * already serves d, S2LET_GPU_ERR_UNSUPPORTED if it serves another device,
 * S2LET_GPU_ERR_INVALID for d < 0.  s2let_gpu_bound_device() returns the
 * device served, or -1 before the first call. */
int s2let_gpu_bind_device(int device);
int s2let_gpu_bound_device(void);

/* Number of this library's kernel launches since load (instrumentation). */
uint64_t s2let_gpu_launch_count(void);

/* Optional per-kernel timing with CUDA events on the launching stream.
 * enable(1) clears previous records; report fills out[c*4 + {0,1,2,3}] =
 * {launches, milliseconds, algorithmic flops, algorithmic bytes} for kernel
 * category c < ncat (0 FP64 contraction, 1 ring DFT, 2 gamma DFT, 3 tiling
 * merge, 4 split-precision tensor-core contraction, 5 other). */
int s2let_gpu_timing_enable(int on);
int s2let_gpu_timing_report(double *out, int ncat);

/* Optional trace of the host <-> device copies made by the host-pointer batch
 * entry points, with CUDA events on the copying streams.  enable(1) clears
 * previous records and starts tracing, enable(0) stops.  report fills
 * out[d*5 + {0,1,2,3,4}] = {copies, bytes, busy milliseconds (sum of the
 * copies' own durations), span milliseconds (first start to last end), copies
 * made by the copy kernel} for direction d = 0 (host to device) and d = 1
 * (device to host).  Page-locked host buffers are moved by a copy kernel
 * (SM loads and stores over the host link); other host memory, or every copy
 * when S2LET_GPU_HOST_COPY=engine, by the copy engines
 * (S2LET_GPU_HOST_COPY=d2h_kernel: the copy kernel device to host only). */
int s2let_gpu_copy_trace_enable(int on);
int s2let_gpu_copy_trace_report(double *out);

/* Autotuning of launch shapes (maps per CTA of the FP64 and recomputed-table
 * contractions; columns per table pass and map groups per launch of the
 * split-precision contraction).  mode 1: the first call of each (kernel,
 * band-limit bucket, batch bucket) times the candidates on the live call and
 * keeps the fastest, which later calls use; the choices are kept in a cache
 * file per GPU model (S2LET_GPU_AUTOTUNE_CACHE, else
 * $XDG_CACHE_HOME/s2let_gb300/autotune.txt or ~/.cache/...) and read by later
 * processes.  mode 0 (default, or S2LET_GPU_AUTOTUNE unset): built-in
 * choices.  Every candidate computes the same result.  Returns the previous
 * mode.  entries() lists the recorded choices: keys[5 i..5 i + 4] = {family,
 * a, b, c, choice} (family 1 FP64 contraction, 2 / 3 recomputed l->t / t->l,
 * 4 split precision), ms[2 i], ms[2 i + 1] = {best, built-in} milliseconds;
 * returns the number of choices (at most max written).  No counterpart in the
 * reference. */
int s2let_gpu_autotune(int mode);
int s2let_gpu_autotune_entries(int *keys, double *ms, int max);

/* Measured FMA throughput of the current GPU, for roofline fractions: one
 * launch of 8 independent FMA chains per thread, `iters` iterations; fp64 != 0
 * times FP64 FMAs, else FP32.  *tflops = 2 x FMAs per second / 1e12.
 * Returns the status. */
int s2let_gpu_fma_rate(int fp64, int iters, double *tflops);

#ifdef __cplusplus
}
#endif
#endif /* S2LET_GPU_H */
