/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.  Never linked into the GPU product.
 *
 * CPU FP64 restatement of the S2LET layer of the reference (tiling, harmonic
 * tiling multiplies, multiresolution bookkeeping, orchestration of the
 * spherical-harmonic and Wigner transforms), written against the public API in
 * include/s2let_gpu.h and the SSHT/SO3 restatement in ssht_so3/.  Each function
 * cites the reference function it restates.  The organisation differs from the
 * reference (one per-scale layout table drives every transform; four harmonic
 * multiply modes share one kernel) but the arithmetic of every output element is
 * the same, including the reference's quirks, which are reproduced on purpose:
 *
 *   - f_wav offsets advance with the parity-fixed N_j while s2let_n_wav sizes
 *     the buffer with N (src/c/s2let_helper.c:78-95 vs src/c/s2let_analysis.c:340-350);
 *   - s2let_n_lmn_wav sizes with min(N, bl) without the parity fix
 *     (src/c/s2let_helper.c:48-52);
 *   - the _manual adjoints multiply by conj(psi) (analysis) and psi (synthesis)
 *     where the exact adjoint would use the other one
 *     (src/c/s2let_analysis_adjoint.c:278, src/c/s2let_synthesis_adjoint.c:266),
 *     and wav2lm_manual / analysis_adjoint_wav2lm_manual accumulate into flm
 *     without clearing it (src/c/s2let_synthesis.c:254,281);
 *   - the axisymmetric scaling map carries no 1/sqrt(2 pi) while the wavelet maps
 *     do (src/c/s2let_transform_axisym_mw.c:153-164);
 *   - hard thresholding compares abs() of a double, i.e. the int-truncated value
 *     (src/c/s2let_transform_axisym_mw.c:1193,1220).
 */
#include <ssht/ssht.h>
#include <so3/so3.h>
#define S2LET_GPU_NO_SSHT_TYPES
#include "s2let_gpu.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define PPI 3.141592653589793238462643383279502884197
#define IMIN(a, b) ((a) < (b) ? (a) : (b))
#define IMAX(a, b) ((a) > (b) ? (a) : (b))

static inline double neg1(int k) { return (k & 1) ? -1.0 : 1.0; }
static inline int lmi(int l, int m) { return l * l + l + m; }

/* ======================================================================== */
/* Tiling (src/c/s2let_tiling.c, src/c/s2let_math.c)                         */
/* ======================================================================== */

typedef enum { K_S2DW = 0, K_NEEDLET = 1, K_SPLINE = 2 } kernel_kind;
static kernel_kind g_kernel = K_S2DW; /* process-global, as src/c/s2let_tiling.c:13-14 */

/* src/c/s2let_tiling.c:24-39 */
void s2let_switch_wavtype(int typenum) {
  if (typenum == 2)
    g_kernel = K_NEEDLET;
  else if (typenum == 3)
    g_kernel = K_SPLINE;
  else {
    if (typenum != 1) printf("Kernel number should be 1, 2 or 3. Default is 1.\n");
    g_kernel = K_S2DW;
  }
}

/* src/c/s2let_tiling.c:105-110 */
int s2let_j_max(const s2let_parameters_t *p) { return ceil(log(p->L) / log(p->B)); }

/* src/c/s2let_tiling.c:51-71 */
int s2let_bandlimit(int j, const s2let_parameters_t *p) {
  if (g_kernel == K_SPLINE) {
    int Jmax = s2let_j_max(p);
    if (j == Jmax) return p->L;
    return ceil(p->L / pow(p->B, Jmax - j - 2));
  }
  return ceil(pow(p->B, j + 1));
}

/* src/c/s2let_tiling.c:82-95 */
int s2let_L0(int j, const s2let_parameters_t *p) {
  if (g_kernel == K_SPLINE) return 0;
  return ceil(pow(p->B, j - 1));
}

/* Schwartz-type integrands, src/c/s2let_math.c:15-26 */
static double s2dw_integrand(double k, double B) {
  double t = (k - (1 / B)) * (2.0 * B / (B - 1)) - 1;
  return exp(-2.0 / (1.0 - pow(t, 2.0))) / k;
}
static double needlet_integrand(double t) { return exp(-1.0 / (1.0 - pow(t, 2.0))); }

/* trapezoid rule skipping non-finite nodes, src/c/s2let_math.c:53-95 */
static double trapezoid(double a, double b, int n, int kind, double B) {
  if (a == b) return 0;
  double h = (b - a) / n, sum = 0;
  for (int i = 0; i < n; i++) {
    double x1 = a + i * h, x2 = a + (i + 1) * h;
    double f1 = kind == 0 ? s2dw_integrand(x1, B) : needlet_integrand(x1);
    double f2 = kind == 0 ? s2dw_integrand(x2, B) : needlet_integrand(x2);
    if (isfinite(f1) && isfinite(f2)) sum += ((f1 + f2) * h) / 2;
  }
  return sum;
}
double s2let_math_kappa0_quadtrap_s2dw(double a, double b, int n, double B) {
  return trapezoid(a, b, n, 0, B);
}
double s2let_math_kappa0_quadtrap_needlet(double a, double b, int n) {
  return trapezoid(a, b, n, 1, 0.0);
}

/* cubic B-spline, src/c/s2let_math.c:28-48 */
static double bspline3(double x) {
  if (fabs(x) < 1e-16) return 0;
  double c[5];
  for (int k = 0; k < 5; ++k) {
    double y = x + (double)(k - 2);
    c[k] = fabs(y * y * y);
  }
  /* weights 1,-4,6,-4,1 over (x-2, x-1, x, x+1, x+2) */
  return 1. / 12. * (c[0] - 4. * c[1] + 6. * c[2] - 4. * c[3] + c[4]);
}
double s2let_math_spline_scalingfct(double x, double y) { return 1.5 * bspline3(2.0 * x / y); }

/* exact n-choose-k with interleaved multiply/divide, src/c/s2let_math.c:241-268;
 * the non-exact branch (log-gamma fit) is not restated. */
unsigned long binomial_coefficient(int n, int k, int exact) {
  (void)exact;
  if (k > n / 2) k = n - k;
  unsigned long r = 1;
  for (unsigned long i = 1; i <= (unsigned long)k; ++i) {
    r *= (unsigned long)n - i + 1UL;
    r /= i;
  }
  return r;
}

/* phi2[l + j L], j = 0..J+1: cumulative tiling profiles, src/c/s2let_tiling.c:131-199 */
static void tiling_phi2(double *phi2, const s2let_parameters_t *p) {
  const int L = p->L, J = s2let_j_max(p);
  const double B = p->B;
  const int nq = 300;
  if (g_kernel == K_SPLINE) {
    for (int l = 0; l < L; ++l) phi2[l + (J + 1) * L] = 1.0;
    for (int j = 1; j <= J + 1; ++j) {
      double bl = (double)L / (double)pow(B, j - 2);
      double *row = phi2 + (J + 1 - j) * L;
      row[0] = 1.0;
      for (int l = 1; l < L; ++l) row[l] = (l > bl) ? 0.0 : s2let_math_spline_scalingfct((double)l, bl);
    }
    return;
  }
  double norm = (g_kernel == K_S2DW) ? s2let_math_kappa0_quadtrap_s2dw(1.0 / B, 1.0, nq, B)
                                     : s2let_math_kappa0_quadtrap_needlet(-1.0, 1.0, nq);
  for (int j = 0; j <= J + 1; j++) {
    for (int l = 0; l < L; l++) {
      double v;
      if (l < pow(B, j - 1))
        v = 1;
      else if (l > pow(B, j))
        v = 0;
      else if (g_kernel == K_S2DW)
        v = s2let_math_kappa0_quadtrap_s2dw((double)l / pow(B, j), 1.0, nq, B) / norm;
      else {
        double u = 1.0 - 2.0 * B / (B - 1.0) * (l * pow(B, -j) - 1.0 / B);
        v = s2let_math_kappa0_quadtrap_needlet(-1.0, u, nq) / norm;
      }
      phi2[l + j * L] = v;
    }
  }
}

void s2let_tiling_axisym_allocate(double **kappa, double **kappa0, const s2let_parameters_t *p) {
  *kappa = calloc((size_t)(s2let_j_max(p) + 1) * p->L, sizeof(double));
  *kappa0 = calloc(p->L, sizeof(double));
}

/* kappa_j(l) = sqrt(phi2_{j+1} - phi2_j), kappa0 = sqrt(phi2_{J_min}),
 * non-finite values replaced as src/c/s2let_tiling.c:212-247 does */
void s2let_tiling_axisym(double *kappa, double *kappa0, const s2let_parameters_t *p) {
  const int L = p->L, J = s2let_j_max(p);
  double *phi2 = calloc((size_t)(J + 2) * L, sizeof(double));
  tiling_phi2(phi2, p);
  for (int l = 0; l < L; l++) kappa0[l] = sqrt(phi2[l + p->J_min * L]);
  double carry = 0.0;
  for (int j = p->J_min; j <= J; j++) {
    double *k = kappa + (size_t)j * L;
    for (int l = 0; l < L; l++) {
      double t = sqrt(phi2[l + (j + 1) * L] - phi2[l + j * L]);
      k[l] = isfinite(t) ? t : carry;
      carry = t;
    }
    for (int l = 0; l < L; l++)
      if (!isfinite(k[l]) && (j * L + l) > 0) k[l] = kappa[(size_t)j * L + l - 1];
  }
  free(phi2);
}

void s2let_tiling_direction_allocate(complex double **s_elm, const s2let_parameters_t *p) {
  *s_elm = calloc((size_t)p->L * p->L, sizeof(complex double));
}

/* s_lm = nu sqrt(C(g, (g-m)/2) / 2^g) on the allowed m, src/c/s2let_tiling.c:281-319 */
void s2let_tiling_direction(complex double *s_elm, const s2let_parameters_t *p) {
  const int L = p->L, N = p->N;
  complex double nu = (N % 2) ? 1.0 : I;
  for (int l = 1; l < L; ++l) {
    int g = ((N + l) % 2) ? IMIN(N - 1, l) : IMIN(N - 1, l - 1);
    for (int m = -l; m <= l; ++m) {
      complex double v = 0.0;
      if (abs(m) < N && ((N + m) % 2))
        v = nu * sqrt(binomial_coefficient(g, (int)((unsigned long)(g - m) / 2UL), 1) / pow(2, g));
      s_elm[lmi(l, m)] = v;
    }
  }
}

void s2let_tiling_wavelet_allocate(complex double **psi, double **phi, const s2let_parameters_t *p) {
  *psi = calloc((size_t)(s2let_j_max(p) + 1) * p->L * p->L, sizeof(complex double));
  *phi = calloc(p->L, sizeof(double));
}

/* sqrt((l+s)!/(l-s)!) or its inverse, src/c/s2let_tiling.c:351-363 */
static double spin_lowering_norm(int l, int s) {
  double f = 1;
  for (int k = -abs(s) + 1; k <= abs(s); ++k) f *= l + k;
  return s > 0 ? sqrt(f) : sqrt(1.0 / f);
}

/* psi_j(l,m) = sqrt((2l+1)/8pi^2) kappa_j(l) s_lm, phi(l) = sqrt((2l+1)/4pi) kappa0(l),
 * src/c/s2let_tiling.c:381-429 */
void s2let_tiling_wavelet(complex double *psi, double *phi, const s2let_parameters_t *p) {
  const int L = p->L, J = s2let_j_max(p), os = p->original_spin;
  double *kappa, *kappa0;
  complex double *s_elm;
  s2let_tiling_axisym_allocate(&kappa, &kappa0, p);
  s2let_tiling_axisym(kappa, kappa0, p);
  s2let_tiling_direction_allocate(&s_elm, p);
  s2let_tiling_direction(s_elm, p);
  const int lmin = IMAX(abs(p->spin), abs(os));
  for (int l = lmin; l < L; ++l) {
    phi[l] = sqrt((2 * l + 1) / (4.0 * PPI)) * kappa0[l];
    if (os != 0) phi[l] *= spin_lowering_norm(l, os) * pow(-1, os);
  }
  for (int j = p->J_min; j <= J; ++j)
    for (int l = lmin; l < L; ++l)
      for (int m = -l; m <= l; ++m) {
        complex double v = sqrt((2 * l + 1) / (8.0 * PPI * PPI)) * kappa[j * L + l] * s_elm[lmi(l, m)];
        if (os != 0) v *= spin_lowering_norm(l, os) * pow(-1, os);
        psi[(size_t)j * L * L + lmi(l, m)] = v;
      }
  free(kappa);
  free(kappa0);
  free(s_elm);
}

/* admissibility checks, src/c/s2let_tiling.c:444-551 */
double s2let_tiling_axisym_check_identity(double *kappa, double *kappa0, const s2let_parameters_t *p) {
  const int L = p->L, J = s2let_j_max(p);
  double err = 0;
  for (int l = 0; l < L; l++) {
    double s = pow(kappa0[l], 2.0);
    for (int j = 0; j <= J; j++) s += pow(kappa[l + j * L], 2.0);
    err = fmax(err, fabs(s - 1.0));
  }
  return err;
}
double s2let_tiling_direction_check_identity(complex double *s_elm, const s2let_parameters_t *p) {
  double err = 0.0;
  for (int l = 1; l < p->L; ++l) {
    double s = 0.0;
    for (int m = -l; m <= l; ++m) s += creal(s_elm[lmi(l, m)] * conj(s_elm[lmi(l, m)]));
    err = fmax(err, fabs(s - 1.0));
  }
  return err;
}
double s2let_tiling_wavelet_check_identity(complex double *psi, double *phi, const s2let_parameters_t *p) {
  const int L = p->L, J = s2let_j_max(p), s = p->spin;
  double *id = calloc(L, sizeof(double)), err = 0.0;
  for (int l = abs(s); l < L; ++l) id[l] += 4.0 * PPI / (2 * l + 1) * phi[l] * phi[l];
  for (int j = 0; j <= J; ++j) {
    int ind = s * s;
    for (int l = abs(s); l < L; ++l)
      for (int m = -l; m <= l; ++m, ++ind)
        id[l] += 8.0 * PPI * PPI / (2 * l + 1) * creal(psi[(size_t)j * L * L + ind] * conj(psi[(size_t)j * L * L + ind]));
  }
  for (int l = abs(s); l < L; ++l) err = fmax(err, fabs(id[l] - 1.0));
  free(id);
  return err;
}

/* ======================================================================== */
/* Sizes, allocation (src/c/s2let_helper.c, src/c/s2let_alloc.c)             */
/* ======================================================================== */

static void so3_for(so3_parameters_t *sp, const s2let_parameters_t *p) {
  memset(sp, 0, sizeof *sp);
  sp->verbosity = p->verbosity;
  sp->L = p->L;
  sp->N = p->N;
  sp->sampling_scheme = (so3_sampling_t)p->sampling_scheme;
  sp->n_order = SO3_N_ORDER_NEGATIVE_FIRST;
  sp->storage = SO3_STORAGE_COMPACT;
  sp->dl_method = p->dl_method;
  sp->reality = p->reality;
  sp->steerable = 0;
  sp->L0 = 0;
  sp->n_mode = (p->N % 2) ? SO3_N_MODE_EVEN : SO3_N_MODE_ODD;
}

int s2let_n_phi(const s2let_parameters_t *p) {
  return p->sampling_scheme == S2LET_SAMPLING_MW_SS ? 2 * p->L : 2 * p->L - 1;
}
int s2let_n_theta(const s2let_parameters_t *p) {
  return p->sampling_scheme == S2LET_SAMPLING_MW_SS ? p->L + 1 : p->L;
}
int s2let_n_px(const s2let_parameters_t *p) { return s2let_n_phi(p) * s2let_n_theta(p); }
int s2let_n_lm(const s2let_parameters_t *p) { return p->L * p->L; }

static int scal_bandlimit(const s2let_parameters_t *p) {
  return p->upsample ? p->L : IMIN(s2let_bandlimit(p->J_min - 1, p), p->L);
}
int s2let_n_lm_scal(const s2let_parameters_t *p) {
  int b = scal_bandlimit(p);
  return b * b;
}
int s2let_n_lmn_wav(const s2let_parameters_t *p) {
  so3_parameters_t sp;
  so3_for(&sp, p);
  int total = 0;
  for (int j = p->J_min; j <= s2let_j_max(p); ++j) {
    if (!p->upsample) {
      int bl = IMIN(s2let_bandlimit(j, p), p->L);
      sp.L = bl;
      sp.N = IMIN(p->N, bl);
    }
    total += so3_sampling_flmn_size(&sp);
  }
  return total;
}
int s2let_n_gamma(const s2let_parameters_t *p) {
  so3_parameters_t sp;
  so3_for(&sp, p);
  return so3_sampling_ngamma(&sp);
}
int s2let_n_scal(const s2let_parameters_t *p) {
  s2let_parameters_t q = *p;
  q.L = scal_bandlimit(p);
  return s2let_n_phi(&q) * s2let_n_theta(&q);
}
int s2let_n_wav(const s2let_parameters_t *p) {
  so3_parameters_t sp;
  so3_for(&sp, p);
  int total = 0;
  for (int j = p->J_min; j <= s2let_j_max(p); ++j) {
    if (!p->upsample) sp.L = IMIN(s2let_bandlimit(j, p), p->L);
    total += so3_sampling_f_size(&sp);
  }
  return total;
}
int s2let_n_wav_j(int j, const s2let_parameters_t *p) {
  so3_parameters_t sp;
  so3_for(&sp, p);
  if (!p->upsample) sp.L = IMIN(s2let_bandlimit(j, p), p->L);
  return so3_sampling_f_size(&sp);
}

void s2let_allocate_mw(complex double **f, int L) { *f = calloc((size_t)L * (2 * L - 1), sizeof **f); }
void s2let_allocate_mw_real(double **f, int L) { *f = calloc((size_t)L * (2 * L - 1), sizeof **f); }
void s2let_allocate_mwss(complex double **f, int L) { *f = calloc((size_t)(2 * L) * (L + 1), sizeof **f); }
void s2let_allocate_mwss_real(double **f, int L) { *f = calloc((size_t)(2 * L) * (L + 1), sizeof **f); }
void s2let_allocate_lm(complex double **flm, int L) { *flm = calloc((size_t)L * L, sizeof **flm); }
void s2let_allocate_lmn_f_wav(complex double **a, complex double **b, const s2let_parameters_t *p) {
  *a = calloc(s2let_n_lmn_wav(p), sizeof **a);
  *b = calloc(s2let_n_lm_scal(p), sizeof **b);
}
void s2let_allocate_f_wav(complex double **a, complex double **b, const s2let_parameters_t *p) {
  *a = calloc(s2let_n_wav(p), sizeof **a);
  *b = calloc(s2let_n_scal(p), sizeof **b);
}
void s2let_allocate_f_wav_real(double **a, double **b, const s2let_parameters_t *p) {
  *a = calloc(s2let_n_wav(p), sizeof **a);
  *b = calloc(s2let_n_scal(p), sizeof **b);
}
void s2let_allocate_f_wav_manual(complex double **a, complex double **b, int *wav_bandlimits,
                                 int scal_bl, int N, int J, const s2let_parameters_t *p) {
  (void)N;
  so3_parameters_t sp;
  so3_for(&sp, p);
  int total = 0;
  for (int j = 0; j <= J; ++j) {
    if (!p->upsample) sp.L = wav_bandlimits[j];
    total += so3_sampling_f_size(&sp);
  }
  s2let_parameters_t q = *p;
  q.L = scal_bl;
  *a = calloc(total, sizeof **a);
  *b = calloc((size_t)s2let_n_phi(&q) * s2let_n_theta(&q), sizeof **b);
}

/* ======================================================================== */
/* Per-scale layout of one parameter set                                     */
/* ======================================================================== */

#define MAXJ 64
typedef struct {
  int L, J, J_min, nscale, bl_scal, real;
  int j[MAXJ], bl[MAXJ], Nj[MAXJ];
  long woff[MAXJ + 1], loff[MAXJ + 1];
  so3_parameters_t sp[MAXJ];
} layout_t;

/* SO3 storage sizes follow p->reality, as fill_so3_parameters does
 * (include/s2let/s2let_so3.h:24-42); `real` only selects the n >= 0 layout. */
static void layout_build(layout_t *g, const s2let_parameters_t *p, int real) {
  memset(g, 0, sizeof *g);
  const s2let_parameters_t q = *p;
  g->L = p->L;
  g->J = s2let_j_max(p);
  g->J_min = p->J_min;
  g->real = real;
  g->bl_scal = scal_bandlimit(p);
  int k = 0;
  for (int j = p->J_min; j <= g->J && k < MAXJ; ++j, ++k) {
    int bl = p->L, Nj = p->N;
    if (!p->upsample) {
      bl = IMIN(s2let_bandlimit(j, p), p->L);
      Nj = IMIN(p->N, bl);
      Nj += (Nj + p->N) % 2;
    }
    g->j[k] = j;
    g->bl[k] = bl;
    g->Nj[k] = Nj;
    so3_for(&g->sp[k], &q);
    g->sp[k].L = bl;
    g->sp[k].N = Nj;
    g->sp[k].L0 = s2let_L0(j, p);
    g->woff[k + 1] = g->woff[k] + so3_sampling_f_size(&g->sp[k]);
    g->loff[k + 1] = g->loff[k] + so3_sampling_flmn_size(&g->sp[k]);
  }
  g->nscale = k;
}

static int lmn_ind(const so3_parameters_t *sp, int l, int m, int n, int real) {
  int ind;
  if (real)
    so3_sampling_elmn2ind_real(&ind, l, m, n, sp);
  else
    so3_sampling_elmn2ind(&ind, l, m, n, sp);
  return ind;
}

/* ======================================================================== */
/* Harmonic tiling multiplies                                                */
/*   src/c/s2let_analysis.c:28-161, src/c/s2let_synthesis.c:25-175,          */
/*   src/c/s2let_analysis_adjoint.c:25-175, src/c/s2let_synthesis_adjoint.c:28-175 */
/* ======================================================================== */

typedef enum {
  SPLIT_ANALYSIS = 0, /* flmn = flm * 8pi^2/(2l+1) conj(psi)  */
  SPLIT_SYNTH_ADJ = 1 /* flmn = flm * conj(psi)               */
} split_mode;
typedef enum {
  MERGE_SYNTH = 0,    /* flm += flmn * psi                   */
  MERGE_ANALYSIS_ADJ = 1 /* flm += flmn * 8pi^2/(2l+1) psi  */
} merge_mode;

static void tiling_split(complex double *flmn, complex double *fscal, const complex double *flm,
                         const complex double *psi, const double *phi, const s2let_parameters_t *p,
                         int real, split_mode mode) {
  layout_t g;
  layout_build(&g, p, real);
  const int L = p->L, s = real ? 0 : p->spin;
  for (int k = 0; k < g.nscale; ++k) {
    const int j = g.j[k], bl = g.bl[k], Nj = g.Nj[k];
    complex double *out = flmn + g.loff[k];
    for (int n = real ? 1 - Nj % 2 : -Nj + 1; n < Nj; n += 2) {
      for (int l = real ? n : IMAX(abs(s), abs(n)); l < bl; ++l) {
        complex double w = conj(psi[(size_t)j * L * L + lmi(l, n)]);
        if (mode == SPLIT_ANALYSIS) w *= 8 * PPI * PPI / (2 * l + 1);
        for (int m = -l; m <= l; ++m) out[lmn_ind(&g.sp[k], l, m, n, real)] = flm[lmi(l, m)] * w;
      }
    }
  }
  for (int l = real ? 0 : abs(s); l < g.bl_scal; ++l) {
    double w = sqrt(4.0 * PPI / (2 * l + 1)) * phi[l];
    for (int m = -l; m <= l; ++m) fscal[lmi(l, m)] = flm[lmi(l, m)] * w;
  }
}

static void tiling_merge(complex double *flm, const complex double *flmn, const complex double *fscal,
                         const complex double *psi, const double *phi, const s2let_parameters_t *p,
                         int real, merge_mode mode) {
  layout_t g;
  layout_build(&g, p, real);
  const int L = p->L, s = real ? 0 : p->spin;
  memset(flm, 0, sizeof(complex double) * (size_t)L * L);
  for (int k = 0; k < g.nscale; ++k) {
    const int j = g.j[k], bl = g.bl[k], Nj = g.Nj[k];
    const complex double *in = flmn + g.loff[k];
    for (int n = real ? 1 - Nj % 2 : -Nj + 1; n < Nj; n += 2) {
      for (int l = real ? n : IMAX(abs(s), abs(n)); l < bl; ++l) {
        double sc = (mode == MERGE_ANALYSIS_ADJ) ? 8 * PPI * PPI / (2 * l + 1) : 1.0;
        complex double w = sc * psi[(size_t)j * L * L + lmi(l, n)];
        complex double wn = (real && n) ? sc * psi[(size_t)j * L * L + lmi(l, -n)] : 0;
        for (int m = -l; m <= l; ++m) {
          flm[lmi(l, m)] += in[lmn_ind(&g.sp[k], l, m, n, real)] * w;
          if (real && n) /* direction -n from the conjugate symmetry of real signals */
            flm[lmi(l, m)] += neg1(m + n) * conj(in[lmn_ind(&g.sp[k], l, -m, n, real)]) * wn;
        }
      }
    }
  }
  for (int l = real ? 0 : abs(s); l < g.bl_scal; ++l) {
    double w = sqrt(4.0 * PPI / (2 * l + 1)) * phi[l];
    for (int m = -l; m <= l; ++m) flm[lmi(l, m)] += fscal[lmi(l, m)] * w;
  }
}

void s2let_analysis_lm2lmn(complex double *a, complex double *b, const complex double *flm,
                           const complex double *psi, const double *phi, const s2let_parameters_t *p) {
  tiling_split(a, b, flm, psi, phi, p, 0, SPLIT_ANALYSIS);
}
void s2let_analysis_lm2lmn_real(complex double *a, complex double *b, const complex double *flm,
                                const complex double *psi, const double *phi, const s2let_parameters_t *p) {
  tiling_split(a, b, flm, psi, phi, p, 1, SPLIT_ANALYSIS);
}
void s2let_synthesis_adjoint_lm2lmn(complex double *a, complex double *b, const complex double *flm,
                                    const complex double *psi, const double *phi,
                                    const s2let_parameters_t *p) {
  tiling_split(a, b, flm, psi, phi, p, 0, SPLIT_SYNTH_ADJ);
}
void s2let_synthesis_adjoint_lm2lmn_real(complex double *a, complex double *b, const complex double *flm,
                                         const complex double *psi, const double *phi,
                                         const s2let_parameters_t *p) {
  tiling_split(a, b, flm, psi, phi, p, 1, SPLIT_SYNTH_ADJ);
}
void s2let_synthesis_lmn2lm(complex double *flm, const complex double *a, const complex double *b,
                            const complex double *psi, const double *phi, const s2let_parameters_t *p) {
  tiling_merge(flm, a, b, psi, phi, p, 0, MERGE_SYNTH);
}
void s2let_synthesis_lmn2lm_real(complex double *flm, const complex double *a, const complex double *b,
                                 const complex double *psi, const double *phi, const s2let_parameters_t *p) {
  tiling_merge(flm, a, b, psi, phi, p, 1, MERGE_SYNTH);
}
void s2let_analysis_adjoint_lmn2lm(complex double *flm, const complex double *a, const complex double *b,
                                   const complex double *psi, const double *phi,
                                   const s2let_parameters_t *p) {
  tiling_merge(flm, a, b, psi, phi, p, 0, MERGE_ANALYSIS_ADJ);
}
void s2let_analysis_adjoint_lmn2lm_real(complex double *flm, const complex double *a,
                                        const complex double *b, const complex double *psi,
                                        const double *phi, const s2let_parameters_t *p) {
  tiling_merge(flm, a, b, psi, phi, p, 1, MERGE_ANALYSIS_ADJ);
}

/* ======================================================================== */
/* Orchestration: harmonic <-> wavelet space                                 */
/* ======================================================================== */

/* src/c/s2let_analysis.c:231-246: MW and MWSS are supported, anything else is an error */
static void check_mw(const s2let_parameters_t *p) {
  if (p->sampling_scheme != S2LET_SAMPLING_MW && p->sampling_scheme != S2LET_SAMPLING_MW_SS) {
    printf("ERROR: Sampling scheme not supported.\n");
    exit(1);
  }
}

/* the SSHT entry point of the parameters' sampling scheme (the switch at e.g.
 * src/c/s2let_analysis.c:322-333): base##suffix for MW, base##_ss##suffix for MWSS */
#define SS_PICK(p, base, suffix) \
  ((p)->sampling_scheme == S2LET_SAMPLING_MW_SS ? base##_ss##suffix : base##suffix)

typedef enum { DIR_ANALYSIS, DIR_SYNTHESIS, DIR_ANALYSIS_ADJ, DIR_SYNTHESIS_ADJ } direction;

/*
 * One driver for the four harmonic <-> wavelet-space maps; `wav`/`scal` are
 * double* for real signals and complex double* otherwise.
 *   DIR_ANALYSIS      lm2wav     src/c/s2let_analysis.c:290-442
 *   DIR_SYNTHESIS     wav2lm     src/c/s2let_synthesis.c:303-458
 *   DIR_ANALYSIS_ADJ  adj wav2lm src/c/s2let_analysis_adjoint.c:304-475
 *   DIR_SYNTHESIS_ADJ adj lm2wav src/c/s2let_synthesis_adjoint.c:294-452
 */
static void wavelet_driver(direction dir, complex double *flm, void *wav, void *scal,
                           const s2let_parameters_t *p, int real) {
  check_mw(p);
  complex double *psi;
  double *phi;
  s2let_parameters_t q = *p;
  if (real) q.reality = 1;
  s2let_tiling_wavelet_allocate(&psi, &phi, &q);
  s2let_tiling_wavelet(psi, phi, &q);
  layout_t g;
  layout_build(&g, &q, real);
  complex double *flmn = calloc(g.loff[g.nscale] + 1, sizeof(complex double));
  complex double *fscal = calloc((size_t)g.bl_scal * g.bl_scal + 1, sizeof(complex double));
  const int bs = g.bl_scal;

  if (dir == DIR_ANALYSIS || dir == DIR_SYNTHESIS_ADJ)
    tiling_split(flmn, fscal, flm, psi, phi, &q, real,
                 dir == DIR_ANALYSIS ? SPLIT_ANALYSIS : SPLIT_SYNTH_ADJ);

  /* scaling part: always a spin-0 transform (src/c/s2let_analysis.c:321) */
  switch (dir) {
  case DIR_ANALYSIS:
    if (real) SS_PICK(p, ssht_core_mw_inverse_sov_sym, _real)(scal, fscal, bs, 0, 0);
    else SS_PICK(p, ssht_core_mw_inverse_sov_sym, )(scal, fscal, bs, 0, 0, 0);
    break;
  case DIR_SYNTHESIS:
    if (real) SS_PICK(p, ssht_core_mw_forward_sov_conv_sym, _real)(fscal, scal, bs, 0, 0);
    else SS_PICK(p, ssht_core_mw_forward_sov_conv_sym, )(fscal, scal, bs, 0, 0, 0);
    break;
  case DIR_ANALYSIS_ADJ:
    if (real) SS_PICK(p, ssht_adjoint_mw_inverse_sov_sym, _real)(fscal, scal, bs, 0, 0);
    else SS_PICK(p, ssht_adjoint_mw_inverse_sov_sym, )(fscal, scal, bs, 0, 0, 0);
    break;
  case DIR_SYNTHESIS_ADJ:
    if (real) SS_PICK(p, ssht_adjoint_mw_forward_sov_sym, _real)(scal, fscal, bs, 0, 0);
    else SS_PICK(p, ssht_adjoint_mw_forward_sov_sym, )(scal, fscal, bs, 0, 0, 0);
    break;
  }

  for (int k = 0; k < g.nscale; ++k) {
    complex double *lmn = flmn + g.loff[k];
    const so3_parameters_t *sp = &g.sp[k];
    if (real) {
      double *w = (double *)wav + g.woff[k];
      if (dir == DIR_ANALYSIS) so3_core_inverse_via_ssht_real(w, lmn, sp);
      else if (dir == DIR_SYNTHESIS) so3_core_forward_via_ssht_real(lmn, w, sp);
      else if (dir == DIR_ANALYSIS_ADJ) so3_adjoint_inverse_direct_real(lmn, w, sp);
      else so3_adjoint_forward_direct_real(w, lmn, sp);
    } else {
      complex double *w = (complex double *)wav + g.woff[k];
      if (dir == DIR_ANALYSIS) so3_core_inverse_direct(w, lmn, sp);
      else if (dir == DIR_SYNTHESIS) so3_core_forward_via_ssht(lmn, w, sp);
      else if (dir == DIR_ANALYSIS_ADJ) so3_adjoint_inverse_direct(lmn, w, sp);
      else so3_adjoint_forward_direct(w, lmn, sp);
    }
  }

  if (dir == DIR_SYNTHESIS || dir == DIR_ANALYSIS_ADJ)
    tiling_merge(flm, flmn, fscal, psi, phi, &q, real,
                 dir == DIR_SYNTHESIS ? MERGE_SYNTH : MERGE_ANALYSIS_ADJ);
  free(psi);
  free(phi);
  free(flmn);
  free(fscal);
}

void s2let_analysis_lm2wav(complex double *w, complex double *s, const complex double *flm,
                           const s2let_parameters_t *p) {
  wavelet_driver(DIR_ANALYSIS, (complex double *)flm, w, s, p, 0);
}
void s2let_analysis_lm2wav_real(double *w, double *s, const complex double *flm, const s2let_parameters_t *p) {
  wavelet_driver(DIR_ANALYSIS, (complex double *)flm, w, s, p, 1);
}
void s2let_synthesis_wav2lm(complex double *flm, const complex double *w, const complex double *s,
                            const s2let_parameters_t *p) {
  wavelet_driver(DIR_SYNTHESIS, flm, (void *)w, (void *)s, p, 0);
}
void s2let_synthesis_wav2lm_real(complex double *flm, const double *w, const double *s,
                                 const s2let_parameters_t *p) {
  wavelet_driver(DIR_SYNTHESIS, flm, (void *)w, (void *)s, p, 1);
}
void s2let_analysis_adjoint_wav2lm(complex double *flm, const complex double *w, const complex double *s,
                                   const s2let_parameters_t *p) {
  wavelet_driver(DIR_ANALYSIS_ADJ, flm, (void *)w, (void *)s, p, 0);
}
void s2let_analysis_adjoint_wav2lm_real(complex double *flm, const double *w, const double *s,
                                        const s2let_parameters_t *p) {
  wavelet_driver(DIR_ANALYSIS_ADJ, flm, (void *)w, (void *)s, p, 1);
}
void s2let_synthesis_adjoint_lm2wav(complex double *w, complex double *s, const complex double *flm,
                                    const s2let_parameters_t *p) {
  wavelet_driver(DIR_SYNTHESIS_ADJ, (complex double *)flm, w, s, p, 0);
}
void s2let_synthesis_adjoint_lm2wav_real(double *w, double *s, const complex double *flm,
                                         const s2let_parameters_t *p) {
  wavelet_driver(DIR_SYNTHESIS_ADJ, (complex double *)flm, w, s, p, 1);
}

/* pixel-space entry points: one full-band SSHT around the harmonic driver,
 * src/c/s2let_analysis.c:456-523, src/c/s2let_synthesis.c:472-539,
 * src/c/s2let_analysis_adjoint.c:488-556, src/c/s2let_synthesis_adjoint.c:465-532 */
void s2let_analysis_px2wav(complex double *w, complex double *s, const complex double *f,
                           const s2let_parameters_t *p) {
  check_mw(p);
  complex double *flm = calloc((size_t)p->L * p->L, sizeof *flm);
  SS_PICK(p, ssht_core_mw_forward_sov_conv_sym, )(flm, f, p->L, p->spin, 0, 0);
  s2let_analysis_lm2wav(w, s, flm, p);
  free(flm);
}
void s2let_analysis_px2wav_real(double *w, double *s, const double *f, const s2let_parameters_t *p) {
  check_mw(p);
  complex double *flm = calloc((size_t)p->L * p->L, sizeof *flm);
  SS_PICK(p, ssht_core_mw_forward_sov_conv_sym, _real)(flm, f, p->L, 0, 0);
  s2let_analysis_lm2wav_real(w, s, flm, p);
  free(flm);
}
void s2let_synthesis_wav2px(complex double *f, const complex double *w, const complex double *s,
                            const s2let_parameters_t *p) {
  check_mw(p);
  complex double *flm = calloc((size_t)p->L * p->L, sizeof *flm);
  s2let_synthesis_wav2lm(flm, w, s, p);
  SS_PICK(p, ssht_core_mw_inverse_sov_sym, )(f, flm, p->L, p->spin, 0, 0);
  free(flm);
}
void s2let_synthesis_wav2px_real(double *f, const double *w, const double *s, const s2let_parameters_t *p) {
  check_mw(p);
  complex double *flm = calloc((size_t)p->L * p->L, sizeof *flm);
  s2let_synthesis_wav2lm_real(flm, w, s, p);
  SS_PICK(p, ssht_core_mw_inverse_sov_sym, _real)(f, flm, p->L, 0, 0);
  free(flm);
}
void s2let_analysis_adjoint_wav2px(complex double *f, const complex double *w, const complex double *s,
                                   const s2let_parameters_t *p) {
  check_mw(p);
  complex double *flm = calloc((size_t)p->L * p->L, sizeof *flm);
  s2let_analysis_adjoint_wav2lm(flm, w, s, p);
  SS_PICK(p, ssht_adjoint_mw_forward_sov_sym, )(f, flm, p->L, p->spin, 0, 0);
  free(flm);
}
void s2let_analysis_adjoint_wav2px_real(double *f, const double *w, const double *s,
                                        const s2let_parameters_t *p) {
  check_mw(p);
  complex double *flm = calloc((size_t)p->L * p->L, sizeof *flm);
  s2let_analysis_adjoint_wav2lm_real(flm, w, s, p);
  SS_PICK(p, ssht_adjoint_mw_forward_sov_sym, _real)(f, flm, p->L, 0, 0);
  free(flm);
}
void s2let_synthesis_adjoint_px2wav(complex double *w, complex double *s, const complex double *f,
                                    const s2let_parameters_t *p) {
  check_mw(p);
  complex double *flm = calloc((size_t)p->L * p->L, sizeof *flm);
  SS_PICK(p, ssht_adjoint_mw_inverse_sov_sym, )(flm, f, p->L, p->spin, 0, 0);
  s2let_synthesis_adjoint_lm2wav(w, s, flm, p);
  free(flm);
}
void s2let_synthesis_adjoint_px2wav_real(double *w, double *s, const double *f, const s2let_parameters_t *p) {
  check_mw(p);
  complex double *flm = calloc((size_t)p->L * p->L, sizeof *flm);
  SS_PICK(p, ssht_adjoint_mw_inverse_sov_sym, _real)(flm, f, p->L, 0, 0);
  s2let_synthesis_adjoint_lm2wav_real(w, s, flm, p);
  free(flm);
}

/* ======================================================================== */
/* Manual tiling variants                                                     */
/*   src/c/s2let_analysis.c:188-276, src/c/s2let_synthesis.c:202-289,         */
/*   src/c/s2let_analysis_adjoint.c:202-291, src/c/s2let_synthesis_adjoint.c:189-281 */
/* ======================================================================== */

static void manual_so3(so3_parameters_t *sp, int L, int N, int bl) {
  s2let_parameters_t q;
  memset(&q, 0, sizeof q);
  q.L = L;
  q.N = N;
  so3_for(sp, &q);
  int Nj = IMIN(N, bl);
  Nj += (Nj + N) % 2;
  sp->L = bl;
  sp->N = Nj;
  sp->L0 = 0;
}

static void manual_driver(direction dir, complex double *flm, complex double *wav, complex double *scal,
                          const double *scal_l, const complex double *wav_lm, int scal_bl,
                          const int *wav_bl, int J, int L, int spin, int N) {
  const int bs = IMIN(scal_bl, L);
  complex double *fscal = calloc((size_t)bs * bs + 1, sizeof(complex double));
  if (dir == DIR_SYNTHESIS_ADJ) { /* src/c/s2let_synthesis_adjoint.c:215-218 prints these */
    printf("J = %i\n", J);
    printf("B = %g\n", pow(L, 1.0 / (float)(J + 2)));
    printf("N = %i\n", N);
    printf("L = %i\n", L);
  }
  if (dir == DIR_ANALYSIS || dir == DIR_SYNTHESIS_ADJ) {
    for (int l = abs(spin); l < bs; ++l)
      for (int m = -l; m <= l; ++m) fscal[lmi(l, m)] = flm[lmi(l, m)] * sqrt(4.0 * PPI / (2 * l + 1)) * scal_l[l];
    if (dir == DIR_ANALYSIS)
      ssht_core_mw_inverse_sov_sym(scal, fscal, bs, 0, 0, 0);
    else
      ssht_adjoint_mw_forward_sov_sym(scal, fscal, bs, 0, 0, 0);
  } else {
    if (dir == DIR_SYNTHESIS)
      ssht_core_mw_forward_sov_conv_sym(fscal, scal, bs, 0, 0, 0);
    else
      ssht_adjoint_mw_inverse_sov_sym(fscal, scal, bs, 0, 0, 0);
    for (int l = abs(spin); l < bs; ++l)
      for (int m = -l; m <= l; ++m) flm[lmi(l, m)] += fscal[lmi(l, m)] * sqrt(4.0 * PPI / (2 * l + 1)) * scal_l[l];
  }
  free(fscal);
  long off = 0;
  for (int j = 0; j <= J; ++j) {
    const int bl = IMIN(wav_bl[j], L);
    so3_parameters_t sp;
    manual_so3(&sp, L, N, bl);
    const int Nj = sp.N;
    complex double *lmn = calloc(so3_sampling_flmn_size(&sp) + 1, sizeof(complex double));
    if (dir == DIR_SYNTHESIS) so3_core_forward_direct(lmn, wav + off, &sp);
    if (dir == DIR_ANALYSIS_ADJ) so3_adjoint_inverse_direct(lmn, wav + off, &sp);
    for (int n = -Nj + 1; n < Nj; n += 2)
      for (int l = IMAX(abs(spin), abs(n)); l < bl; ++l) {
        complex double ps = wav_lm[(size_t)j * L * L + lmi(l, n)];
        complex double w;
        switch (dir) {
        case DIR_ANALYSIS: w = 8 * PPI * PPI / (2 * l + 1) * conj(ps); break;
        case DIR_SYNTHESIS: w = ps; break;
        case DIR_ANALYSIS_ADJ: w = 8 * PPI * PPI / (2 * l + 1) * conj(ps); break;
        default: w = ps; break;
        }
        for (int m = -l; m <= l; ++m) {
          int ind = lmn_ind(&sp, l, m, n, 0);
          if (dir == DIR_ANALYSIS || dir == DIR_SYNTHESIS_ADJ)
            lmn[ind] = flm[lmi(l, m)] * w;
          else
            flm[lmi(l, m)] += lmn[ind] * w;
        }
      }
    if (dir == DIR_ANALYSIS) so3_core_inverse_direct(wav + off, lmn, &sp);
    if (dir == DIR_SYNTHESIS_ADJ) so3_adjoint_forward_direct(wav + off, lmn, &sp);
    free(lmn);
    off += so3_sampling_f_size(&sp);
  }
}

void s2let_analysis_lm2wav_manual(complex double *w, complex double *s, const complex double *flm,
                                  const double *scal_l, const complex double *wav_lm, const int sb,
                                  const int *wb, int J, int L, int spin, int N) {
  manual_driver(DIR_ANALYSIS, (complex double *)flm, w, s, scal_l, wav_lm, sb, wb, J, L, spin, N);
}
void s2let_synthesis_wav2lm_manual(complex double *flm, const complex double *w, const complex double *s,
                                   const double *scal_l, const complex double *wav_lm, const int sb,
                                   const int *wb, int J, int L, int spin, int N) {
  manual_driver(DIR_SYNTHESIS, flm, (complex double *)w, (complex double *)s, scal_l, wav_lm, sb, wb, J, L,
                spin, N);
}
void s2let_analysis_adjoint_wav2lm_manual(complex double *flm, const complex double *w,
                                          const complex double *s, const double *scal_l,
                                          const complex double *wav_lm, const int sb, const int *wb,
                                          int J, int L, int spin, int N) {
  manual_driver(DIR_ANALYSIS_ADJ, flm, (complex double *)w, (complex double *)s, scal_l, wav_lm, sb, wb, J,
                L, spin, N);
}
void s2let_synthesis_adjoint_lm2wav_manual(complex double *w, complex double *s, const complex double *flm,
                                           const double *scal_l, const complex double *wav_lm,
                                           const int sb, const int *wb, int J, int L, int spin, int N) {
  manual_driver(DIR_SYNTHESIS_ADJ, (complex double *)flm, w, s, scal_l, wav_lm, sb, wb, J, L, spin, N);
}

/* ======================================================================== */
/* Axisymmetric wavelets (src/c/s2let_transform_axisym_lm.c, _mw.c)          */
/* ======================================================================== */

void s2let_transform_axisym_lm_allocate_f_wav(complex double **a, complex double **b,
                                              const s2let_parameters_t *p) {
  *a = calloc((size_t)(s2let_j_max(p) + 1 - p->J_min) * p->L * p->L, sizeof **a);
  *b = calloc((size_t)p->L * p->L, sizeof **b);
}
void s2let_transform_axisym_lm_allocate_f_wav_multires(complex double **a, complex double **b,
                                                       const s2let_parameters_t *p) {
  long tot = 0;
  for (int j = p->J_min; j <= s2let_j_max(p); ++j) {
    long bl = IMIN(s2let_bandlimit(j, p), p->L);
    tot += bl * bl;
  }
  long bs = IMIN(s2let_bandlimit(p->J_min - 1, p), p->L);
  *a = calloc(tot, sizeof **a);
  *b = calloc(bs * bs, sizeof **b);
}
void s2let_transform_axisym_lm_allocate_wav(double **w, double **s, const s2let_parameters_t *p) {
  *w = calloc((size_t)(s2let_j_max(p) + 1) * p->L, sizeof(double));
  *s = calloc(p->L, sizeof(double));
}
/* wav_lm[j L + l] = sqrt((2l+1)/4pi) kappa_j(l), src/c/s2let_transform_axisym_lm.c:91-118 */
void s2let_transform_axisym_lm_wav(double *wav_lm, double *scal_lm, const s2let_parameters_t *p) {
  const int L = p->L, J = s2let_j_max(p);
  double *kappa, *kappa0;
  s2let_tiling_axisym_allocate(&kappa, &kappa0, p);
  s2let_tiling_axisym(kappa, kappa0, p);
  for (int j = p->J_min; j <= J; j++)
    for (int l = 0; l < L; l++) wav_lm[j * L + l] = sqrt((2 * l + 1) / (4.0 * PPI)) * kappa[l + j * L];
  for (int l = 0; l < L; l++) scal_lm[l] = sqrt((2 * l + 1) / (4.0 * PPI)) * kappa0[l];
  free(kappa);
  free(kappa0);
}

/* analysis writes, synthesis accumulates (src/c/s2let_transform_axisym_lm.c:133-308) */
static void axisym_lm_apply(complex double *flm, complex double *fwav, complex double *fscal,
                            const double *wav_lm, const double *scal_lm, const s2let_parameters_t *p,
                            int multires, int synth) {
  const int L = p->L, J = s2let_j_max(p);
  long off = 0;
  for (int j = p->J_min; j <= J; j++) {
    int bl = multires ? IMIN(s2let_bandlimit(j, p), L) : L;
    for (int l = 0; l < bl; l++) {
      double w = sqrt((4.0 * PPI) / (2.0 * l + 1.0)) * wav_lm[j * L + l];
      for (int m = -l; m <= l; m++) {
        if (synth)
          flm[lmi(l, m)] += fwav[off + lmi(l, m)] * w;
        else
          fwav[off + lmi(l, m)] = flm[lmi(l, m)] * w;
      }
    }
    off += (long)bl * bl;
  }
  int bs = multires ? IMIN(s2let_bandlimit(p->J_min - 1, p), L) : L;
  for (int l = 0; l < bs; l++) {
    double w = sqrt((4.0 * PPI) / (2.0 * l + 1.0)) * scal_lm[l];
    for (int m = -l; m <= l; m++) {
      if (synth)
        flm[lmi(l, m)] += fscal[lmi(l, m)] * w;
      else
        fscal[lmi(l, m)] = flm[lmi(l, m)] * w;
    }
  }
}
void s2let_transform_axisym_lm_wav_analysis(complex double *a, complex double *b, const complex double *flm,
                                            const double *w, const double *s, const s2let_parameters_t *p) {
  axisym_lm_apply((complex double *)flm, a, b, w, s, p, 0, 0);
}
void s2let_transform_axisym_lm_wav_synthesis(complex double *flm, const complex double *a,
                                             const complex double *b, const double *w, const double *s,
                                             const s2let_parameters_t *p) {
  axisym_lm_apply(flm, (complex double *)a, (complex double *)b, w, s, p, 0, 1);
}
void s2let_transform_axisym_lm_wav_analysis_multires(complex double *a, complex double *b,
                                                     const complex double *flm, const double *w,
                                                     const double *s, const s2let_parameters_t *p) {
  axisym_lm_apply((complex double *)flm, a, b, w, s, p, 1, 0);
}
void s2let_transform_axisym_lm_wav_synthesis_multires(complex double *flm, const complex double *a,
                                                      const complex double *b, const double *w,
                                                      const double *s, const s2let_parameters_t *p) {
  axisym_lm_apply(flm, (complex double *)a, (complex double *)b, w, s, p, 1, 1);
}

void s2let_transform_axisym_allocate_mw_f_wav(complex double **a, complex double **b, const s2let_parameters_t *p) {
  *a = calloc((size_t)(s2let_j_max(p) + 1 - p->J_min) * p->L * (2 * p->L - 1), sizeof **a);
  *b = calloc((size_t)p->L * (2 * p->L - 1), sizeof **b);
}
static long axisym_mr_total(const s2let_parameters_t *p, long *scal) {
  long tot = 0;
  for (int j = p->J_min; j <= s2let_j_max(p); ++j) {
    long bl = IMIN(s2let_bandlimit(j, p), p->L);
    tot += bl * (2 * bl - 1);
  }
  long bs = IMIN(s2let_bandlimit(p->J_min - 1, p), p->L);
  *scal = bs * (2 * bs - 1);
  return tot;
}
void s2let_transform_axisym_allocate_mw_f_wav_multires(complex double **a, complex double **b,
                                                       const s2let_parameters_t *p) {
  long sc, tot = axisym_mr_total(p, &sc);
  *a = calloc(tot, sizeof **a);
  *b = calloc(sc, sizeof **b);
}
void s2let_transform_axisym_allocate_mw_f_wav_real(double **a, double **b, const s2let_parameters_t *p) {
  *a = calloc((size_t)(s2let_j_max(p) + 1 - p->J_min) * p->L * (2 * p->L - 1), sizeof **a);
  *b = calloc((size_t)p->L * (2 * p->L - 1), sizeof **b);
}
void s2let_transform_axisym_allocate_mw_f_wav_multires_real(double **a, double **b,
                                                            const s2let_parameters_t *p) {
  long sc, tot = axisym_mr_total(p, &sc);
  *a = calloc(tot, sizeof **a);
  *b = calloc(sc, sizeof **b);
}

/*
 * Axisymmetric pixel-space transforms (src/c/s2let_transform_axisym_mw.c:124-1171).
 * Spin 0 always.  Wavelet maps carry 1/sqrt(2pi) (analysis) or sqrt(2pi)
 * (synthesis and the adjoints' inputs/outputs); the scaling map carries none.
 * op: 0 analysis, 1 analysis adjoint, 2 synthesis, 3 synthesis adjoint.
 */
static void axisym_mw(int op, void *f, void *fwav, void *fscal, const s2let_parameters_t *p, int multires,
                      int real) {
  const int L = p->L, J = s2let_j_max(p);
  const double r2pi = sqrt(2 * PPI);
  double *wav_lm, *scal_lm;
  s2let_transform_axisym_lm_allocate_wav(&wav_lm, &scal_lm, p);
  s2let_transform_axisym_lm_wav(wav_lm, scal_lm, p);
  complex double *flm = calloc((size_t)L * L, sizeof *flm), *wlm, *slm;
  if (multires)
    s2let_transform_axisym_lm_allocate_f_wav_multires(&wlm, &slm, p);
  else
    s2let_transform_axisym_lm_allocate_f_wav(&wlm, &slm, p);
  const int bs = multires ? IMIN(s2let_bandlimit(p->J_min - 1, p), L) : L;
  const size_t esz = real ? sizeof(double) : sizeof(complex double);
  void *tmp = calloc((size_t)L * (2 * L - 1), esz);

#define SSHT_FWD(out, in, b) (real ? ssht_core_mw_forward_sov_conv_sym_real(out, in, b, 0, 0) \
                                   : ssht_core_mw_forward_sov_conv_sym(out, in, b, 0, 0, 0))
#define SSHT_INV(out, in, b) (real ? ssht_core_mw_inverse_sov_sym_real(out, in, b, 0, 0) \
                                   : ssht_core_mw_inverse_sov_sym(out, in, b, 0, 0, 0))
#define SSHT_AINV(out, in, b) (real ? ssht_adjoint_mw_inverse_sov_sym_real(out, in, b, 0, 0) \
                                    : ssht_adjoint_mw_inverse_sov_sym(out, in, b, 0, 0, 0))
#define SSHT_AFWD(out, in, b) (real ? ssht_adjoint_mw_forward_sov_sym_real(out, in, b, 0, 0) \
                                    : ssht_adjoint_mw_forward_sov_sym(out, in, b, 0, 0, 0))

  /* scale a block of n elements: dst = src * s (div = 0) or src / s (div = 1) */
#define SCALE(dst, src, n, s, div)                                                                \
  do {                                                                                            \
    for (size_t i_ = 0; i_ < (size_t)(n); ++i_) {                                                 \
      if (real) {                                                                                 \
        double v_ = ((const double *)(src))[i_];                                                  \
        ((double *)(dst))[i_] = (div) ? v_ / (s) : v_ * (s);                                      \
      } else {                                                                                    \
        complex double v_ = ((const complex double *)(src))[i_];                                  \
        ((complex double *)(dst))[i_] = (div) ? v_ / (s) : v_ * (s);                              \
      }                                                                                           \
    }                                                                                             \
  } while (0)

  if (op == 0 || op == 3) { /* pixels -> harmonic on the full map */
    if (op == 0) SSHT_FWD(flm, f, L);
    else SSHT_AINV(flm, f, L);
    axisym_lm_apply(flm, wlm, slm, wav_lm, scal_lm, p, multires, 0);
    if (op == 0) SSHT_INV(fscal, slm, bs);
    else SSHT_AFWD(fscal, slm, bs);
    long off = 0, offl = 0;
    for (int j = p->J_min; j <= J; ++j) {
      int bl = multires ? IMIN(s2let_bandlimit(j, p), L) : L;
      void *dst = (char *)fwav + off * esz;
      if (op == 0) SSHT_INV(dst, wlm + offl, bl);
      else SSHT_AFWD(dst, wlm + offl, bl);
      SCALE(dst, dst, (size_t)bl * (2 * bl - 1), r2pi, op == 0);
      off += (long)bl * (2 * bl - 1);
      offl += (long)bl * bl;
    }
  } else { /* wavelet maps -> harmonic -> pixels */
    if (op == 2) SSHT_FWD(slm, fscal, bs);
    else SSHT_AINV(slm, fscal, bs);
    long off = 0, offl = 0;
    for (int j = p->J_min; j <= J; ++j) {
      int bl = multires ? IMIN(s2let_bandlimit(j, p), L) : L;
      const char *src = (const char *)fwav + off * esz;
      SCALE(tmp, src, (size_t)bl * (2 * bl - 1), r2pi, op == 1);
      if (op == 2) SSHT_FWD(wlm + offl, tmp, bl);
      else SSHT_AINV(wlm + offl, tmp, bl);
      off += (long)bl * (2 * bl - 1);
      offl += (long)bl * bl;
    }
    axisym_lm_apply(flm, wlm, slm, wav_lm, scal_lm, p, multires, 1);
    if (op == 2) SSHT_INV(f, flm, L);
    else SSHT_AFWD(f, flm, L);
  }
#undef SSHT_FWD
#undef SSHT_INV
#undef SSHT_AINV
#undef SSHT_AFWD
#undef SCALE
  free(tmp);
  free(flm);
  free(wlm);
  free(slm);
  free(wav_lm);
  free(scal_lm);
}

/* analysis: (f_wav, f_scal, f) */
void s2let_transform_axisym_wav_analysis_mw(complex double *w, complex double *s, const complex double *f,
                                            const s2let_parameters_t *p) { axisym_mw(0, (void *)f, w, s, p, 0, 0); }
void s2let_transform_axisym_wav_analysis_mw_multires(complex double *w, complex double *s,
                                                     const complex double *f, const s2let_parameters_t *p) {
  axisym_mw(0, (void *)f, w, s, p, 1, 0);
}
void s2let_transform_axisym_wav_analysis_mw_real(double *w, double *s, const double *f,
                                                 const s2let_parameters_t *p) { axisym_mw(0, (void *)f, w, s, p, 0, 1); }
void s2let_transform_axisym_wav_analysis_mw_multires_real(double *w, double *s, const double *f,
                                                          const s2let_parameters_t *p) {
  axisym_mw(0, (void *)f, w, s, p, 1, 1);
}
/* analysis adjoint: (f, f_wav, f_scal) */
void s2let_transform_axisym_wav_analysis_adjoint_mw(complex double *f, const complex double *w,
                                                    const complex double *s, const s2let_parameters_t *p) {
  axisym_mw(1, f, (void *)w, (void *)s, p, 0, 0);
}
void s2let_transform_axisym_wav_analysis_adjoint_mw_multires(complex double *f, const complex double *w,
                                                             const complex double *s,
                                                             const s2let_parameters_t *p) {
  axisym_mw(1, f, (void *)w, (void *)s, p, 1, 0);
}
void s2let_transform_axisym_wav_analysis_adjoint_mw_real(double *f, const double *w, const double *s,
                                                         const s2let_parameters_t *p) {
  axisym_mw(1, f, (void *)w, (void *)s, p, 0, 1);
}
void s2let_transform_axisym_wav_analysis_adjoint_mw_multires_real(double *f, const double *w,
                                                                  const double *s,
                                                                  const s2let_parameters_t *p) {
  axisym_mw(1, f, (void *)w, (void *)s, p, 1, 1);
}
/* synthesis: (f, f_wav, f_scal) */
void s2let_transform_axisym_wav_synthesis_mw(complex double *f, const complex double *w,
                                             const complex double *s, const s2let_parameters_t *p) {
  axisym_mw(2, f, (void *)w, (void *)s, p, 0, 0);
}
void s2let_transform_axisym_wav_synthesis_mw_multires(complex double *f, const complex double *w,
                                                      const complex double *s, const s2let_parameters_t *p) {
  axisym_mw(2, f, (void *)w, (void *)s, p, 1, 0);
}
void s2let_transform_axisym_wav_synthesis_mw_real(double *f, const double *w, const double *s,
                                                  const s2let_parameters_t *p) {
  axisym_mw(2, f, (void *)w, (void *)s, p, 0, 1);
}
void s2let_transform_axisym_wav_synthesis_mw_multires_real(double *f, const double *w, const double *s,
                                                           const s2let_parameters_t *p) {
  axisym_mw(2, f, (void *)w, (void *)s, p, 1, 1);
}
/* synthesis adjoint: (f_wav, f_scal, f) */
void s2let_transform_axisym_wav_synthesis_adjoint_mw(complex double *w, complex double *s,
                                                     const complex double *f, const s2let_parameters_t *p) {
  axisym_mw(3, (void *)f, w, s, p, 0, 0);
}
void s2let_transform_axisym_wav_synthesis_adjoint_mw_multires(complex double *w, complex double *s,
                                                              const complex double *f,
                                                              const s2let_parameters_t *p) {
  axisym_mw(3, (void *)f, w, s, p, 1, 0);
}
void s2let_transform_axisym_wav_synthesis_adjoint_mw_real(double *w, double *s, const double *f,
                                                          const s2let_parameters_t *p) {
  axisym_mw(3, (void *)f, w, s, p, 0, 1);
}
void s2let_transform_axisym_wav_synthesis_adjoint_mw_multires_real(double *w, double *s, const double *f,
                                                                   const s2let_parameters_t *p) {
  axisym_mw(3, (void *)f, w, s, p, 1, 1);
}

/* |g| < threshold_j -> 0, with the reference's int truncation of |g|
 * (src/c/s2let_transform_axisym_mw.c:1183-1225) */
static void hard_threshold(double *g, const double *thr, const s2let_parameters_t *p, int multires) {
  long off = 0;
  for (int j = p->J_min; j <= s2let_j_max(p); j++) {
    long bl = multires ? IMIN(s2let_bandlimit(j, p), p->L) : p->L;
    for (long i = 0; i < bl * (2 * bl - 1); i++) {
      int truncated = (int)g[off + i];
      if (abs(truncated) < thr[j - p->J_min]) g[off + i] = 0;
    }
    off += bl * (2 * bl - 1);
  }
}
void s2let_transform_axisym_wav_hardthreshold_real(double *g, const double *t, const s2let_parameters_t *p) {
  hard_threshold(g, t, p, 0);
}
void s2let_transform_axisym_wav_hardthreshold_multires_real(double *g, const double *t,
                                                            const s2let_parameters_t *p) {
  hard_threshold(g, t, p, 1);
}

/* ======================================================================== */
/* MW spherical-harmonic helpers (src/c/s2let_mw.c, src/c/s2let_lm.c)        */
/* ======================================================================== */

void s2let_mw_alm2map(complex double *f, const complex double *flm, int L, int spin) {
  ssht_core_mw_inverse_sov_sym(f, flm, L, spin, 0, 0);
}
void s2let_mw_map2alm(complex double *flm, const complex double *f, int L, int spin) {
  ssht_core_mw_forward_sov_conv_sym(flm, f, L, spin, 0, 0);
}
void s2let_mw_alm2map_real(double *f, const complex double *flm, int L) {
  ssht_core_mw_inverse_sov_sym_real(f, flm, L, 0, 0);
}
void s2let_mw_map2alm_real(complex double *flm, const double *f, int L) {
  ssht_core_mw_forward_sov_conv_sym_real(flm, f, L, 0, 0);
}
double s2let_lm_power(complex double *flm, int L) {
  double t = 0.0;
  for (int i = 0; i < L * L; ++i) t += pow(cabs(flm[i]), 2.0);
  return t / (L * L);
}
double s2let_mw_power(complex double *f, int L) {
  complex double *flm = calloc((size_t)L * L, sizeof *flm);
  s2let_mw_map2alm(flm, f, L, 0);
  double r = s2let_lm_power(flm, L);
  free(flm);
  return r;
}
double s2let_mw_power_real(double *f, int L) {
  complex double *flm = calloc((size_t)L * L, sizeof *flm);
  s2let_mw_map2alm_real(flm, f, L);
  double r = s2let_lm_power(flm, L);
  free(flm);
  return r;
}
