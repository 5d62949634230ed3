/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.  Never linked into the GPU product.
 *
 * CPU FP64 restatement of the SO3 entry points that the reference S2LET layer
 * calls (include/so3/so3.h next to this file documents conventions).  Written
 * from the SO3 sampling theorem: each direction n of a Wigner transform is a
 * spin-(-n) spherical-harmonic transform (relation
 *   e^{i m a} d^l_{mn}(b) = (-1)^n sY_lm(b,a) / sqrt((2l+1)/4pi),  s = -n)
 * followed by a DFT over the 2N-1 gamma samples; the spherical-harmonic parts
 * reuse the SSHT restatement, with Delta shared across directions.  Both
 * SO3_SAMPLING_MW and SO3_SAMPLING_MW_SS take the (alpha, beta) grid of the
 * matching SSHT sampling; gamma has 2N-1 samples in both.
 *
 * "direct" and "via_ssht" variants compute the same linear map and share one
 * implementation here.  L0 (a lower band-limit hint in SO3) only skips work in
 * SO3 and never changes results that the reference reads, so it is ignored.
 */
#include "so3/so3.h"

#include <math.h>
#include <string.h>

#include "oracle_internal.h"

#define SPI 3.14159265358979323846264338327950288

static inline double neg1(int k) { return (k & 1) ? -1.0 : 1.0; }
static long tri(long k) { return k < 0 ? 0 : k * (k + 1) * (2 * k + 1) / 6; } /* sum_{i<=k} i^2 */

static void *xcalloc(size_t n, size_t sz) {
  void *p = calloc(n ? n : 1, sz);
  if (!p) {
    fprintf(stderr, "oracle: out of memory\n");
    exit(1);
  }
  return p;
}

/* ---------------- sampling / storage ----------------------------------- */

int so3_sampling_ngamma(const so3_parameters_t *p) { return p->steerable ? p->N : 2 * p->N - 1; }
int so3_sampling_nalpha(const so3_parameters_t *p) {
  return p->sampling_scheme == SO3_SAMPLING_MW_SS ? 2 * p->L : 2 * p->L - 1;
}
int so3_sampling_nbeta(const so3_parameters_t *p) {
  return p->sampling_scheme == SO3_SAMPLING_MW_SS ? p->L + 1 : p->L;
}
int so3_sampling_f_size(const so3_parameters_t *p) {
  return so3_sampling_ngamma(p) * so3_sampling_nalpha(p) * so3_sampling_nbeta(p);
}

int so3_sampling_flmn_size(const so3_parameters_t *p) {
  long L = p->L, N = p->N;
  if (p->reality) {
    if (p->storage == SO3_STORAGE_PADDED) return (int)(N * L * L);
    return (int)(N * L * L - tri(N - 1));
  }
  if (p->storage == SO3_STORAGE_PADDED) return (int)((2 * N - 1) * L * L);
  return (int)((2 * N - 1) * L * L - 2 * tri(N - 1));
}

void so3_sampling_elmn2ind(int *ind, int el, int m, int n, const so3_parameters_t *p) {
  long L = p->L, N = p->N;
  if (p->n_order != SO3_N_ORDER_NEGATIVE_FIRST) {
    fprintf(stderr, "oracle: only SO3_N_ORDER_NEGATIVE_FIRST is restated\n");
    exit(1);
  }
  if (p->storage == SO3_STORAGE_PADDED) {
    *ind = (int)((n + N - 1) * L * L + (long)el * el + el + m);
    return;
  }
  /* compact: blocks n = -N+1..N-1, each holding l = |n|..L-1 */
  long before = (n + N - 1) * L * L; /* L^2 per preceding block, minus the dropped l<|n'| */
  long drop;
  if (n <= 0)
    drop = tri(N - 1) - tri(-n);
  else
    drop = tri(N - 1) + tri(n - 1);
  *ind = (int)(before - drop + (long)el * el - (long)n * n + el + m);
}

void so3_sampling_elmn2ind_real(int *ind, int el, int m, int n, const so3_parameters_t *p) {
  long L = p->L;
  if (p->storage == SO3_STORAGE_PADDED) {
    *ind = (int)((long)n * L * L + (long)el * el + el + m);
    return;
  }
  *ind = (int)((long)n * L * L - tri(n - 1) + (long)el * el - (long)n * n + el + m);
}

/* directions n computed for the given n_mode; real signals keep n >= 0 */
static int n_list(int *ns, const so3_parameters_t *p, int real_only) {
  int N = p->N, cnt = 0;
  for (int n = real_only ? 0 : -N + 1; n <= N - 1; ++n) {
    int ok = 1;
    switch (p->n_mode) {
    case SO3_N_MODE_EVEN: ok = (n % 2 == 0); break;
    case SO3_N_MODE_ODD: ok = (n % 2 != 0); break;
    case SO3_N_MODE_MAXIMUM: ok = (abs(n) == N - 1); break;
    default: ok = 1;
    }
    if (ok) ns[cnt++] = n;
  }
  return cnt;
}

static void check_params(const so3_parameters_t *p) {
  if (p->sampling_scheme != SO3_SAMPLING_MW && p->sampling_scheme != SO3_SAMPLING_MW_SS) {
    fprintf(stderr, "oracle: unknown SO3 sampling scheme\n");
    exit(1);
  }
  if (p->steerable) {
    fprintf(stderr, "oracle: steerable SO3 signals are not restated\n");
    exit(1);
  }
}

static int flmn_index(int l, int m, int n, const so3_parameters_t *p, int real) {
  int ind;
  if (real)
    so3_sampling_elmn2ind_real(&ind, l, m, n, p);
  else
    so3_sampling_elmn2ind(&ind, l, m, n, p);
  return ind;
}

/* ---------------- inverse ---------------------------------------------- */

/* real = 1: flmn in real storage, f real. */
static void inverse_any(void *fout, const complex double *flmn, const so3_parameters_t *p,
                        int real) {
  check_params(p);
  const int L = p->L, N = p->N, ng = so3_sampling_ngamma(p);
  const size_t npx = (size_t)so3_sampling_nalpha(p) * so3_sampling_nbeta(p);
  const int ss = p->sampling_scheme == SO3_SAMPLING_MW_SS;
  int ns[256];
  int nn = n_list(ns, p, real);
  complex double **x = (complex double **)xcalloc(nn, sizeof(void *));
  void **maps = (void **)xcalloc(nn, sizeof(void *));
  int *spin = (int *)xcalloc(nn, sizeof(int));
  int *rl = (int *)xcalloc(nn, sizeof(int));
  for (int k = 0; k < nn; ++k) {
    int n = ns[k];
    x[k] = (complex double *)xcalloc((size_t)L * L, sizeof(complex double));
    for (int l = abs(n); l < L; ++l) {
      double sc = (2.0 * l + 1.0) / (8.0 * SPI * SPI) * neg1(n) / sqrt((2.0 * l + 1.0) / (4.0 * SPI));
      for (int m = -l; m <= l; ++m) x[k][l * l + l + m] = flmn[flmn_index(l, m, n, p, real)] * sc;
    }
    spin[k] = -n;
    rl[k] = real && n == 0;
    maps[k] = rl[k] ? xcalloc(npx, sizeof(double)) : xcalloc(npx, sizeof(complex double));
  }
  oracle_ssht_inverse_multi(maps, (const complex double **)x, spin, rl, nn, L, ss);
  for (int g = 0; g < ng; ++g) {
    double gam = 2.0 * SPI * g / ng;
#pragma omp parallel for schedule(static) if (npx >= 4096)
    for (size_t i = 0; i < npx; ++i) {
      complex double acc = 0;
      for (int k = 0; k < nn; ++k) {
        int n = ns[k];
        complex double v = rl[k] ? ((double *)maps[k])[i] : ((complex double *)maps[k])[i];
        complex double e = cos(n * gam) + I * sin(n * gam);
        if (real && n > 0)
          acc += 2.0 * creal(e * v);
        else
          acc += e * v;
      }
      if (real)
        ((double *)fout)[(size_t)g * npx + i] = creal(acc);
      else
        ((complex double *)fout)[(size_t)g * npx + i] = acc;
    }
  }
  for (int k = 0; k < nn; ++k) {
    free(x[k]);
    free(maps[k]);
  }
  free(x);
  free(maps);
  free(spin);
  free(rl);
  (void)N;
}

void so3_core_inverse_direct(complex double *f, const complex double *flmn, const so3_parameters_t *p) {
  inverse_any(f, flmn, p, 0);
}
void so3_core_inverse_via_ssht(complex double *f, const complex double *flmn, const so3_parameters_t *p) {
  inverse_any(f, flmn, p, 0);
}
void so3_core_inverse_direct_real(double *f, const complex double *flmn, const so3_parameters_t *p) {
  inverse_any(f, flmn, p, 1);
}
void so3_core_inverse_via_ssht_real(double *f, const complex double *flmn, const so3_parameters_t *p) {
  inverse_any(f, flmn, p, 1);
}

/* ---------------- forward ---------------------------------------------- */

static void forward_any(complex double *flmn, const void *fin, const so3_parameters_t *p, int real) {
  check_params(p);
  const int L = p->L, ng = so3_sampling_ngamma(p);
  const size_t npx = (size_t)so3_sampling_nalpha(p) * so3_sampling_nbeta(p);
  const int ss = p->sampling_scheme == SO3_SAMPLING_MW_SS;
  int ns[256];
  int nn = n_list(ns, p, real);
  memset(flmn, 0, sizeof(complex double) * so3_sampling_flmn_size(p));
  complex double **y = (complex double **)xcalloc(nn, sizeof(void *));
  void **maps = (void **)xcalloc(nn, sizeof(void *));
  int *spin = (int *)xcalloc(nn, sizeof(int));
  int *rl = (int *)xcalloc(nn, sizeof(int));
  for (int k = 0; k < nn; ++k) {
    int n = ns[k];
    spin[k] = -n;
    rl[k] = real && n == 0;
    y[k] = (complex double *)xcalloc((size_t)L * L, sizeof(complex double));
    maps[k] = rl[k] ? xcalloc(npx, sizeof(double)) : xcalloc(npx, sizeof(complex double));
#pragma omp parallel for schedule(static) if (npx >= 4096)
    for (size_t i = 0; i < npx; ++i) {
      complex double acc = 0;
      for (int g = 0; g < ng; ++g) {
        double gam = 2.0 * SPI * g / ng;
        complex double v = real ? ((const double *)fin)[(size_t)g * npx + i]
                                : ((const complex double *)fin)[(size_t)g * npx + i];
        acc += v * (cos(n * gam) - I * sin(n * gam));
      }
      acc /= (double)ng;
      if (rl[k])
        ((double *)maps[k])[i] = creal(acc);
      else
        ((complex double *)maps[k])[i] = acc;
    }
  }
  oracle_ssht_forward_multi(y, (const void **)maps, spin, rl, nn, L, ss);
  for (int k = 0; k < nn; ++k) {
    int n = ns[k];
    for (int l = abs(n); l < L; ++l) {
      double sc = 2.0 * SPI * neg1(n) / sqrt((2.0 * l + 1.0) / (4.0 * SPI));
      for (int m = -l; m <= l; ++m) flmn[flmn_index(l, m, n, p, real)] = y[k][l * l + l + m] * sc;
    }
    free(y[k]);
    free(maps[k]);
  }
  free(y);
  free(maps);
  free(spin);
  free(rl);
}

void so3_core_forward_direct(complex double *flmn, const complex double *f, const so3_parameters_t *p) {
  forward_any(flmn, f, p, 0);
}
void so3_core_forward_via_ssht(complex double *flmn, const complex double *f, const so3_parameters_t *p) {
  forward_any(flmn, f, p, 0);
}
void so3_core_forward_direct_real(complex double *flmn, const double *f, const so3_parameters_t *p) {
  forward_any(flmn, f, p, 1);
}
void so3_core_forward_via_ssht_real(complex double *flmn, const double *f, const so3_parameters_t *p) {
  forward_any(flmn, f, p, 1);
}

/* ---------------- adjoint of the inverse -------------------------------- */

static void adjoint_inverse_any(complex double *flmn, const void *fin, const so3_parameters_t *p,
                                int real) {
  check_params(p);
  const int L = p->L, ng = so3_sampling_ngamma(p);
  const size_t npx = (size_t)so3_sampling_nalpha(p) * so3_sampling_nbeta(p);
  const int ss = p->sampling_scheme == SO3_SAMPLING_MW_SS;
  int ns[256];
  int nn = n_list(ns, p, real);
  memset(flmn, 0, sizeof(complex double) * so3_sampling_flmn_size(p));
  complex double **y = (complex double **)xcalloc(nn, sizeof(void *));
  void **maps = (void **)xcalloc(nn, sizeof(void *));
  int *spin = (int *)xcalloc(nn, sizeof(int));
  int *rl = (int *)xcalloc(nn, sizeof(int));
  for (int k = 0; k < nn; ++k) {
    int n = ns[k];
    spin[k] = -n;
    rl[k] = real && n == 0;
    y[k] = (complex double *)xcalloc((size_t)L * L, sizeof(complex double));
    maps[k] = rl[k] ? xcalloc(npx, sizeof(double)) : xcalloc(npx, sizeof(complex double));
#pragma omp parallel for schedule(static) if (npx >= 4096)
    for (size_t i = 0; i < npx; ++i) {
      complex double acc = 0;
      for (int g = 0; g < ng; ++g) {
        double gam = 2.0 * SPI * g / ng;
        complex double v = real ? ((const double *)fin)[(size_t)g * npx + i]
                                : ((const complex double *)fin)[(size_t)g * npx + i];
        acc += v * (cos(n * gam) - I * sin(n * gam));
      }
      if (rl[k])
        ((double *)maps[k])[i] = creal(acc);
      else
        ((complex double *)maps[k])[i] = acc;
    }
  }
  oracle_ssht_adjoint_inverse_multi(y, (const void **)maps, spin, rl, nn, L, ss);
  for (int k = 0; k < nn; ++k) {
    int n = ns[k];
    for (int l = abs(n); l < L; ++l) {
      double sc = (2.0 * l + 1.0) / (8.0 * SPI * SPI) * neg1(n) / sqrt((2.0 * l + 1.0) / (4.0 * SPI));
      for (int m = -l; m <= l; ++m) flmn[flmn_index(l, m, n, p, real)] = y[k][l * l + l + m] * sc;
    }
    free(y[k]);
    free(maps[k]);
  }
  free(y);
  free(maps);
  free(spin);
  free(rl);
}

void so3_adjoint_inverse_direct(complex double *flmn, const complex double *f, const so3_parameters_t *p) {
  adjoint_inverse_any(flmn, f, p, 0);
}
void so3_adjoint_inverse_direct_real(complex double *flmn, const double *f, const so3_parameters_t *p) {
  adjoint_inverse_any(flmn, f, p, 1);
}

/* ---------------- adjoint of the forward -------------------------------- */

static void adjoint_forward_any(void *fout, const complex double *flmn, const so3_parameters_t *p,
                                int real) {
  check_params(p);
  const int L = p->L, ng = so3_sampling_ngamma(p);
  const size_t npx = (size_t)so3_sampling_nalpha(p) * so3_sampling_nbeta(p);
  const int ss = p->sampling_scheme == SO3_SAMPLING_MW_SS;
  int ns[256];
  int nn = n_list(ns, p, 0); /* all directions; the real case is Re of the complex adjoint */
  complex double **x = (complex double **)xcalloc(nn, sizeof(void *));
  void **maps = (void **)xcalloc(nn, sizeof(void *));
  int *spin = (int *)xcalloc(nn, sizeof(int));
  int *rl = (int *)xcalloc(nn, sizeof(int));
  for (int k = 0; k < nn; ++k) {
    int n = ns[k];
    spin[k] = -n;
    rl[k] = 0;
    x[k] = (complex double *)xcalloc((size_t)L * L, sizeof(complex double));
    maps[k] = xcalloc(npx, sizeof(complex double));
    for (int l = abs(n); l < L; ++l) {
      double sc = 2.0 * SPI * neg1(n) / sqrt((2.0 * l + 1.0) / (4.0 * SPI));
      for (int m = -l; m <= l; ++m) {
        complex double v;
        if (!real)
          v = flmn[flmn_index(l, m, n, p, 0)];
        else if (n >= 0)
          v = flmn[flmn_index(l, m, n, p, 1)];
        else /* f_{l,m,-k} = (-1)^{m+k} conj(f_{l,-m,k}) */
          v = neg1(m - n) * conj(flmn[flmn_index(l, -m, -n, p, 1)]);
        x[k][l * l + l + m] = v * sc;
      }
    }
  }
  oracle_ssht_adjoint_forward_multi(maps, (const complex double **)x, spin, rl, nn, L, ss);
  for (int g = 0; g < ng; ++g) {
    double gam = 2.0 * SPI * g / ng;
#pragma omp parallel for schedule(static) if (npx >= 4096)
    for (size_t i = 0; i < npx; ++i) {
      complex double acc = 0;
      for (int k = 0; k < nn; ++k) {
        int n = ns[k];
        acc += (cos(n * gam) + I * sin(n * gam)) * ((complex double *)maps[k])[i];
      }
      acc /= (double)ng;
      if (real)
        ((double *)fout)[(size_t)g * npx + i] = creal(acc);
      else
        ((complex double *)fout)[(size_t)g * npx + i] = acc;
    }
  }
  for (int k = 0; k < nn; ++k) {
    free(x[k]);
    free(maps[k]);
  }
  free(x);
  free(maps);
  free(spin);
  free(rl);
}

void so3_adjoint_forward_direct(complex double *f, const complex double *flmn, const so3_parameters_t *p) {
  adjoint_forward_any(f, flmn, p, 0);
}
void so3_adjoint_forward_direct_real(double *f, const complex double *flmn, const so3_parameters_t *p) {
  adjoint_forward_any(f, flmn, p, 1);
}
