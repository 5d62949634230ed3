/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.  Never linked into the GPU product.
 *
 * CPU FP64 restatement of the SSHT entry points that the reference S2LET layer
 * calls (declared in include/ssht/ssht.h next to this file).  SSHT itself is an
 * external dependency of the reference and is not in its tree; this file is
 * written from the McEwen-Wiaux sampling theorem:
 *
 *   inverse:  f(theta_t, phi_p) = sum_{l,m} flm sY_lm(theta_t, phi_p)  evaluated by
 *             separation of variables, expanding d^l_{m,n}(theta) in Fourier
 *             series through Wigner d at pi/2 ("Delta"):
 *                 d^l_{mn}(theta) = i^{n-m} sum_{m'} Delta^l_{m'm} Delta^l_{m'n} e^{i m' theta}
 *   forward:  the exact MW quadrature: phi-DFT per ring, extension of each
 *             m-signal to the full theta circle with parity (-1)^{m+s}, theta-DFT,
 *             convolution with w(p) = int_0^pi e^{ipt} sin t dt, then the Delta
 *             contraction.  Exact for band-limited signals.
 *   adjoints: each of the steps above transposed (true adjoints, not inverses).
 *   MWSS:     the same operators on the symmetric grid (theta_t = pi t/L with
 *             both poles, 2L samples per ring): the extension to the full
 *             circle mirrors ring t to 2L - t and carries no half-step phase,
 *             both DFTs have length 2L and their Nyquist bins are dropped.
 *
 * Delta^l is generated per l by a three-term recursion in its second index,
 * started from the closed form Delta^l_{m',l} = sqrt(C(2l, l+m'))/2^l and kept
 * in a mantissa/exponent form so that deep-underflow starts stay exact.
 * Several transforms that share L can be evaluated in one sweep over l (the
 * SO3 restatement uses this to share Delta across directions n).
 */
#include "ssht/ssht.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "offt.h"
#include "oracle_internal.h"

#define SPI 3.14159265358979323846264338327950288

static inline double neg1(int k) { return (k & 1) ? -1.0 : 1.0; }
static inline complex double ipow(int k) {
  switch (((k % 4) + 4) % 4) {
  case 0: return 1.0;
  case 1: return I;
  case 2: return -1.0;
  default: return -I;
  }
}
static inline int modk(int a, int K) { int r = a % K; return r < 0 ? r + K : r; }

static void *xcalloc(size_t n, size_t sz) {
  void *p = calloc(n ? n : 1, sz);
  if (!p) {
    fprintf(stderr, "oracle: out of memory\n");
    exit(1);
  }
  return p;
}

/* ------------------------------------------------------------------------ */
/* Wigner d                                                                 */
/* ------------------------------------------------------------------------ */

void oracle_delta_quadrant(double *D, int l) {
  const int w = l + 1;
  if (l == 0) {
    D[0] = 1.0;
    return;
  }
  double *a = (double *)xcalloc(w + 1, sizeof(double));
  double *b = (double *)xcalloc(w + 1, sizeof(double));
  double *sv = (double *)xcalloc(w, sizeof(double));
  int *se = (int *)xcalloc(w, sizeof(int));
  for (int n = 1; n <= l; ++n) {
    a[n] = sqrt((double)(l - n) * (double)(l + n + 1));
    b[n] = sqrt((double)(l + n) * (double)(l - n + 1));
  }
  /* start values sqrt(C(2l, l+mp)/4^l) = sv[mp] * 2^se[mp], from r(0) = C(2l,l)/4^l
   * and r(mp)/r(mp-1) = (l-mp+1)/(l+mp), kept as mantissa * 2^exponent */
  double rm = 1.0;
  int re = 0;
  for (int k = 1; k <= l; ++k) {
    int e;
    rm = frexp(rm * ((2.0 * k - 1.0) / (2.0 * k)), &e);
    re += e;
  }
  for (int mp = 0; mp <= l; ++mp) {
    if (mp > 0) {
      int e;
      rm = frexp(rm * ((double)(l - mp + 1) / (double)(l + mp)), &e);
      re += e;
    }
    if (re & 1) {
      sv[mp] = sqrt(rm * 2.0);
      se[mp] = (re - 1) / 2;
    } else {
      sv[mp] = sqrt(rm);
      se[mp] = re / 2;
    }
  }
  /* three-term recursion in the second index, downward from n = l */
#pragma omp parallel for schedule(static) if (l >= 64)
  for (int mp = 0; mp <= l; ++mp) {
    double *row = D + (size_t)mp * w;
    double vn = sv[mp], vn1 = 0.0;
    int E = se[mp];
    row[l] = ldexp(vn, E);
    for (int n = l; n >= 1; --n) {
      double vm = (-2.0 * mp * vn - a[n] * vn1) / b[n];
      vn1 = vn;
      vn = vm;
      if (fabs(vn) > 0x1p600) {
        vn = ldexp(vn, -600);
        vn1 = ldexp(vn1, -600);
        E += 600;
      }
      row[n - 1] = ldexp(vn, E);
    }
  }
  free(a);
  free(b);
  free(sv);
  free(se);
}

void oracle_wigner_d_column(double *out, int L, int m, int n, double theta) {
  /* d^l_{mn}(theta), l = l0..L-1 stored at out[l]; scaled three-term recursion */
  int l0 = abs(m) > abs(n) ? abs(m) : abs(n);
  for (int l = 0; l < L; ++l) out[l] = 0.0;
  if (l0 >= L) return;
  double c = cos(theta / 2), s = sin(theta / 2);
  /* closed form at l0 in log space */
  int ka, kb;
  double sign = 1.0;
  int k; /* binomial C(2 l0, k) */
  /* closed forms of d^{l0}: second index = l0 gives sqrt(C(2l0, l0+m)) c^{l0+m} s^{l0-m};
   * the others follow from d_{mn} = (-1)^{m-n} d_{nm} and d_{-m,-n} = (-1)^{m-n} d_{mn} */
  if (l0 == m) {
    ka = m + n; kb = m - n; k = m + n; sign = neg1(l0 - n);
  } else if (l0 == -m) {
    ka = l0 - n; kb = l0 + n; k = l0 - n;
  } else if (l0 == n) {
    ka = l0 + m; kb = l0 - m; k = l0 + m;
  } else {
    ka = l0 - m; kb = l0 + m; k = l0 - m; sign = neg1(m + l0);
  }
  double lg = 0.5 * (lgamma(2.0 * l0 + 1) - lgamma(k + 1.0) - lgamma(2.0 * l0 - k + 1.0));
  double lv = lg + (ka ? ka * log(fabs(c)) : 0.0) + (kb ? kb * log(fabs(s)) : 0.0);
  double sg = sign * ((ka & 1) && c < 0 ? -1.0 : 1.0) * ((kb & 1) && s < 0 ? -1.0 : 1.0);
  int E = (int)floor(lv / log(2.0));
  double v = sg * exp(lv - E * log(2.0));
  double vprev = 0.0;
  out[l0] = ldexp(v, E);
  double ct = cos(theta);
  int lstart = l0;
  if (l0 == 0) { /* m = n = 0: d^0 = 1, d^1_{00} = cos(theta) */
    if (L > 1) out[1] = ldexp(ct * v, E);
    vprev = v;
    v = ct * v;
    lstart = 1;
  }
  for (int l = lstart; l + 1 < L; ++l) {
    double num = (2.0 * l + 1) * ((double)l * (l + 1) * ct - (double)m * n) * v -
                 (l + 1.0) * sqrt(((double)l * l - (double)m * m) * ((double)l * l - (double)n * n)) * vprev;
    double den = l * sqrt(((l + 1.0) * (l + 1) - (double)m * m) * ((l + 1.0) * (l + 1) - (double)n * n));
    vprev = v;
    v = num / den;
    if (fabs(v) > 0x1p600) {
      v = ldexp(v, -600);
      vprev = ldexp(vprev, -600);
      E += 600;
    }
    out[l + 1] = ldexp(v, E);
  }
}

/* ------------------------------------------------------------------------ */
/* Delta contraction helpers                                                */
/* ------------------------------------------------------------------------ */

/* P[mp] = Delta^l_{mp,n} for mp = 0..l, from the quadrant (rows are first index). */
static void delta_column(double *P, const double *D, int l, int n) {
  const int w = l + 1;
  int an = abs(n);
  for (int mp = 0; mp <= l; ++mp) {
    /* Delta_{mp,an} = (-1)^{an-mp} Delta_{an,mp} = (-1)^{an-mp} D[an][mp] */
    double v = neg1(an - mp) * D[(size_t)an * w + mp];
    if (n < 0) v *= neg1(l + mp); /* Delta_{mp,-k} = (-1)^{l+mp} Delta_{mp,k} */
    P[mp] = v;
  }
}

/*
 * Row access for Delta_{mp,m} over mp with the sign folded:
 *   m >= 0:  Delta_{mp,m} = (-1)^{mp+m} D[m][mp]
 *   m <  0:  Delta_{mp,m} = (-1)^{l+|m|} D[|m|][mp]
 * Returned as (row pointer, constant factor, alternate flag).
 */
/* ------------------------------------------------------------------------ */
/* Sampling grids                                                           */
/* ------------------------------------------------------------------------ */

/*
 * MW   (McEwen & Wiaux 2011): theta_t = pi (2t+1)/(2L-1), t < L;  phi_p = 2 pi p/(2L-1).
 * MWSS (the symmetric variant): theta_t = pi t / L, t <= L (both poles);
 *      phi_p = 2 pi p/(2L).
 * The rings and their mirror images theta -> 2 pi - theta are kt equispaced
 * samples of the full theta circle: kt = 2L-1 starting half a step in (MW) or
 * kt = 2L starting at theta = 0 (MWSS).  A band-limited m-signal extends to the
 * circle with parity (-1)^{m+s}, and the kt samples give its Fourier
 * coefficients m' in [-(L-1), L-1] exactly.  With an even number of samples
 * (MWSS) the Nyquist bins (m' = L on the circle, m = L on a ring) are not
 * harmonic content of a band-limited signal and are dropped.
 */
typedef struct {
  int L, ss;
  int nt; /* rings */
  int np; /* samples per ring = phi-DFT length */
  int kt; /* samples on the full theta circle = theta-DFT length */
} grid_t;

static grid_t grid_of(int L, int ss) {
  grid_t g;
  g.L = L;
  g.ss = ss;
  g.nt = ss ? L + 1 : L;
  g.np = ss ? 2 * L : 2 * L - 1;
  g.kt = ss ? 2 * L : 2 * L - 1;
  return g;
}

/* e^{i m' theta_0}: the MW rings start half a step into the circle */
static complex double theta_phase(const grid_t *g, int mp) {
  if (g->ss) return 1.0;
  double a = SPI * mp / g->kt;
  return cos(a) + I * sin(a);
}

/* position on the full circle of the mirror image of ring t, or -1 for the
 * rings that are their own mirror image (theta = 0 or pi) */
static int mirror_of(const grid_t *g, int t) {
  if (g->ss) return (t >= 1 && t <= g->L - 1) ? 2 * g->L - t : -1;
  return (t < g->L - 1) ? g->kt - 1 - t : -1;
}

/* quadrature scale of the forward transform: 2 pi (phi integral) over the two
 * unnormalised DFT lengths */
static double fwd_scale(const grid_t *g) { return 2.0 * SPI / ((double)g->np * g->kt); }

/* ------------------------------------------------------------------------ */
/* Fourier-space weight for the exact forward transform                     */
/* ------------------------------------------------------------------------ */

static complex double wsin(int p) {
  /* w(p) = int_0^pi e^{i p t} sin t dt */
  if (p == 1) return I * SPI / 2.0;
  if (p == -1) return -I * SPI / 2.0;
  if (p & 1) return 0.0;
  return 2.0 / (1.0 - (double)p * (double)p);
}

typedef struct conv_plan {
  int L, P;
  complex double *bhat;  /* FFT of w(q-(2L-2)),       q in [0,4L-4] */
  complex double *bhatc; /* FFT of conj(w(q-(2L-2))) */
} conv_plan;

static _Thread_local conv_plan cp_cache[8];
static _Thread_local int cp_count;

static conv_plan *get_conv(int L) {
  for (int i = 0; i < cp_count; ++i)
    if (cp_cache[i].L == L) return &cp_cache[i];
  conv_plan *c = (cp_count < 8) ? &cp_cache[cp_count++] : &cp_cache[7];
  int P = 1;
  while (P < 4 * L - 3) P <<= 1;
  c->L = L;
  c->P = P;
  c->bhat = (complex double *)xcalloc(P, sizeof(complex double));
  c->bhatc = (complex double *)xcalloc(P, sizeof(complex double));
  for (int q = 0; q <= 4 * L - 4; ++q) {
    c->bhat[q] = wsin(q - (2 * L - 2));
    c->bhatc[q] = conj(wsin(q - (2 * L - 2)));
  }
  offt_dft(c->bhat, P, -1);
  offt_dft(c->bhatc, P, -1);
  return c;
}

/* out_{j} = sum_{i} in_{i} W(i + j), i,j in [-(L-1), L-1]; arrays indexed by +L-1.
 * W = w (conj_w = 0) or conj(w) (conj_w = 1). */
static void wconv(complex double *out, const complex double *in, int L, int conj_w,
                  complex double *scratch /* P */) {
  conv_plan *c = get_conv(L);
  const int K = 2 * L - 1, P = c->P;
  memset(scratch, 0, sizeof(complex double) * P);
  for (int k = 0; k < K; ++k) scratch[k] = in[(L - 1) - k + (L - 1)]; /* in_{(L-1)-k} */
  offt_dft(scratch, P, -1);
  const complex double *bh = conj_w ? c->bhatc : c->bhat;
  for (int k = 0; k < P; ++k) scratch[k] *= bh[k];
  offt_dft(scratch, P, +1);
  double inv = 1.0 / (double)P;
  for (int j = -(L - 1); j <= L - 1; ++j) out[j + L - 1] = scratch[(j + 3 * L - 3) % P] * inv;
}

/* ------------------------------------------------------------------------ */
/* Multi-transform cores                                                    */
/* ------------------------------------------------------------------------ */

/*
 * Harmonic -> (m, m') Fourier coefficients for several spins at once.
 * F[j][mi*L + mp] = sum_l coef_l flm_j(l,m) Delta_{mp,m} Delta_{mp,n_j}, mp >= 0,
 * with coef_l = (-1)^s sqrt((2l+1)/4pi) i^{n-m} (inverse) or its conjugate
 * times the forward-adjoint scale (adjoint forward).  mode 0: inverse, 1: adjoint-forward.
 */
static void harm_to_mm(complex double **F, const complex double **flm, const int *spin,
                       int njob, const grid_t *g, int mlo, int mode) {
  const int L = g->L, K = 2 * L - 1;
  double *D = (double *)xcalloc((size_t)L * L, sizeof(double));
  double *Pn = (double *)xcalloc((size_t)L, sizeof(double));
  double *Pa = (double *)xcalloc((size_t)L, sizeof(double));
  for (int j = 0; j < njob; ++j) memset(F[j], 0, sizeof(complex double) * (size_t)K * L);
  int smin = L;
  for (int j = 0; j < njob; ++j) smin = abs(spin[j]) < smin ? abs(spin[j]) : smin;
  for (int l = smin; l < L; ++l) {
    oracle_delta_quadrant(D, l);
    const int w = l + 1;
    const double cl = sqrt((2.0 * l + 1.0) / (4.0 * SPI));
    for (int j = 0; j < njob; ++j) {
      const int s = spin[j], n = -s;
      if (l < abs(s)) continue;
      delta_column(Pn, D, l, n);
      for (int mp = 0; mp <= l; ++mp) Pa[mp] = neg1(mp) * Pn[mp];
      const int m0 = mlo > -l ? mlo : -l;
#pragma omp parallel for schedule(static) if (l >= 64)
      for (int m = m0; m <= l; ++m) {
        complex double a = flm[j][l * l + l + m];
        if (a == 0) continue;
        complex double ph = neg1(s) * cl * ipow(n - m);
        if (mode == 1) ph = conj(ph) * fwd_scale(g);
        a *= ph;
        complex double *row = F[j] + (size_t)(m + L - 1) * L;
        const double *drow = D + (size_t)abs(m) * w;
        if (m >= 0) {
          a *= neg1(m);
          for (int mp = 0; mp <= l; ++mp) row[mp] += a * (drow[mp] * Pa[mp]);
        } else {
          a *= neg1(l - m);
          for (int mp = 0; mp <= l; ++mp) row[mp] += a * (drow[mp] * Pn[mp]);
        }
      }
    }
  }
  free(D);
  free(Pn);
  free(Pa);
}

/*
 * (m, m') coefficients -> harmonic, for several spins at once.
 * flm_j(l,m) = scale_l sum_{mp>=0} Delta_{mp,m} Delta_{mp,n} G_j[mi*L+mp]
 * mode 0: forward (scale (-1)^s c_l i^{n-m} times the quadrature scale); mode 1:
 * adjoint-inverse (scale (-1)^s c_l i^{n-m}).
 */
static void mm_to_harm(complex double **flm, complex double **G, const int *spin, int njob,
                       const grid_t *g, int mlo, int mode) {
  const int L = g->L;
  double *D = (double *)xcalloc((size_t)L * L, sizeof(double));
  double *Pn = (double *)xcalloc((size_t)L, sizeof(double));
  double *Pa = (double *)xcalloc((size_t)L, sizeof(double));
  for (int j = 0; j < njob; ++j) memset(flm[j], 0, sizeof(complex double) * (size_t)L * L);
  int smin = L;
  for (int j = 0; j < njob; ++j) smin = abs(spin[j]) < smin ? abs(spin[j]) : smin;
  for (int l = smin; l < L; ++l) {
    oracle_delta_quadrant(D, l);
    const int w = l + 1;
    const double cl = sqrt((2.0 * l + 1.0) / (4.0 * SPI));
    for (int j = 0; j < njob; ++j) {
      const int s = spin[j], n = -s;
      if (l < abs(s)) continue;
      delta_column(Pn, D, l, n);
      for (int mp = 0; mp <= l; ++mp) Pa[mp] = neg1(mp) * Pn[mp];
      const int m0 = mlo > -l ? mlo : -l;
#pragma omp parallel for schedule(static) if (l >= 64)
      for (int m = m0; m <= l; ++m) {
        const complex double *row = G[j] + (size_t)(m + L - 1) * L;
        const double *drow = D + (size_t)abs(m) * w;
        complex double acc = 0;
        if (m >= 0) {
          for (int mp = 0; mp <= l; ++mp) acc += row[mp] * (drow[mp] * Pa[mp]);
          acc *= neg1(m);
        } else {
          for (int mp = 0; mp <= l; ++mp) acc += row[mp] * (drow[mp] * Pn[mp]);
          acc *= neg1(l - m);
        }
        complex double ph = neg1(s) * cl * ipow(n - m);
        if (mode == 0) ph *= fwd_scale(g);
        flm[j][l * l + l + m] = acc * ph;
      }
    }
  }
  free(D);
  free(Pn);
  free(Pa);
}

/* ------------------------------------------------------------------------ */
/* Inverse                                                                  */
/* ------------------------------------------------------------------------ */

/* F (m,mp>=0) -> map; real != 0 writes Re into fr, else complex into fc. */
static void mm_to_map(complex double *fc, double *fr, const complex double *F, const grid_t *g,
                      int s, int mlo) {
  const int L = g->L, n = -s, nt = g->nt, np = g->np, kt = g->kt;
  complex double *ring = (complex double *)xcalloc((size_t)nt * np, sizeof(complex double));
#pragma omp parallel if (L >= 64)
  {
  complex double *x = (complex double *)xcalloc(kt, sizeof(complex double));
#pragma omp for schedule(static)
  for (int m = mlo; m <= L - 1; ++m) {
    const complex double *row = F + (size_t)(m + L - 1) * L;
    memset(x, 0, sizeof(complex double) * kt);
    double sym = neg1(m + n);
    for (int mp = -(L - 1); mp <= L - 1; ++mp) {
      complex double v = (mp >= 0) ? row[mp] : sym * row[-mp];
      x[modk(mp, kt)] += v * theta_phase(g, mp);
    }
    offt_dft(x, kt, +1);
    for (int t = 0; t < nt; ++t) ring[(size_t)t * np + modk(m, np)] = x[t];
  }
  free(x);
  }
#pragma omp parallel for schedule(static) if (L >= 64)
  for (int t = 0; t < nt; ++t) {
    complex double *r = ring + (size_t)t * np;
    if (mlo == 0) /* Hermitian completion for a real signal */
      for (int m = 1; m <= L - 1; ++m) r[modk(-m, np)] = conj(r[m]);
    offt_dft(r, np, +1);
    for (int p = 0; p < np; ++p) {
      if (fr)
        fr[(size_t)t * np + p] = creal(r[p]);
      else
        fc[(size_t)t * np + p] = r[p];
    }
  }
  free(ring);
}

void oracle_ssht_inverse_multi(void **f, const complex double **flm, const int *spin,
                               const int *real, int njob, int L, int ss) {
  const grid_t g = grid_of(L, ss);
  const int K = 2 * L - 1;
  complex double **F = (complex double **)xcalloc(njob, sizeof(void *));
  for (int j = 0; j < njob; ++j) F[j] = (complex double *)xcalloc((size_t)K * L, sizeof(complex double));
  int allreal = 1;
  for (int j = 0; j < njob; ++j) allreal &= real[j] != 0;
  harm_to_mm(F, flm, spin, njob, &g, allreal ? 0 : -(L - 1), 0);
  for (int j = 0; j < njob; ++j) {
    if (real[j])
      mm_to_map(NULL, (double *)f[j], F[j], &g, spin[j], 0);
    else
      mm_to_map((complex double *)f[j], NULL, F[j], &g, spin[j], -(L - 1));
    free(F[j]);
  }
  free(F);
}

/* ------------------------------------------------------------------------ */
/* Forward                                                                  */
/* ------------------------------------------------------------------------ */

/* map -> per-m ring spectra Fm[mi*nt + t] (unnormalised phi-DFT). */
static void map_to_rings(complex double *Fm, const complex double *fc, const double *fr,
                         const grid_t *g) {
  const int L = g->L, nt = g->nt, np = g->np;
#pragma omp parallel if (L >= 64)
  {
    complex double *x = (complex double *)xcalloc(np, sizeof(complex double));
#pragma omp for schedule(static)
    for (int t = 0; t < nt; ++t) {
      for (int p = 0; p < np; ++p) x[p] = fr ? fr[(size_t)t * np + p] : fc[(size_t)t * np + p];
      offt_dft(x, np, -1);
      for (int m = -(L - 1); m <= L - 1; ++m) Fm[(size_t)(m + L - 1) * nt + t] = x[modk(m, np)];
    }
    free(x);
  }
}

/* per-m ring spectra -> G (mp >= 0, symmetrised) for the forward contraction */
static void rings_to_G(complex double *G, const complex double *Fm, const grid_t *g, int s, int mlo) {
  const int L = g->L, K = 2 * L - 1, n = -s, nt = g->nt, kt = g->kt;
  memset(G, 0, sizeof(complex double) * (size_t)K * L);
#pragma omp parallel if (L >= 64)
  {
  conv_plan *cp = get_conv(L);
  complex double *ext = (complex double *)xcalloc(kt, sizeof(complex double));
  complex double *Fh = (complex double *)xcalloc(K, sizeof(complex double));
  complex double *Gf = (complex double *)xcalloc(K, sizeof(complex double));
  complex double *scr = (complex double *)xcalloc(cp->P, sizeof(complex double));
#pragma omp for schedule(static)
  for (int m = mlo; m <= L - 1; ++m) {
    const complex double *Fr = Fm + (size_t)(m + L - 1) * nt;
    double eps = neg1(m + s);
    /* extension to the full circle with parity eps */
    memset(ext, 0, sizeof(complex double) * kt);
    for (int t = 0; t < nt; ++t) {
      ext[t] = Fr[t];
      const int mt = mirror_of(g, t);
      if (mt >= 0) ext[mt] = eps * Fr[t];
    }
    offt_dft(ext, kt, -1);
    for (int mp = -(L - 1); mp <= L - 1; ++mp) Fh[mp + L - 1] = ext[modk(mp, kt)] * conj(theta_phase(g, mp));
    wconv(Gf, Fh, L, 0, scr);
    complex double *gr = G + (size_t)(m + L - 1) * L;
    double sym = neg1(m + n);
    gr[0] = Gf[L - 1];
    for (int mp = 1; mp <= L - 1; ++mp) gr[mp] = Gf[mp + L - 1] + sym * Gf[-mp + L - 1];
  }
  free(ext);
  free(Fh);
  free(Gf);
  free(scr);
  }
}

void oracle_ssht_forward_multi(complex double **flm, const void **f, const int *spin,
                               const int *real, int njob, int L, int ss) {
  const grid_t g = grid_of(L, ss);
  const int K = 2 * L - 1;
  complex double *Fm = (complex double *)xcalloc((size_t)K * g.nt, sizeof(complex double));
  complex double **G = (complex double **)xcalloc(njob, sizeof(void *));
  int allreal = 1;
  for (int j = 0; j < njob; ++j) allreal &= real[j] != 0;
  for (int j = 0; j < njob; ++j) {
    G[j] = (complex double *)xcalloc((size_t)K * L, sizeof(complex double));
    if (real[j])
      map_to_rings(Fm, NULL, (const double *)f[j], &g);
    else
      map_to_rings(Fm, (const complex double *)f[j], NULL, &g);
    rings_to_G(G[j], Fm, &g, spin[j], real[j] ? 0 : -(L - 1));
  }
  mm_to_harm(flm, G, spin, njob, &g, allreal ? 0 : -(L - 1), 0);
  for (int j = 0; j < njob; ++j) {
    if (real[j])
      for (int l = 0; l < L; ++l)
        for (int m = 1; m <= l; ++m) flm[j][l * l + l - m] = neg1(m) * conj(flm[j][l * l + l + m]);
    free(G[j]);
  }
  free(G);
  free(Fm);
}

/* ------------------------------------------------------------------------ */
/* Adjoint of the inverse: a_lm = sum_{t,p} f(t,p) conj(sY_lm(t,p))         */
/* ------------------------------------------------------------------------ */

static void rings_to_H(complex double *H, const complex double *Fm, const grid_t *g, int s, int mlo) {
  const int L = g->L, K = 2 * L - 1, n = -s, nt = g->nt, kt = g->kt;
  memset(H, 0, sizeof(complex double) * (size_t)K * L);
#pragma omp parallel if (L >= 64)
  {
  complex double *x = (complex double *)xcalloc(kt, sizeof(complex double));
#pragma omp for schedule(static)
  for (int m = mlo; m <= L - 1; ++m) {
    const complex double *Fr = Fm + (size_t)(m + L - 1) * nt;
    memset(x, 0, sizeof(complex double) * kt);
    for (int t = 0; t < nt; ++t) x[t] = Fr[t];
    offt_dft(x, kt, +1);
    complex double *h = H + (size_t)(m + L - 1) * L;
    double sym = neg1(m + n);
    for (int mp = 0; mp <= L - 1; ++mp) {
      h[mp] = x[modk(mp, kt)] * theta_phase(g, mp);
      if (mp > 0) h[mp] += sym * x[modk(-mp, kt)] * theta_phase(g, -mp);
    }
  }
  free(x);
  }
}

void oracle_ssht_adjoint_inverse_multi(complex double **flm, const void **f, const int *spin,
                                       const int *real, int njob, int L, int ss) {
  const grid_t g = grid_of(L, ss);
  const int K = 2 * L - 1;
  complex double *Fm = (complex double *)xcalloc((size_t)K * g.nt, sizeof(complex double));
  complex double **H = (complex double **)xcalloc(njob, sizeof(void *));
  int allreal = 1;
  for (int j = 0; j < njob; ++j) allreal &= real[j] != 0;
  for (int j = 0; j < njob; ++j) {
    H[j] = (complex double *)xcalloc((size_t)K * L, sizeof(complex double));
    if (real[j])
      map_to_rings(Fm, NULL, (const double *)f[j], &g);
    else
      map_to_rings(Fm, (const complex double *)f[j], NULL, &g);
    rings_to_H(H[j], Fm, &g, spin[j], real[j] ? 0 : -(L - 1));
  }
  mm_to_harm(flm, H, spin, njob, &g, allreal ? 0 : -(L - 1), 1);
  for (int j = 0; j < njob; ++j) {
    if (real[j])
      for (int l = 0; l < L; ++l)
        for (int m = 1; m <= l; ++m) flm[j][l * l + l - m] = neg1(m) * conj(flm[j][l * l + l + m]);
    free(H[j]);
  }
  free(H);
  free(Fm);
}

/* ------------------------------------------------------------------------ */
/* Adjoint of the forward                                                   */
/* ------------------------------------------------------------------------ */

static void G_to_map_adj(complex double *fc, double *fr, const complex double *Gs, const grid_t *g,
                         int s, int mlo) {
  const int L = g->L, K = 2 * L - 1, n = -s, nt = g->nt, np = g->np, kt = g->kt;
  complex double *ring = (complex double *)xcalloc((size_t)nt * np, sizeof(complex double));
#pragma omp parallel if (L >= 64)
  {
  conv_plan *cp = get_conv(L);
  complex double *Gf = (complex double *)xcalloc(K, sizeof(complex double));
  complex double *Fh = (complex double *)xcalloc(K, sizeof(complex double));
  complex double *x = (complex double *)xcalloc(kt, sizeof(complex double));
  complex double *scr = (complex double *)xcalloc(cp->P, sizeof(complex double));
#pragma omp for schedule(static)
  for (int m = mlo; m <= L - 1; ++m) {
    const complex double *gr = Gs + (size_t)(m + L - 1) * L;
    double sym = neg1(m + n);
    for (int mp = 0; mp <= L - 1; ++mp) {
      Gf[mp + L - 1] = gr[mp];
      if (mp > 0) Gf[-mp + L - 1] = sym * gr[mp];
    }
    wconv(Fh, Gf, L, 1, scr);
    memset(x, 0, sizeof(complex double) * kt);
    for (int mp = -(L - 1); mp <= L - 1; ++mp) x[modk(mp, kt)] += Fh[mp + L - 1] * theta_phase(g, mp);
    offt_dft(x, kt, +1); /* x[k] = adjoint of the theta DFT at circle position k */
    double eps = neg1(m + s);
    for (int t = 0; t < nt; ++t) {
      complex double v = x[t];
      const int mt = mirror_of(g, t);
      if (mt >= 0) v += eps * x[mt];
      ring[(size_t)t * np + modk(m, np)] = v;
    }
  }
  free(Gf);
  free(Fh);
  free(x);
  free(scr);
  }
#pragma omp parallel for schedule(static) if (L >= 64)
  for (int t = 0; t < nt; ++t) {
    complex double *r = ring + (size_t)t * np;
    offt_dft(r, np, +1);
    for (int p = 0; p < np; ++p) {
      if (fr)
        fr[(size_t)t * np + p] = creal(r[p]);
      else
        fc[(size_t)t * np + p] = r[p];
    }
  }
  free(ring);
}

void oracle_ssht_adjoint_forward_multi(void **f, const complex double **flm, const int *spin,
                                       const int *real, int njob, int L, int ss) {
  const grid_t g = grid_of(L, ss);
  const int K = 2 * L - 1;
  complex double **G = (complex double **)xcalloc(njob, sizeof(void *));
  for (int j = 0; j < njob; ++j) G[j] = (complex double *)xcalloc((size_t)K * L, sizeof(complex double));
  /* the real adjoint is Re of the complex adjoint: all m are needed */
  harm_to_mm(G, flm, spin, njob, &g, -(L - 1), 1);
  for (int j = 0; j < njob; ++j) {
    if (real[j])
      G_to_map_adj(NULL, (double *)f[j], G[j], &g, spin[j], -(L - 1));
    else
      G_to_map_adj((complex double *)f[j], NULL, G[j], &g, spin[j], -(L - 1));
    free(G[j]);
  }
  free(G);
}

/* ------------------------------------------------------------------------ */
/* Public single-transform entry points (MW and MWSS)                       */
/* ------------------------------------------------------------------------ */

static void one_inverse(void *f, const complex double *flm, int L, int spin, int real, int ss) {
  void *fo[1] = {f};
  const complex double *fi[1] = {flm};
  int sp[1] = {spin}, re[1] = {real};
  oracle_ssht_inverse_multi(fo, fi, sp, re, 1, L, ss);
}
static void one_forward(complex double *flm, const void *f, int L, int spin, int real, int ss) {
  complex double *fo[1] = {flm};
  const void *fi[1] = {f};
  int sp[1] = {spin}, re[1] = {real};
  oracle_ssht_forward_multi(fo, fi, sp, re, 1, L, ss);
}
static void one_adjoint_inverse(complex double *flm, const void *f, int L, int spin, int real, int ss) {
  complex double *fo[1] = {flm};
  const void *fi[1] = {f};
  int sp[1] = {spin}, re[1] = {real};
  oracle_ssht_adjoint_inverse_multi(fo, fi, sp, re, 1, L, ss);
}
static void one_adjoint_forward(void *f, const complex double *flm, int L, int spin, int real, int ss) {
  void *fo[1] = {f};
  const complex double *fi[1] = {flm};
  int sp[1] = {spin}, re[1] = {real};
  oracle_ssht_adjoint_forward_multi(fo, fi, sp, re, 1, L, ss);
}

#define UNUSED_DL (void)dl_method, (void)verbosity

void ssht_core_mw_inverse_sov_sym(complex double *f, const complex double *flm, int L, int spin,
                                  ssht_dl_method_t dl_method, int verbosity) {
  UNUSED_DL;
  one_inverse(f, flm, L, spin, 0, 0);
}
void ssht_core_mw_inverse_sov_sym_real(double *f, const complex double *flm, int L,
                                       ssht_dl_method_t dl_method, int verbosity) {
  UNUSED_DL;
  one_inverse(f, flm, L, 0, 1, 0);
}
void ssht_core_mw_forward_sov_conv_sym(complex double *flm, const complex double *f, int L,
                                       int spin, ssht_dl_method_t dl_method, int verbosity) {
  UNUSED_DL;
  one_forward(flm, f, L, spin, 0, 0);
}
void ssht_core_mw_forward_sov_conv_sym_real(complex double *flm, const double *f, int L,
                                            ssht_dl_method_t dl_method, int verbosity) {
  UNUSED_DL;
  one_forward(flm, f, L, 0, 1, 0);
}
void ssht_adjoint_mw_inverse_sov_sym(complex double *flm, const complex double *f, int L,
                                     int spin, ssht_dl_method_t dl_method, int verbosity) {
  UNUSED_DL;
  one_adjoint_inverse(flm, f, L, spin, 0, 0);
}
void ssht_adjoint_mw_inverse_sov_sym_real(complex double *flm, const double *f, int L,
                                          ssht_dl_method_t dl_method, int verbosity) {
  UNUSED_DL;
  one_adjoint_inverse(flm, f, L, 0, 1, 0);
}
void ssht_adjoint_mw_forward_sov_sym(complex double *f, const complex double *flm, int L,
                                     int spin, ssht_dl_method_t dl_method, int verbosity) {
  UNUSED_DL;
  one_adjoint_forward(f, flm, L, spin, 0, 0);
}
void ssht_adjoint_mw_forward_sov_sym_real(double *f, const complex double *flm, int L,
                                          ssht_dl_method_t dl_method, int verbosity) {
  UNUSED_DL;
  one_adjoint_forward(f, flm, L, 0, 1, 0);
}

/* MWSS: the same operators on the symmetric grid */
void ssht_core_mw_inverse_sov_sym_ss(complex double *f, const complex double *flm, int L, int spin,
                                     ssht_dl_method_t dl_method, int verbosity) {
  UNUSED_DL;
  one_inverse(f, flm, L, spin, 0, 1);
}
void ssht_core_mw_inverse_sov_sym_ss_real(double *f, const complex double *flm, int L,
                                          ssht_dl_method_t dl_method, int verbosity) {
  UNUSED_DL;
  one_inverse(f, flm, L, 0, 1, 1);
}
void ssht_core_mw_forward_sov_conv_sym_ss(complex double *flm, const complex double *f, int L,
                                          int spin, ssht_dl_method_t dl_method, int verbosity) {
  UNUSED_DL;
  one_forward(flm, f, L, spin, 0, 1);
}
void ssht_core_mw_forward_sov_conv_sym_ss_real(complex double *flm, const double *f, int L,
                                               ssht_dl_method_t dl_method, int verbosity) {
  UNUSED_DL;
  one_forward(flm, f, L, 0, 1, 1);
}
void ssht_adjoint_mw_inverse_sov_sym_ss(complex double *flm, const complex double *f, int L,
                                        int spin, ssht_dl_method_t dl_method, int verbosity) {
  UNUSED_DL;
  one_adjoint_inverse(flm, f, L, spin, 0, 1);
}
void ssht_adjoint_mw_inverse_sov_sym_ss_real(complex double *flm, const double *f, int L,
                                             ssht_dl_method_t dl_method, int verbosity) {
  UNUSED_DL;
  one_adjoint_inverse(flm, f, L, 0, 1, 1);
}
void ssht_adjoint_mw_forward_sov_sym_ss(complex double *f, const complex double *flm, int L,
                                        int spin, ssht_dl_method_t dl_method, int verbosity) {
  UNUSED_DL;
  one_adjoint_forward(f, flm, L, spin, 0, 1);
}
void ssht_adjoint_mw_forward_sov_sym_ss_real(double *f, const complex double *flm, int L,
                                             ssht_dl_method_t dl_method, int verbosity) {
  UNUSED_DL;
  one_adjoint_forward(f, flm, L, 0, 1, 1);
}
