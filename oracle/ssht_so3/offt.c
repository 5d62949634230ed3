/*
 * ORACLE / TEST INFRASTRUCTURE ONLY.  Not part of the GPU product path.
 *
 * Arbitrary-length complex DFT used by the CPU oracle's restatement of the
 * SSHT/SO3 transforms.  The reference obtains its FFTs from FFTW3 through SSHT
 * and SO3 (external to the reference tree; see the FFTW calls inside SSHT that
 * s2let reaches through ssht_core_* at src/c/s2let_analysis.c:471).  This file
 * restates the textbook algorithms instead:
 *   - iterative radix-2 Cooley-Tukey for power-of-two lengths,
 *   - Bluestein's chirp-z reformulation for every other length, with the chirp
 *     convolution evaluated by a power-of-two FFT,
 *   - a direct O(n^2) sum for tiny lengths.
 * Plans are cached per thread and per length.
 */
#include "offt.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define OFFT_PI 3.14159265358979323846264338327950288

typedef struct pow2_plan {
  int n;
  complex double *tw; /* tw[k] = exp(-2 pi i k / n), k < n/2 */
  int *rev;
} pow2_plan;

typedef struct blue_plan {
  int n, p;
  complex double *chirp;  /* exp(i pi k^2 / n), k < n            */
  complex double *bhat;   /* FFT_p of the wrapped chirp kernel   */
  complex double *work;   /* p scratch                           */
} blue_plan;

#define OFFT_CACHE 24
static _Thread_local pow2_plan *p2_cache[OFFT_CACHE];
static _Thread_local int p2_count;
static _Thread_local blue_plan *bl_cache[OFFT_CACHE];
static _Thread_local int bl_count;

static pow2_plan *get_pow2(int n) {
  for (int i = 0; i < p2_count; ++i)
    if (p2_cache[i]->n == n) return p2_cache[i];
  pow2_plan *pl = (pow2_plan *)malloc(sizeof *pl);
  pl->n = n;
  pl->tw = (complex double *)malloc(sizeof(complex double) * (n / 2 > 0 ? n / 2 : 1));
  for (int k = 0; k < n / 2; ++k) {
    double a = -2.0 * OFFT_PI * (double)k / (double)n;
    pl->tw[k] = cos(a) + I * sin(a);
  }
  pl->rev = (int *)malloc(sizeof(int) * n);
  int bits = 0;
  while ((1 << bits) < n) ++bits;
  for (int k = 0; k < n; ++k) {
    int r = 0;
    for (int b = 0; b < bits; ++b)
      if (k & (1 << b)) r |= 1 << (bits - 1 - b);
    pl->rev[k] = r;
  }
  if (p2_count < OFFT_CACHE) p2_cache[p2_count++] = pl;
  return pl; /* beyond the cache size the plan leaks; lengths per process are few */
}

/* in-place radix-2 FFT; sign = -1 forward, +1 backward (unnormalised) */
static void fft_pow2(complex double *x, int n, int sign) {
  if (n <= 1) return;
  pow2_plan *pl = get_pow2(n);
  for (int k = 0; k < n; ++k) {
    int r = pl->rev[k];
    if (r > k) {
      complex double t = x[k];
      x[k] = x[r];
      x[r] = t;
    }
  }
  for (int len = 2; len <= n; len <<= 1) {
    int half = len >> 1, step = n / len;
    for (int start = 0; start < n; start += len) {
      for (int j = 0; j < half; ++j) {
        complex double w = pl->tw[j * step];
        if (sign > 0) w = conj(w);
        complex double u = x[start + j];
        complex double v = x[start + j + half] * w;
        x[start + j] = u + v;
        x[start + j + half] = u - v;
      }
    }
  }
}

static int is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

static blue_plan *get_blue(int n) {
  for (int i = 0; i < bl_count; ++i)
    if (bl_cache[i]->n == n) return bl_cache[i];
  blue_plan *pl = (blue_plan *)malloc(sizeof *pl);
  int p = 1;
  while (p < 2 * n - 1) p <<= 1;
  pl->n = n;
  pl->p = p;
  pl->chirp = (complex double *)malloc(sizeof(complex double) * n);
  for (long k = 0; k < n; ++k) {
    long q = (k * k) % (2L * n); /* keep the angle argument small */
    double a = OFFT_PI * (double)q / (double)n;
    pl->chirp[k] = cos(a) + I * sin(a);
  }
  pl->bhat = (complex double *)calloc(p, sizeof(complex double));
  pl->bhat[0] = pl->chirp[0];
  for (int k = 1; k < n; ++k) {
    pl->bhat[k] = pl->chirp[k];
    pl->bhat[p - k] = pl->chirp[k];
  }
  fft_pow2(pl->bhat, p, -1);
  pl->work = (complex double *)malloc(sizeof(complex double) * p);
  if (bl_count < OFFT_CACHE) bl_cache[bl_count++] = pl;
  return pl;
}

/*
 * Bluestein: X_k = sum_j x_j e^{-2 pi i jk/n}
 *          = conj(c_k) sum_j (x_j conj(c_j)) c_{k-j},  c_j = e^{i pi j^2/n}.
 */
static void dft_bluestein(complex double *x, int n, int sign) {
  blue_plan *pl = get_blue(n);
  int p = pl->p;
  complex double *a = pl->work;
  memset(a, 0, sizeof(complex double) * p);
  if (sign < 0) {
    for (int j = 0; j < n; ++j) a[j] = x[j] * conj(pl->chirp[j]);
  } else { /* backward transform = conj(forward(conj(x))) */
    for (int j = 0; j < n; ++j) a[j] = conj(x[j]) * conj(pl->chirp[j]);
  }
  fft_pow2(a, p, -1);
  for (int k = 0; k < p; ++k) a[k] *= pl->bhat[k];
  fft_pow2(a, p, +1);
  double inv = 1.0 / (double)p;
  for (int k = 0; k < n; ++k) {
    complex double v = a[k] * inv * conj(pl->chirp[k]);
    x[k] = (sign < 0) ? v : conj(v);
  }
}

static void dft_direct(complex double *x, int n, int sign) {
  complex double tmp[16];
  for (int k = 0; k < n; ++k) {
    complex double s = 0;
    for (int j = 0; j < n; ++j) {
      long q = ((long)j * k) % n;
      double a = (double)sign * 2.0 * OFFT_PI * (double)q / (double)n;
      s += x[j] * (cos(a) + I * sin(a));
    }
    tmp[k] = s;
  }
  memcpy(x, tmp, sizeof(complex double) * n);
}

void offt_dft(complex double *x, int n, int sign) {
  if (n <= 1) return;
  if (is_pow2(n))
    fft_pow2(x, n, sign);
  else if (n <= 16)
    dft_direct(x, n, sign);
  else
    dft_bluestein(x, n, sign);
}
