/* ORACLE / TEST INFRASTRUCTURE ONLY: arbitrary-length complex DFT. */
#ifndef ORACLE_OFFT_H
#define ORACLE_OFFT_H
#include <complex.h>

/* In-place unnormalised DFT: X_k = sum_j x_j exp(sign * 2 pi i j k / n). */
void offt_dft(complex double *x, int n, int sign);

#endif
