// Host-side FP64 part of the wavelet transforms: tiling kernels, sizes and the
// per-scale layout of the wavelet coefficients.  Everything here is O(J L^2) or
// less and runs once per parameter set; the results are cached and uploaded.
#pragma once

#include <complex>
#include <cstdint>
#include <vector>

#include "s2let_gpu.h"

namespace s2g {

using cplx = std::complex<double>;

// Wigner-space storage of one scale: the SO3 "compact, n negative first" layout
// (n >= 0 only for real signals) that s2let_analysis_lm2lmn writes.
struct SO3Shape {
  int L = 0, N = 0, reality = 0, n_mode_odd = 0, mwss = 0;
  int64_t flmn_size() const;
  // (2N-1) gamma samples times the (alpha, beta) grid of the MW / MWSS sampling
  int64_t f_size() const { return (int64_t)(2 * N - 1) * (mwss ? (int64_t)2 * L * (L + 1) : (int64_t)L * (2 * L - 1)); }
  int64_t index(int l, int m, int n) const;       // complex storage
  int64_t index_real(int l, int m, int n) const;  // n >= 0 storage
};

// One parameter set's multiresolution bookkeeping, reproducing the reference's
// arithmetic (band-limits from ceil(pow(B, j+1)), N_j = min(N, bl) with the
// parity fix, offsets advancing with N_j).
struct Layout {
  int L = 0, N = 0, J = 0, J_min = 0, spin = 0, upsample = 0, real = 0, bl_scal = 0;
  std::vector<int> j, bl, Nj;
  std::vector<SO3Shape> so3;
  std::vector<int64_t> woff, loff;  // size nscale+1
  int nscale() const { return (int)j.size(); }
  // directions n of scale k that the transforms visit (n >= 0 for real signals)
  std::vector<int> directions(int k) const;
};

Layout make_layout(const s2let_parameters_t &p, bool real);

// Tiling: psi[(J+1) L^2] complex, phi[L] (src/c/s2let_tiling.c:381-429).
void tiling_wavelet(cplx *psi, double *phi, const s2let_parameters_t &p);
// Axisymmetric kernels wav_lm[(J+1) L], scal_lm[L] (src/c/s2let_transform_axisym_lm.c:91-118).
void axisym_kernels(double *wav_lm, double *scal_lm, const s2let_parameters_t &p);

int j_max(const s2let_parameters_t &p);
int bandlimit(int j, const s2let_parameters_t &p);

// Validation shared by every entry point; throws s2g::Error.  check_sampling:
// the sampling scheme must be MW or MWSS (the entry points whose reference
// counterpart reads it).
void validate(const s2let_parameters_t *p, bool check_sampling = true);

}  // namespace s2g
