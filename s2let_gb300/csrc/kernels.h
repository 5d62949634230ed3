// Launch wrappers of the transform kernels (FP64 path).  All pointers are
// device pointers; every wrapper is asynchronous on `st`.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "plan.h"

namespace s2g {

// Ring DFTs over a batch of rings of length K = grid_ring_len(bl, ss)
// (2bl-1 on MW, 2bl on MWSS sampling).
//   forward:  spec[r][m - mlo] = sum_p ring_r[p] e^{-2 pi i m p / K},  m in [mlo, bl-1]
//   inverse:  ring_r[p] = sum_m spec[r][m - mlo] e^{+2 pi i m p / K}   (MWSS: no m = bl term)
// real != 0: rings are real; spectra hold m >= 0 only (mlo = 0) and are
// Hermitian-completed on the inverse.  Spectrum rows have width `sw`.
// Ring r lives at (r / rpm) * map_stride + (r % rpm) * ring_stride elements.
void ring_forward(const void *rings, int64_t ring_stride, int64_t map_stride, int rpm, double2 *spec,
                  int64_t spec_stride, int sw, int mlo, int nrings, int bl, int ss, bool real, cudaStream_t st);
void ring_inverse(const double2 *spec, int64_t spec_stride, int sw, int mlo, void *rings,
                  int64_t ring_stride, int64_t map_stride, int rpm, int nrings, int bl, int ss, bool real,
                  cudaStream_t st);

// Contraction over l producing ring spectra ("l -> t", t < tb->nt):
//   out[b][t][m - omlo] = sum_l A_m[t][l] x_b(l, m) w(l)
// A = D (use_q = false) or Q^T (use_q = true) of the |n| table at band-limit bl,
// read at direction n (sign/mirror for n < 0).  x_b(l,m) = x[b*xs + l^2+l+m]
// (band-limit xL >= bl); when x_half, x holds m >= 0 only and
// x(l,-m) = (-1)^m conj(x(l,m)).  w(l) = wre/wim arrays (nullable => 1) times
// wscale, conjugated when wconj.  Rows l < lmin contribute nothing.
// Complex rings with two-level spectrum addressing: spectrum of ring r at
// spec + (r / spec_rpm) * spec_map_stride + (r % spec_rpm) * spec_stride.
// herm (inverse): columns m < 0 are conj of m > 0 (a real-valued ring held as complex).
void ring_forward_c(const double2 *rings, int64_t ring_stride, int64_t map_stride, int rpm, double2 *spec,
                    int64_t spec_stride, int64_t spec_map_stride, int spec_rpm, int sw, int mlo, int nrings, int bl,
                    int ss, cudaStream_t st);
void ring_inverse_c(const double2 *spec, int64_t spec_stride, int64_t spec_map_stride, int spec_rpm, int sw,
                    int mlo, bool herm, double2 *rings, int64_t ring_stride, int64_t map_stride, int rpm, int nrings,
                    int bl, int ss, cudaStream_t st);

// Kind of a per-l weight array: every entry real, every entry imaginary, or
// general complex.  The directional weights are a real profile times 1 or i
// (odd or even N), the axisymmetric and scaling weights are real.
enum { WKIND_COMPLEX = 0, WKIND_REAL = 1, WKIND_IMAG = 2 };

struct L2T {
  const WignerTable *tb;
  int n;
  bool use_q;
  int mlo, mhi;  // m range computed
  const double2 *x;
  int64_t xs;
  int xL;
  bool x_half;
  const double2 *w;  // per-l weight (length >= bl) or nullptr
  double wscale;
  bool wconj;
  int wkind;  // WKIND_* of w: lets the kernels multiply by a real or imaginary weight with 2 products
  int lmin;
  double2 *out;
  int64_t os;  // batch stride of out
  int ow;      // row width (per t) of out
  int omlo;    // m of column 0
  int nb;
};
// double-float copies of the stored Wigner tables (split-precision
// contractions on the FP32 pipe): freed with the plans; on/off switch
void release_df_tables();
size_t df_table_bytes();
void set_split_tables(int on);
int get_split_tables();
// split precision: batches of at most this many maps (0-4) contract in
// double-float on the FP64 tables instead of on the tensor cores
void set_df_max_maps(int maps);
int get_df_max_maps();

void contract_l2t(const L2T &a, cudaStream_t st);
// n problems on the same table (same band-limit, n, m range and batch): one
// table pass on the split-precision path when n <= 2, else one call each.
void contract_l2t_group(const L2T *a, int n, cudaStream_t st);

// Contraction over t producing harmonic coefficients ("t -> l"):
//   y[b*ys + l^2+l+m] = w(l) sum_t A_m[l][t] in[b][t][m - imlo]
// A = Q (use_q = true) or D^T (use_q = false).  Overwrites y for l in
// [max(l0(m), lmin), bl) and m in [mlo, mhi]; other entries untouched.
struct T2L {
  const WignerTable *tb;
  int n;
  bool use_q;
  int mlo, mhi;
  const double2 *in;
  int64_t is;
  int iw;
  int imlo;
  const double2 *w;
  double wscale;
  bool wconj;
  int wkind;  // WKIND_* of w
  int lmin;
  double2 *y;
  int64_t ys;
  int nb;
};
void contract_t2l(const T2L &a, cudaStream_t st);
void contract_t2l_group(const T2L *a, int n, cudaStream_t st);

// gamma synthesis: spec[b][g][t][m - (real?0:-(bl-1))] from coefficients
// G[b][k][t][m + bl - 1] of directions ns[k], t < grid_rings(bl, ss); real:
// Hermitian in (m, n).
//   spec_g(m) = c sum_k e^{i n_k gamma_g} G_k(m)  (+ conj mirror for real n > 0)
void gamma_synthesis(const double2 *G, double2 *spec, const int *ns, int nn, int ng, int bl, int ss, int nb,
                     bool real, double c, cudaStream_t st);
// gamma analysis: G[b][k][t][m + bl - 1] = c sum_g e^{-i n_k gamma_g} spec_g(m), all m.
void gamma_analysis(const double2 *spec, double2 *G, const int *ns, int nn, int ng, int bl, int ss, int nb,
                    bool real, double c, cudaStream_t st);
// gamma DFT on pixels between F[b][k][t][p] (complex, k < nn) and the gamma slices
// out[b * ms + g * npx + t * K + p] (double for real signals, else double2),
// npx = nt * K the pixels of one slice on the sampling's grid
void gamma_px_synthesis(const double2 *F, void *out, int64_t out_ms, const int *ns, int nn, int ng, int bl,
                        int ss, int nb, bool real, double c, cudaStream_t st);
void gamma_px_analysis(const void *in, int64_t in_ms, double2 *F, const int *ns, int nn, int ng, int bl, int ss,
                       int nb, bool real, double c, cudaStream_t st);

// Ring DFTs fused with the gamma DFT in one launch (split precision; a
// thread-block cluster per ring, one CTA per n-component), usable when
// ring_gamma_fusable(nn, ng, bl, ss): the split-precision path, 2 <= nn <= 8,
// nn ng <= 128, and a cluster of nn CTAs fits on this GPU (asked once per
// shape; otherwise the ring and gamma DFTs run as separate launches).
// Component k of ring (b, t), t < nt, has its
// spectrum at G + b gms + k gks + t W (W = 2bl-1, m from -(bl-1); on real
// signals the component with n = 0 holds m >= 0 at offset bl-1, the rest by
// Hermitian symmetry); gamma slice g of ring (b, t) lives at
// fw + b fms + g npx + t K (npx = nt K; double when real, else double2).
//   ring_inverse_gamma:  f_g = c sum_k e^{i n_k gamma_g} F_k (real: 2 Re for
//                        n_k > 0, Re for n_k = 0), F_k the inverse ring DFT
//   gamma_ring_forward:  F_k = c sum_g e^{-i n_k gamma_g} f_g, then the
//                        forward ring DFT of every F_k to G (all m)
bool ring_gamma_fusable(int nn, int ng, int bl, int ss);
void ring_inverse_gamma(const double2 *G, int64_t gms, int64_t gks, const std::vector<int> &ns, int ng, bool real,
                        double c, void *fw, int64_t fms, int nb, int bl, int ss, cudaStream_t st);
void gamma_ring_forward(const void *fw, int64_t fms, const std::vector<int> &ns, int ng, bool real, double c,
                        double2 *Gout, int64_t gms, int64_t gks, int nb, int bl, int ss, cudaStream_t st);

// FP32 storage conversions: `rows` rows of n values, row r at src + r ss and
// dst + r ds (elements; complex values as interleaved pairs).  Widening is
// exact; narrowing rounds to nearest.
void widen_rows(const float *src, int64_t ss, double *dst, int64_t ds, int64_t n, int rows, cudaStream_t st);
void narrow_rows(const double *src, int64_t ss, float *dst, int64_t ds, int64_t n, int rows, cudaStream_t st);

// Merge of per-(scale, direction) Wigner coefficients into flm (lmn2lm):
//   flm(l,m) = sum_pairs [ psi_p(l) z_p(l,m) + real&&n>0 : (-1)^{m+n} conj(z_p(l,-m)) psin_p(l) ]
//              + zs(l,m)
struct MergePair {
  int64_t off;  // element offset of z_p inside the z buffer (per batch item)
  int bl, n, lmin;
  int64_t woff;  // offset of psi_p / psin_p (length bl each) in the weight buffer
};
void merge_lmn(double2 *flm, int L, int64_t fs, const double2 *z, int64_t zs, const MergePair *pairs,
               int npairs, const double2 *wts, const double2 *zscal, int64_t zss, int bl_scal,
               bool real, bool accumulate, int nb, cudaStream_t st);

// flm(l,-m) = (-1)^m conj(flm(l,m)) for m > 0 (real-signal completion)
void symmetrize_flm(double2 *flm, int L, int64_t fs, int nb, cudaStream_t st);

// elementwise: y[i] = x[i] * s (complex or real, as doubles)
void scale_copy(const double *x, double *y, int64_t n, double s, cudaStream_t st);
// batched elementwise on doubles: y_b = a x_b + c y_b (rows of n at strides xs, ys)
void axpby(const double *x, int64_t xs, double *y, int64_t ys, int64_t n, int nb, double a, double c,
           cudaStream_t st);

}  // namespace s2g

namespace s2g {

// ---- harmonic tiling multiplies on the reference's Wigner (flmn) layout ----
// One scale of SO3 compact storage (n negative first; n >= 0 only when real).
struct LmnScale {
  int j;         // row of the wavelet array psi[(J+1) L^2]
  int bl, Nj;    // band-limit and direction band-limit of the scale
  int64_t loff;  // element offset of the scale inside f_wav_lmn
};
// mode 0: flmn = flm 8pi^2/(2l+1) conj(psi)  (s2let_analysis_lm2lmn)
// mode 1: flmn = flm conj(psi)                (s2let_synthesis_adjoint_lm2lmn)
// Scaling part: fscal_lm = flm sqrt(4pi/(2l+1)) phi(l), l < bl_scal.
void lmn_split(double2 *flmn, double2 *fscal, const double2 *flm, const double2 *psi, const double *phi,
               const LmnScale *scales, int nscale, int Nmax, int L, int bl_scal, int spin, bool real,
               int mode, cudaStream_t st);
// mode 0: flm = sum flmn psi            (s2let_synthesis_lmn2lm)
// mode 1: flm = sum flmn 8pi^2/(2l+1) psi (s2let_analysis_adjoint_lmn2lm)
void lmn_merge(double2 *flm, const double2 *flmn, const double2 *fscal, const double2 *psi,
               const double *phi, const LmnScale *scales, int nscale, int L, int bl_scal, int spin,
               bool real, int mode, cudaStream_t st);

// ---- axisymmetric harmonic multiplies (src/c/s2let_transform_axisym_lm.c:133-308) ----
// synth = 0: fwav[off_j + lm] = flm[lm] sqrt(4pi/(2l+1)) wav_lm[j L + l];  fscal likewise
// synth = 1: flm[lm] += sum_j fwav[off_j + lm] sqrt(4pi/(2l+1)) wav_lm[jL+l] + fscal term
void axisym_lm(double2 *flm, double2 *fwav, double2 *fscal, const double *wav_lm, const double *scal_lm,
               const int *bl, const int64_t *off, int J_min, int nscale, int L, int bl_scal, int synth,
               cudaStream_t st);

// g[i] = 0 where |(int) g[i]| < threshold[scale]   (reference hard threshold)
void hard_threshold(double *g, const double *thr, const int64_t *off, int nscale, int64_t total,
                    cudaStream_t st);

}  // namespace s2g
