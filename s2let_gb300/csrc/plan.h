// Cached device-side plans: Wigner tables per (band-limit, |n|) and Bluestein
// FFT data per ring length.  Built once, kept until s2let_gpu_release_plans().
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <vector>

namespace s2g {

// Wigner-d table of one band-limit bl and direction an = |n| >= 0 on the theta
// grid of one sampling scheme, for m in [mlo, bl-1] (mlo = 0 when an = 0, else
// -(bl-1)); per m the l-range is [l0(m), bl), l0 = max(|m|, an), nl = bl - l0.
//   MW   (ss = 0): nt = bl rings,     theta_t = pi (2t+1)/(2bl-1)
//   MWSS (ss = 1): nt = bl + 1 rings, theta_t = pi t / bl (both poles)
//   D (inverse)  block m: row-major [t][l - l0]      value d^l_{m,an}(theta_t)
//   Q (forward)  block m: row-major [l - l0][t']     value sum_t d^l_{m,an}(theta_t) W_eps[t][t']
// where W_eps (eps = (-1)^{m+an}) is the exact quadrature operator of the
// sampling: extension of a ring signal to the full theta circle with parity
// eps (kt = 2bl-1 or 2bl samples), Fourier transform, convolution with
// w(p) = int_0^pi e^{ipt} sin t dt, and folding back, divided by kt^2.
// Entries for n < 0 are read from the |n| table at -m with sign (-1)^{m+|n|}.
//
// A recomputed table (rc = true) stores neither D nor Q.  It keeps, per m,
// theta ring t and segment c of kSeg degrees starting at lc = l0 + c kSeg,
// the checkpoint pair (d^{lc}, d^{lc+1}) = (a, b) 2^E from the double-double
// recursion (ck / ck_e at [coff[mi] + c nt + t]); the contraction kernels
// regenerate the segment from it with the FP64 three-term recursion, written
// in u = 2 sin^2(theta/2) (north) or 2 cos^2(theta/2) (south) as uq[t] =
// (u, north).  The forward quadrature is applied as the nt x nt operators
// W_eps (W[0]: eps = +1, W[1]: eps = -1), shared by all tables of (bl, ss).
// Memory: 20 B per kSeg entries instead of 16 B per entry.
constexpr int kSeg = 64;
constexpr int kCkZeroExp = -100000;  // exponent of an all-zero checkpoint

struct WignerTable {
  int bl = 0, an = 0, ss = 0, nt = 0, mlo = 0, nm = 0;
  bool rc = false;
  std::vector<int64_t> off;  // host copy, nm+1 entries (elements)
  int64_t *d_off = nullptr;
  double *D = nullptr;
  double *Q = nullptr;
  // recomputed tables
  std::vector<int64_t> coff;  // host copy, nm+1 entries (checkpoints)
  int64_t *d_coff = nullptr;
  double2 *ck = nullptr;
  int *ck_e = nullptr;
  double2 *uq = nullptr;
  const double *W[2] = {nullptr, nullptr};
  int64_t elems() const { return off.empty() ? 0 : off.back(); }
  int l0(int m) const { return (m < 0 ? -m : m) > an ? (m < 0 ? -m : m) : an; }
  int nseg(int m) const { return (bl - l0(m) + kSeg - 1) / kSeg; }
};

// Ring geometry of a sampling scheme at band-limit bl: rings per map and
// samples per ring (= phi-DFT length).  The spectra of both keep m in
// [-(bl-1), bl-1]; the MWSS Nyquist bin m = bl is dropped / zero.
inline int grid_rings(int bl, int ss) { return ss ? bl + 1 : bl; }
inline int grid_ring_len(int bl, int ss) { return ss ? 2 * bl : 2 * bl - 1; }

// Bluestein data for ring length K (odd or even), padded FFT size P = 2^logP >= 2K-1.
struct RingFFT {
  int K = 0, P = 0, logP = 0;
  double2 *chirp = nullptr;  // K entries, exp(i pi k^2 / K)
  double2 *bhat = nullptr;   // P entries, FFT_P of the wrapped chirp
  double2 *tw = nullptr;     // P/2 entries, exp(-2 pi i k / P)
  // the same three arrays as double-float pairs (re.hi, re.lo, im.hi, im.lo)
  // for the FP32-pipe transform of the split-precision path
  float4 *chirp_df = nullptr, *bhat_df = nullptr, *tw_df = nullptr;
};

// rc: recomputed (checkpointed) table instead of stored D and Q
const WignerTable &wigner_table(int bl, int an, int ss = 0, bool rc = false);
// device bytes of the stored D and Q tables of (bl, an) on the sampling's grid
// (for the choice between stored and recomputed tables)
int64_t stored_table_bytes(int bl, int an, int ss);
const RingFFT &ring_fft(int K);
void release_plans();
size_t plan_bytes();

}  // namespace s2g
