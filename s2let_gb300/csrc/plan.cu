// Plan construction: Wigner-d tables (double-double three-term recursion on
// the GPU), the exact forward-quadrature operator W_eps of the MW or MWSS
// sampling, the forward tables Q = D^T W (FP64 GEMM on the GPU), and Bluestein
// FFT data.
#include <cmath>
#include <complex>
#include <map>
#include <mutex>
#include <tuple>

#include "common.h"
#include "plan.h"

namespace s2g {

namespace {

// ---------------------------------------------------------------------------
// double-double arithmetic (pairs hi + lo, |lo| <= ulp(hi)/2), used where the
// Wigner tables are built so that the stored doubles are correctly rounded
// ---------------------------------------------------------------------------
struct dd {
  double hi, lo;
};
__device__ __forceinline__ dd dd_quick(double a, double b) {
  const double s = a + b;
  return dd{s, b - (s - a)};
}
__device__ __forceinline__ dd dd_add(dd a, dd b) {
  const double s = a.hi + b.hi, bb = s - a.hi;
  const double e = (a.hi - (s - bb)) + (b.hi - bb) + a.lo + b.lo;
  return dd_quick(s, e);
}
__device__ __forceinline__ dd dd_neg(dd a) { return dd{-a.hi, -a.lo}; }
__device__ __forceinline__ dd dd_mul(dd a, dd b) {
  const double p = a.hi * b.hi;
  double e = fma(a.hi, b.hi, -p);
  e = fma(a.hi, b.lo, e);
  e = fma(a.lo, b.hi, e);
  return dd_quick(p, e);
}
__device__ __forceinline__ dd dd_mul_d(dd a, double b) {
  const double p = a.hi * b;
  double e = fma(a.hi, b, -p);
  e = fma(a.lo, b, e);
  return dd_quick(p, e);
}
__device__ __forceinline__ dd dd_div(dd a, dd b) {
  const double q1 = a.hi / b.hi;
  dd r = dd_add(a, dd_neg(dd_mul_d(b, q1)));
  const double q2 = r.hi / b.hi;
  r = dd_add(r, dd_neg(dd_mul_d(b, q2)));
  const double q3 = r.hi / b.hi;
  return dd_add(dd_quick(q1, q2), dd{q3, 0.0});
}
// sqrt of an exactly representable double, to double-double accuracy
__device__ __forceinline__ dd dd_sqrt_d(double x) {
  const double r = sqrt(x);
  if (r == 0.0) return dd{0.0, 0.0};
  return dd_quick(r, fma(-r, r, x) / (2.0 * r));
}
__device__ __forceinline__ void dd_renorm(dd &a, int &E) {
  int e;
  frexp(a.hi, &e);
  a.hi = ldexp(a.hi, -e);
  a.lo = ldexp(a.lo, -e);
  E += e;
}
// x^k as mantissa * 2^E (x > 0), square-and-multiply with renormalisation
__device__ dd dd_pow(dd x, int k, int &E) {
  dd r{1.0, 0.0};
  E = 0;
  int Eb = 0;
  dd_renorm(x, Eb);
  while (k) {
    if (k & 1) {
      r = dd_mul(r, x);
      E += Eb;
      dd_renorm(r, E);
    }
    k >>= 1;
    if (k) {
      x = dd_mul(x, x);
      Eb *= 2;
      dd_renorm(x, Eb);
    }
  }
  return r;
}

// ---------------------------------------------------------------------------
// d^l_{m,an}(theta_t), l = l0..bl-1, for one (m, t) per thread (t < nt), in double-double.
//
// Start value at l0 = max(|m|, an) (closed forms of d^{l0}):
//   l0 = m  >= an : (-1)^{l0-an} sqrt(C(2l0, l0+an)) c^{l0+an} s^{l0-an}
//   l0 = -m >= an : sqrt(C(2l0, l0-an)) c^{l0-an} s^{l0+an}
//   l0 = an > |m| : sqrt(C(2l0, l0+m)) c^{l0+m} s^{l0-m}
// c = cos(theta/2), s = sin(theta/2), both supplied by the host in double-double
// from the exact rational theta_t (pi (2t+1)/(2bl-1) for MW, pi t/bl for MWSS,
// where the poles give s = 0 or c = 0 exactly); sqrt(C) arrives as
// double-double mantissa * 2^e.  Three-term recursion in l:
//   d^{l+1} = [(2l+1)(l(l+1) x - m an) d^l - (l+1) sqrt((l^2-m^2)(l^2-an^2)) d^{l-1}]
//             / [l sqrt(((l+1)^2-m^2)((l+1)^2-an^2))],     x = cos(theta).
// x is never formed (its rounding is amplified by l^2 near the poles):
//   l(l+1) x - m an = (l(l+1) - m an) - l(l+1) u,   u = 2 s^2   (northern half)
//                   = l(l+1) v - (l(l+1) + m an),   v = 2 c^2   (southern half)
// with exact integer parts.  The mantissa carries a separate power-of-two
// exponent so that starts far below the double range stay exact.
// ---------------------------------------------------------------------------
struct AngleDD {
  double s_hi, s_lo, c_hi, c_lo, u_hi, u_lo;  // u = 2 s^2 (north) or 2 c^2 (south)
  int north, pad;                             // theta <= pi/2
};

// One row of the recursion, (m, an) at one angle: calls sink(i, v, vp, E) for
// i = l - l0 in [0, nl) with d^{l0+i} = v 2^E and d^{l0+i-1} = vp 2^E (vp = 0
// at i = 0), or sink.zero() when the closed form, hence the row, vanishes.
template <class Sink>
__device__ void wigner_row(int bl, int an, int m, const AngleDD &A, double st_hi, double st_lo, int st_e,
                           Sink &sink) {
  const int am = m < 0 ? -m : m;
  const int l0 = am > an ? am : an;
  const int nl = bl - l0;
  if (nl <= 0) return;
  const dd s{A.s_hi, A.s_lo}, c{A.c_hi, A.c_lo}, u{A.u_hi, A.u_lo};
  const bool north = A.north != 0;
  int ka, kb;
  double sign = 1.0;
  if (m >= 0 && m >= an) {
    ka = l0 + an; kb = l0 - an; sign = ((l0 - an) & 1) ? -1.0 : 1.0;
  } else if (m < 0 && am >= an) {
    ka = l0 - an; kb = l0 + an;
  } else {
    ka = l0 + m; kb = l0 - m;
  }
  if ((ka > 0 && c.hi == 0.0) || (kb > 0 && s.hi == 0.0)) {
    sink.zero();  // the closed form vanishes (a pole); so does the whole recursion
    return;
  }
  int E = st_e, e1 = 0, e2 = 0;
  dd v{st_hi, st_lo};
  if (ka) {
    v = dd_mul(v, dd_pow(c, ka, e1));
    E += e1;
  }
  if (kb) {
    v = dd_mul(v, dd_pow(s, kb, e2));
    E += e2;
  }
  v.hi *= sign;
  v.lo *= sign;
  dd vp{0.0, 0.0};
  sink(0, v.hi, 0.0, E);
  const double mn = (double)m * (double)an, m2 = (double)m * m, n2 = (double)an * an;
  int l = l0;
  if (l0 == 0 && nl > 1) { /* m = an = 0: d^1_{00} = cos(theta) */
    const dd x = north ? dd_add(dd{1.0, 0.0}, dd_neg(u)) : dd_add(u, dd{-1.0, 0.0});
    vp = v;
    v = dd_mul(x, v);
    sink(1, v.hi, vp.hi, E);
    l = 1;
  }
  for (; l + 1 < bl; ++l) {
    const double dl = (double)l;
    const double ll1 = dl * (dl + 1.0);
    const dd lu = dd_mul_d(u, ll1);
    const dd xterm = north ? dd_add(dd{ll1 - mn, 0.0}, dd_neg(lu)) : dd_add(lu, dd{-(ll1 + mn), 0.0});
    const dd a = dd_mul_d(xterm, 2.0 * dl + 1.0);
    const dd b = dd_mul_d(dd_sqrt_d((dl * dl - m2) * (dl * dl - n2)), dl + 1.0);
    const dd q = dd_mul_d(dd_sqrt_d(((dl + 1.0) * (dl + 1.0) - m2) * ((dl + 1.0) * (dl + 1.0) - n2)), dl);
    const dd vn = dd_div(dd_add(dd_mul(a, v), dd_neg(dd_mul(b, vp))), q);
    vp = v;
    v = vn;
    if (fabs(v.hi) > 0x1p500) {
      v.hi = ldexp(v.hi, -500);
      v.lo = ldexp(v.lo, -500);
      vp.hi = ldexp(vp.hi, -500);
      vp.lo = ldexp(vp.lo, -500);
      E += 500;
    }
    sink(l + 1 - l0, v.hi, vp.hi, E);
  }
}

// the full row D[t][l - l0] of a stored table
struct RowSink {
  double *row;
  int nl;
  __device__ void zero() {
    for (int i = 0; i < nl; ++i) row[i] = 0.0;
  }
  __device__ void operator()(int i, double v, double, int E) { row[i] = ldexp(v, E); }
};

__global__ void k_wigner_d(double *__restrict__ D, const int64_t *__restrict__ off, int bl, int nt, int an,
                           int mlo, int nm, const double *__restrict__ start_hi,
                           const double *__restrict__ start_lo, const int *__restrict__ start_exp,
                           const AngleDD *__restrict__ ang) {
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= (int64_t)nm * nt) return;
  const int mi = (int)(gid / nt), t = (int)(gid % nt);
  const int m = mlo + mi;
  const int am = m < 0 ? -m : m;
  const int nl = bl - (am > an ? am : an);
  if (nl <= 0) return;
  RowSink sink{D + off[mi] + (int64_t)t * nl, nl};
  wigner_row(bl, an, m, ang[t], start_hi[mi], start_lo[mi], start_exp[mi], sink);
}

// Checkpoints of a recomputed table: for segment c (l from l0 + c kSeg), the
// pair (d^{lc}, d^{lc+1}) = (a, b) 2^E with max(|a|, |b|) in [1/2, 1) (b = 0
// when the segment holds one value; E = kCkZeroExp when the pair is zero),
// stored at [off[mi] + c nt + t].
struct CkptSink {
  double2 *ab;
  int *ex;
  int64_t base;  // off[mi] + t
  int nt, nl;
  __device__ void put(int c, double a, double b, int E) {
    const double mx = fmax(fabs(a), fabs(b));
    if (mx == 0.0) {
      ab[base + (int64_t)c * nt] = make_double2(0.0, 0.0);
      ex[base + (int64_t)c * nt] = kCkZeroExp;
      return;
    }
    int k;
    frexp(mx, &k);
    ab[base + (int64_t)c * nt] = make_double2(ldexp(a, -k), ldexp(b, -k));
    ex[base + (int64_t)c * nt] = E + k;
  }
  __device__ void zero() {
    for (int c = 0; c * kSeg < nl; ++c) put(c, 0.0, 0.0, 0);
  }
  __device__ void operator()(int i, double v, double vp, int E) {
    const int r = i % kSeg;
    if (r == 1) put(i / kSeg, vp, v, E);
    else if (r == 0 && i == nl - 1) put(i / kSeg, v, 0.0, E);  // a segment of one value
  }
};

__global__ void k_wigner_ckpt(double2 *__restrict__ ab, int *__restrict__ ex, const int64_t *__restrict__ off,
                              int bl, int nt, int an, int mlo, int nm, const double *__restrict__ start_hi,
                              const double *__restrict__ start_lo, const int *__restrict__ start_exp,
                              const AngleDD *__restrict__ ang) {
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= (int64_t)nm * nt) return;
  const int mi = (int)(gid / nt), t = (int)(gid % nt);
  const int m = mlo + mi;
  const int am = m < 0 ? -m : m;
  const int nl = bl - (am > an ? am : an);
  if (nl <= 0) return;
  CkptSink sink{ab, ex, off[mi] + t, nt, nl};
  wigner_row(bl, an, m, ang[t], start_hi[mi], start_lo[mi], start_exp[mi], sink);
}

// w(p) = int_0^pi e^{ipt} sin t dt  (complex: +-i pi/2 at p = +-1)
__device__ inline double2 wsin(int p) {
  if (p == 1) return make_double2(0.0, 0.5 * kPi);
  if (p == -1) return make_double2(0.0, -0.5 * kPi);
  if (p & 1) return make_double2(0.0, 0.0);
  return make_double2(2.0 / (1.0 - (double)p * (double)p), 0.0);
}

// A[m'][t] = e^{-i m' theta_t} + [ring t has a distinct mirror] eps e^{i m' theta_t}
// (m' in [-(bl-1), bl-1]): the Fourier basis on the full theta circle folded
// onto the rings.  Mirrors: MW rings t < bl-1 (theta = pi is its own);
// MWSS rings 1 <= t <= bl-1 (the poles are their own).
__device__ inline double2 fold_basis(int mp, int t, int bl, int ss, int eps) {
  double sn, cs;
  bool mirrored;
  if (!ss) {
    const int K = 2 * bl - 1;
    // angle m' pi (2t+1)/K reduced modulo 2K for accuracy
    const long q = ((long)mp * (2 * t + 1)) % (2L * K);
    sincospi((double)q / (double)K, &sn, &cs);
    mirrored = t < bl - 1;
  } else {
    // angle m' pi t / bl reduced modulo 2 bl
    const long q = ((long)mp * t) % (2L * bl);
    sincospi((double)q / (double)bl, &sn, &cs);
    mirrored = t >= 1 && t <= bl - 1;
  }
  double2 r = make_double2(cs, -sn);
  if (mirrored) {
    r.x += eps * cs;
    r.y += eps * sn;
  }
  return r;
}

// TA[m''][t'] = sum_{m'} w(m' + m'') A[m'][t']   (t' < nt)
__global__ void k_wmat_ta(double2 *__restrict__ TA, int bl, int nt, int ss, int eps) {
  const int K = 2 * bl - 1;
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= (int64_t)K * nt) return;
  const int mpp = (int)(gid / nt) - (bl - 1), tp = (int)(gid % nt);
  double2 acc = make_double2(0.0, 0.0);
  for (int mp = -(bl - 1); mp <= bl - 1; ++mp) {
    const int p = mp + mpp;
    if ((p & 1) && p != 1 && p != -1) continue;
    const double2 w = wsin(p), a = fold_basis(mp, tp, bl, ss, eps);
    acc.x += w.x * a.x - w.y * a.y;
    acc.y += w.x * a.y + w.y * a.x;
  }
  TA[gid] = acc;
}

// W[t][t'] = Re sum_{m''} A[m''][t] TA[m''][t'] / kt^2,  kt = samples on the full circle
__global__ void k_wmat_w(double *__restrict__ W, const double2 *__restrict__ TA, int bl, int nt, int ss,
                         int eps) {
  const int kt = ss ? 2 * bl : 2 * bl - 1;
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= (int64_t)nt * nt) return;
  const int t = (int)(gid / nt), tp = (int)(gid % nt);
  double acc = 0.0;
  for (int mpp = -(bl - 1); mpp <= bl - 1; ++mpp) {
    const double2 a = fold_basis(mpp, t, bl, ss, eps);
    const double2 b = TA[(int64_t)(mpp + bl - 1) * nt + tp];
    acc += a.x * b.x - a.y * b.y;
  }
  W[gid] = acc / ((double)kt * (double)kt);
}

// Q_m[l][t'] = sum_t D_m[t][l] W_eps(m)[t][t'], tiled FP64 GEMM per m (grid.z = m).
constexpr int QG_T = 64, QG_K = 16;
__global__ void __launch_bounds__(256) k_qgemm(double *__restrict__ Q, const double *__restrict__ D,
                                               const int64_t *__restrict__ off,
                                               const double *__restrict__ Wp,
                                               const double *__restrict__ Wm, int bl, int nt,
                                               int an, int mlo) {
  const int mi = blockIdx.z, m = mlo + mi;
  const int am = m < 0 ? -m : m;
  const int l0 = am > an ? am : an, nl = bl - l0;
  const int row0 = blockIdx.y * QG_T, col0 = blockIdx.x * QG_T;  // rows: l-l0, cols: t'
  if (row0 >= nl) return;
  const double *W = (((m + an) & 1) == 0) ? Wp : Wm;
  const double *Dm = D + off[mi];
  double *Qm = Q + off[mi];
  __shared__ double sA[QG_K][QG_T + 1];  // [t][l]
  __shared__ double sB[QG_K][QG_T + 1];  // [t][t']
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc[4][4] = {};
  for (int k0 = 0; k0 < nt; k0 += QG_K) {
    for (int i = threadIdx.x; i < QG_K * QG_T; i += 256) {
      const int kk = i / QG_T, c = i % QG_T;
      const int t = k0 + kk;
      sA[kk][c] = (t < nt && row0 + c < nl) ? Dm[(int64_t)t * nl + row0 + c] : 0.0;
      sB[kk][c] = (t < nt && col0 + c < nt) ? W[(int64_t)t * nt + col0 + c] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < QG_K; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = sA[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = sB[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = row0 + ty * 4 + i;
    if (r >= nl) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = col0 + tx * 4 + j;
      if (c < nt) Qm[(int64_t)r * nt + c] = acc[i][j];
    }
  }
}

// host FFT (radix-2) for the Bluestein kernel spectrum
void host_fft(std::vector<std::complex<double>> &x) {
  const size_t n = x.size();
  for (size_t i = 1, j = 0; i < n; ++i) {
    size_t bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) std::swap(x[i], x[j]);
  }
  for (size_t len = 2; len <= n; len <<= 1) {
    for (size_t i = 0; i < n; i += len)
      for (size_t k = 0; k < len / 2; ++k) {
        const double a = -2.0 * kPi * (double)k / (double)len;
        std::complex<double> w(cos(a), sin(a));
        auto u = x[i + k], v = x[i + k + len / 2] * w;
        x[i + k] = u + v;
        x[i + k + len / 2] = u - v;
      }
  }
}

std::mutex g_plan_mu;
std::map<std::tuple<int, int, int, int>, std::unique_ptr<WignerTable>> g_tables;  // (bl, an, ss, rc)
std::map<int, std::unique_ptr<RingFFT>> g_rings;
size_t g_bytes = 0;

template <class T>
T *dev_alloc(size_t n) {
  T *p = nullptr;
  S2G_CUDA(cudaMalloc(&p, sizeof(T) * (n ? n : 1)));
  g_bytes += sizeof(T) * (n ? n : 1);
  return p;
}

// the quadrature operators W_+ and W_- of (bl, ss), nt x nt each, cached
// (caller holds g_plan_mu)
std::map<std::pair<int, int>, std::pair<double *, double *>> g_wmat;
std::pair<double *, double *> wmat_locked(int bl, int ss) {
  auto key = std::make_pair(bl, ss);
  auto it = g_wmat.find(key);
  if (it != g_wmat.end()) return it->second;
  const int nt = grid_rings(bl, ss), K = 2 * bl - 1;
  double2 *TA = nullptr;
  S2G_CUDA(cudaMalloc(&TA, sizeof(double2) * (size_t)K * nt));
  double *W[2];
  for (int e = 0; e < 2; ++e) {
    W[e] = dev_alloc<double>((size_t)nt * nt);
    const int eps = e == 0 ? 1 : -1;
    k_wmat_ta<<<ceil_div((int64_t)K * nt, 128), 128>>>(TA, bl, nt, ss, eps);
    S2G_LAUNCHED();
    k_wmat_w<<<ceil_div((int64_t)nt * nt, 128), 128>>>(W[e], TA, bl, nt, ss, eps);
    S2G_LAUNCHED();
  }
  S2G_CUDA(cudaDeviceSynchronize());
  cudaFree(TA);
  auto w = std::make_pair(W[0], W[1]);
  g_wmat.emplace(key, w);
  return w;
}

std::unique_ptr<WignerTable> build_table(int bl, int an, int ss, bool rc) {
  auto tb = std::make_unique<WignerTable>();
  tb->bl = bl;
  tb->an = an;
  tb->ss = ss;
  tb->rc = rc;
  tb->nt = grid_rings(bl, ss);
  const int nt = tb->nt;
  tb->mlo = an == 0 ? 0 : -(bl - 1);
  tb->nm = bl - tb->mlo;
  tb->off.assign(tb->nm + 1, 0);
  std::vector<double> st_hi(tb->nm), st_lo(tb->nm);
  std::vector<int> ex(tb->nm);
  const long double ln2 = 0.693147180559945309417232121458176568L;
  for (int mi = 0; mi < tb->nm; ++mi) {
    const int m = tb->mlo + mi;
    const int l0 = tb->l0(m);
    const int64_t nl = std::max(0, bl - l0);
    tb->off[mi + 1] = tb->off[mi] + nl * nt;
    // sqrt(C(2 l0, ka)) in extended precision, split into (hi + lo) * 2^e
    int ka;
    const int am = std::abs(m);
    if (m >= 0 && m >= an) ka = l0 + an;
    else if (m < 0 && am >= an) ka = l0 - an;
    else ka = l0 + m;
    long double lc = 0.0L;
    const int kk = std::min(ka, 2 * l0 - ka);
    for (int i = 1; i <= kk; ++i) lc += logl((long double)(2 * l0 - kk + i)) - logl((long double)i);
    lc *= 0.5L;
    const int e = (int)floorl(lc / ln2);
    const long double mant = expl(lc - e * ln2);
    st_hi[mi] = (double)mant;
    st_lo[mi] = (double)(mant - (long double)st_hi[mi]);
    ex[mi] = e;
  }
  // half-angles of the rings in extended precision:
  //   MW:   theta_t / 2 = pi (2t+1) / (2(2bl-1)),   MWSS: theta_t / 2 = pi t / (2 bl)
  // written as pi a / b with integers a / b <= 1/2 (north) or >= 1/2 (south)
  std::vector<AngleDD> ang(nt);
  {
    const long double pi_l = 3.141592653589793238462643383279502884197L;
    auto split = [](long double x, double &hi, double &lo) {
      hi = (double)x;
      lo = (double)(x - (long double)hi);
    };
    for (int t = 0; t < nt; ++t) {
      const long a = ss ? t : 2 * t + 1;            // theta_t / pi = a / b
      const long b = ss ? bl : 2 * bl - 1;
      long double sl, cl;
      if (a == 0) {
        sl = 0.0L;  // theta = 0 exactly
        cl = 1.0L;
      } else if (a == b) {
        sl = 1.0L;  // theta = pi exactly
        cl = 0.0L;
      } else {
        const long double h = pi_l * (long double)a / (long double)(2 * b);
        sl = sinl(h);
        cl = cosl(h);
      }
      const bool north = 2 * a <= b;
      const long double u = north ? 2.0L * sl * sl : 2.0L * cl * cl;
      split(sl, ang[t].s_hi, ang[t].s_lo);
      split(cl, ang[t].c_hi, ang[t].c_lo);
      split(u, ang[t].u_hi, ang[t].u_lo);
      ang[t].north = north ? 1 : 0;
      ang[t].pad = 0;
    }
  }
  const auto W = wmat_locked(bl, ss);
  tb->W[0] = W.first;
  tb->W[1] = W.second;
  double *d_hi = nullptr, *d_lo = nullptr;
  int *d_ex = nullptr;
  AngleDD *d_ang = nullptr;
  S2G_CUDA(cudaMalloc(&d_hi, sizeof(double) * tb->nm));
  S2G_CUDA(cudaMalloc(&d_lo, sizeof(double) * tb->nm));
  S2G_CUDA(cudaMalloc(&d_ex, sizeof(int) * tb->nm));
  S2G_CUDA(cudaMalloc(&d_ang, sizeof(AngleDD) * nt));
  S2G_CUDA(cudaMemcpy(d_hi, st_hi.data(), sizeof(double) * tb->nm, cudaMemcpyHostToDevice));
  S2G_CUDA(cudaMemcpy(d_lo, st_lo.data(), sizeof(double) * tb->nm, cudaMemcpyHostToDevice));
  S2G_CUDA(cudaMemcpy(d_ex, ex.data(), sizeof(int) * tb->nm, cudaMemcpyHostToDevice));
  S2G_CUDA(cudaMemcpy(d_ang, ang.data(), sizeof(AngleDD) * nt, cudaMemcpyHostToDevice));
  const int64_t nthr = (int64_t)tb->nm * nt;
  if (!rc) {
    const int64_t n = tb->elems();
    tb->D = dev_alloc<double>(n);
    tb->Q = dev_alloc<double>(n);
    tb->d_off = dev_alloc<int64_t>(tb->nm + 1);
    S2G_CUDA(cudaMemcpy(tb->d_off, tb->off.data(), sizeof(int64_t) * (tb->nm + 1), cudaMemcpyHostToDevice));
    k_wigner_d<<<ceil_div(nthr, 128), 128>>>(tb->D, tb->d_off, bl, nt, an, tb->mlo, tb->nm, d_hi, d_lo, d_ex,
                                             d_ang);
    S2G_LAUNCHED();
    // Q = D^T W per m
    dim3 grid(ceil_div(nt, QG_T), ceil_div(bl, QG_T), tb->nm);
    k_qgemm<<<grid, 256>>>(tb->Q, tb->D, tb->d_off, W.first, W.second, bl, nt, an, tb->mlo);
    S2G_LAUNCHED();
  } else {
    tb->coff.assign(tb->nm + 1, 0);
    for (int mi = 0; mi < tb->nm; ++mi) tb->coff[mi + 1] = tb->coff[mi] + (int64_t)tb->nseg(tb->mlo + mi) * nt;
    const int64_t nc = tb->coff.back();
    tb->ck = dev_alloc<double2>(nc);
    tb->ck_e = dev_alloc<int>(nc);
    tb->d_coff = dev_alloc<int64_t>(tb->nm + 1);
    S2G_CUDA(cudaMemcpy(tb->d_coff, tb->coff.data(), sizeof(int64_t) * (tb->nm + 1), cudaMemcpyHostToDevice));
    std::vector<double2> uq(nt);
    for (int t = 0; t < nt; ++t) uq[t] = make_double2(ang[t].u_hi, ang[t].north ? 1.0 : 0.0);
    tb->uq = dev_alloc<double2>(nt);
    S2G_CUDA(cudaMemcpy(tb->uq, uq.data(), sizeof(double2) * nt, cudaMemcpyHostToDevice));
    k_wigner_ckpt<<<ceil_div(nthr, 128), 128>>>(tb->ck, tb->ck_e, tb->d_coff, bl, nt, an, tb->mlo, tb->nm, d_hi,
                                                d_lo, d_ex, d_ang);
    S2G_LAUNCHED();
  }
  S2G_CUDA(cudaDeviceSynchronize());
  cudaFree(d_hi);
  cudaFree(d_lo);
  cudaFree(d_ex);
  cudaFree(d_ang);
  return tb;
}

std::unique_ptr<RingFFT> build_ring(int K) {
  auto r = std::make_unique<RingFFT>();
  r->K = K;
  int P = 1, logP = 0;
  while (P < 2 * K - 1) {
    P <<= 1;
    ++logP;
  }
  r->P = P;
  r->logP = logP;
  std::vector<std::complex<double>> chirp(K), b(P, 0.0), tw(std::max(1, P / 2));
  for (long k = 0; k < K; ++k) {
    long q = (k * k) % (2L * K);
    const double a = kPi * (double)q / (double)K;
    chirp[k] = {cos(a), sin(a)};
  }
  b[0] = chirp[0];
  for (int k = 1; k < K; ++k) b[k] = b[P - k] = chirp[k];
  host_fft(b);
  for (int k = 0; k < P / 2; ++k) {
    const double a = -2.0 * kPi * (double)k / (double)P;
    tw[k] = {cos(a), sin(a)};
  }
  r->chirp = dev_alloc<double2>(K);
  r->bhat = dev_alloc<double2>(P);
  r->tw = dev_alloc<double2>(std::max(1, P / 2));
  S2G_CUDA(cudaMemcpy(r->chirp, chirp.data(), sizeof(double2) * K, cudaMemcpyHostToDevice));
  S2G_CUDA(cudaMemcpy(r->bhat, b.data(), sizeof(double2) * P, cudaMemcpyHostToDevice));
  S2G_CUDA(cudaMemcpy(r->tw, tw.data(), sizeof(double2) * std::max(1, P / 2), cudaMemcpyHostToDevice));
  auto to_df = [](const std::vector<std::complex<double>> &v) {
    std::vector<float4> o(v.size());
    for (size_t i = 0; i < v.size(); ++i) {
      const float rh = (float)v[i].real(), ih = (float)v[i].imag();
      o[i] = make_float4(rh, (float)(v[i].real() - (double)rh), ih, (float)(v[i].imag() - (double)ih));
    }
    return o;
  };
  const auto cdf = to_df(chirp), bdf = to_df(b), tdf = to_df(tw);
  r->chirp_df = dev_alloc<float4>(K);
  r->bhat_df = dev_alloc<float4>(P);
  r->tw_df = dev_alloc<float4>(std::max(1, P / 2));
  S2G_CUDA(cudaMemcpy(r->chirp_df, cdf.data(), sizeof(float4) * K, cudaMemcpyHostToDevice));
  S2G_CUDA(cudaMemcpy(r->bhat_df, bdf.data(), sizeof(float4) * P, cudaMemcpyHostToDevice));
  S2G_CUDA(cudaMemcpy(r->tw_df, tdf.data(), sizeof(float4) * std::max(1, P / 2), cudaMemcpyHostToDevice));
  return r;
}

}  // namespace

const WignerTable &wigner_table(int bl, int an, int ss, bool rc) {
  std::lock_guard<std::mutex> lk(g_plan_mu);
  auto key = std::make_tuple(bl, an, ss, rc ? 1 : 0);
  auto it = g_tables.find(key);
  if (it != g_tables.end()) return *it->second;
  auto tb = build_table(bl, an, ss, rc);
  const WignerTable &ref = *tb;
  g_tables.emplace(key, std::move(tb));
  return ref;
}

const RingFFT &ring_fft(int K) {
  std::lock_guard<std::mutex> lk(g_plan_mu);
  auto it = g_rings.find(K);
  if (it != g_rings.end()) return *it->second;
  auto r = build_ring(K);
  const RingFFT &ref = *r;
  g_rings.emplace(K, std::move(r));
  return ref;
}

void release_plans() {
  std::lock_guard<std::mutex> lk(g_plan_mu);
  cudaDeviceSynchronize();
  for (auto &kv : g_tables) {
    cudaFree(kv.second->D);
    cudaFree(kv.second->Q);
    cudaFree(kv.second->d_off);
    cudaFree(kv.second->ck);
    cudaFree(kv.second->ck_e);
    cudaFree(kv.second->d_coff);
    cudaFree(kv.second->uq);
  }
  for (auto &kv : g_wmat) {
    cudaFree(kv.second.first);
    cudaFree(kv.second.second);
  }
  g_wmat.clear();
  for (auto &kv : g_rings) {
    cudaFree(kv.second->chirp);
    cudaFree(kv.second->bhat);
    cudaFree(kv.second->tw);
    cudaFree(kv.second->chirp_df);
    cudaFree(kv.second->bhat_df);
    cudaFree(kv.second->tw_df);
  }
  g_tables.clear();
  g_rings.clear();
  g_bytes = 0;
}

int64_t stored_table_bytes(int bl, int an, int ss) {
  // sum over m of (bl - l0(m)) nt entries, D and Q, 8 B each
  const int nt = grid_rings(bl, ss), mlo = an == 0 ? 0 : -(bl - 1);
  int64_t e = 0;
  for (int m = mlo; m < bl; ++m) {
    const int am = m < 0 ? -m : m, l0 = am > an ? am : an;
    if (l0 < bl) e += (int64_t)(bl - l0) * nt;
  }
  return 16 * e;
}

size_t plan_bytes() {
  std::lock_guard<std::mutex> lk(g_plan_mu);
  return g_bytes;
}

}  // namespace s2g
