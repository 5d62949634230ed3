// Contractions against recomputed (checkpointed) Wigner tables, FP64.
//
// A recomputed table keeps, per m, theta ring t and segment of kSeg degrees,
// the pair (d^{lc}, d^{lc+1}) = (a, b) 2^E from the double-double recursion
// (plan.cu).  The kernels here regenerate each segment in FP64 with the
// three-term recursion in l, written with u = 2 sin^2(theta/2) (north) or
// u = 2 cos^2(theta/2) (south) so that the large integer parts cancel exactly:
//   d^{l+1} = (q_l + p_l u) d^l - c2_l d^{l-1}
//   north: p_l = -r l(l+1), q_l = r (l(l+1) - m n);  south: p_l = r l(l+1), q_l = -r (l(l+1) + m n)
//   r = (2l+1) / (l S_{l+1}),  c2_l = (l+1) S_l / (l S_{l+1}),  S_l = sqrt((l^2-m^2)(l^2-n^2))
// Three FP64 instructions per value; restarting every kSeg degrees from the
// double-double checkpoints keeps the recursion's rounding growth to a few
// ulps (a plain FP64 run over l < 2048 drifts by ~3e-12 near the poles).
// Values are carried scaled by 2^-E, one scale per ring and segment, applied
// once per segment: to the partial sums (l -> t) or to the inputs (t -> l).
//
//   k_rc_l2t   out[b][t][m] = sign sum_l d^l(theta_t) w(l) x_b(l, m)       one thread per ring t
//   k_rc_t2l   y_b(l, m)   = sign w(l) sum_t d^l(theta_t) in_b(t, m)       a 128 x 64 d tile in shared memory
//   k_apply_w  the forward quadrature W_eps(m) (or its transpose) on ring spectra: the
//              stored path's Q = D^T W becomes D^T applied after W (FP64 tiled GEMM)
#include <algorithm>

#include "autotune.h"
#include "common.h"
#include "dfarith.h"
#include "kernels.h"
#include "mixed.h"
#include "recompute.h"
#include "timing.h"

namespace s2g {

namespace {

constexpr int kRcT = 128;  // threads per CTA: rings per tile
static_assert(kRcT == 2 * kSeg, "t -> l maps two threads per degree of a segment");

struct RcArgs {
  int bl, nt, an, tmlo, n;
  const int64_t *coff;
  const double2 *ck;
  const int *ck_e;
  const double2 *uq;
  int mlo, lmin;
  const double2 *w;
  double wscale;
  int wconj;
  const double2 *src;  // l -> t: x (l^2 + l + m);  t -> l: spectra [t][m - s_mlo]
  int64_t ss;
  int sw, s_mlo, x_half;
  double2 *dst;  // l -> t: spectra [t][m - d_mlo];  t -> l: y (l^2 + l + m)
  int64_t ds;
  int dw, d_mlo;
  int nb;
};

__device__ __forceinline__ double2 cmul_(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 weight_of(const RcArgs &a, int l) {
  double2 w = a.w ? a.w[l] : make_double2(1.0, 0.0);
  if (a.wconj) w.y = -w.y;
  return make_double2(w.x * a.wscale, w.y * a.wscale);
}

// table row (mirror for n < 0, or n = 0 and m < 0 on a table holding m >= 0)
struct RcRef {
  int mi, mt;
  double sign;
};
__device__ __forceinline__ RcRef rc_ref(const RcArgs &a, int m) {
  RcRef r;
  if (a.n > 0 || (a.n == 0 && m >= 0)) {
    r.mi = m - a.tmlo;
    r.sign = 1.0;
  } else {
    r.mi = -m - a.tmlo;
    r.sign = ((m + a.an) & 1) ? -1.0 : 1.0;
  }
  r.mt = a.tmlo + r.mi;
  return r;
}

// recursion coefficients of degree l for (m, an): cn = (p, q) north, cs = (p, q) south
__device__ __forceinline__ void rec_coef(int l, int m, int an, double2 &cn, double2 &cs, double &c2) {
  const double dl = l, ll1 = dl * (dl + 1.0), mn = (double)m * an, m2 = (double)m * m, n2 = (double)an * an;
  const double s1 = sqrt(((dl + 1.0) * (dl + 1.0) - m2) * ((dl + 1.0) * (dl + 1.0) - n2));
  const double s0 = sqrt((dl * dl - m2) * (dl * dl - n2));
  const double r = (2.0 * dl + 1.0) / (dl * s1);
  cn = make_double2(-r * ll1, r * (ll1 - mn));
  cs = make_double2(r * ll1, -r * (ll1 + mn));
  c2 = (dl + 1.0) * s0 / (dl * s1);
}

__device__ __forceinline__ int exp_bits(double v) { return (int)((__double_as_longlong(v) >> 52) & 0x7FF); }
constexpr int kRenorm = 600;  // rescale step when a carried value passes 2^kRenorm

// 2^E as a double (0 below the subnormal range)
__device__ __forceinline__ double pow2(int E) { return E < -1074 ? 0.0 : ldexp(1.0, E); }

// ---------------------------------------------------------------------------
// l -> t
// ---------------------------------------------------------------------------

template <int NBT>
__global__ void __launch_bounds__(kRcT) k_rc_l2t(RcArgs a) {
  __shared__ double2 scn[kSeg], scs[kSeg];
  __shared__ double sc2[kSeg];
  __shared__ double2 sx[kSeg][NBT];
  const int m = a.mlo + blockIdx.x;
  const int am = m < 0 ? -m : m;
  const RcRef r = rc_ref(a, m);
  const int amt = r.mt < 0 ? -r.mt : r.mt;
  const int l0 = amt > a.an ? amt : a.an, bl = a.bl, nl = bl - l0;
  const int lst = l0 > a.lmin ? l0 : a.lmin;
  const int t = blockIdx.y * kRcT + threadIdx.x;
  const bool live = t < a.nt;
  const int b0 = blockIdx.z * NBT;
  double2 acc[NBT];
#pragma unroll
  for (int b = 0; b < NBT; ++b) acc[b] = make_double2(0.0, 0.0);
  double u = 0.0;
  bool north = true;
  if (live) {
    const double2 q = a.uq[t];
    u = q.x;
    north = q.y != 0.0;
  }
  if (nl > 0 && lst < bl) {
    const int nseg = (nl + kSeg - 1) / kSeg, c0 = (lst - l0) / kSeg;
    const double2 *ck = a.ck + a.coff[r.mi];
    const int *cke = a.ck_e + a.coff[r.mi];
    const double2 *cc = north ? scn : scs;
    for (int c = c0; c < nseg; ++c) {
      const int lc = l0 + c * kSeg, n = min(kSeg, bl - lc);
      __syncthreads();
      for (int i = threadIdx.x; i < n; i += kRcT)
        if (i >= 1) rec_coef(lc + i, r.mt, a.an, scn[i], scs[i], sc2[i]);
      for (int i = threadIdx.x; i < kSeg * NBT; i += kRcT) {
        const int kk = i / NBT, b = i % NBT, l = lc + kk;
        double2 v = make_double2(0.0, 0.0);
        if (kk < n && l >= lst && b0 + b < a.nb) {
          const int64_t base = (int64_t)(b0 + b) * a.ss + (int64_t)l * l + l;
          if (a.x_half && m < 0) {
            v = a.src[base - m];
            v.y = -v.y;
            if (am & 1) v = make_double2(-v.x, -v.y);
          } else {
            v = a.src[base + m];
          }
          v = cmul_(v, weight_of(a, l));
        }
        sx[kk][b] = v;
      }
      __syncthreads();
      if (!live) continue;
      int E = cke[(int64_t)c * a.nt + t];
      if (E < -1074 - 2 * kRenorm) continue;  // the whole segment is below the double range
      const double2 ab = ck[(int64_t)c * a.nt + t];
      double vp = ab.x, v = ab.y;
      double2 s[NBT];
#pragma unroll
      for (int b = 0; b < NBT; ++b) {
        s[b].x = vp * sx[0][b].x;
        s[b].y = vp * sx[0][b].y;
        if (n > 1) {
          s[b].x = fma(v, sx[1][b].x, s[b].x);
          s[b].y = fma(v, sx[1][b].y, s[b].y);
        }
      }
      for (int i = 1; i + 1 < n; ++i) {
        const double2 k = cc[i];
        const double xt = fma(k.x, u, k.y);
        const double vn = fma(xt, v, -sc2[i] * vp);
        vp = v;
        v = vn;
        if (exp_bits(v) > 1023 + kRenorm) {  // flush at the old scale, continue at the new one
          const double sc = pow2(E);
#pragma unroll
          for (int b = 0; b < NBT; ++b) {
            acc[b].x = fma(s[b].x, sc, acc[b].x);
            acc[b].y = fma(s[b].y, sc, acc[b].y);
            s[b] = make_double2(0.0, 0.0);
          }
          v = ldexp(v, -kRenorm);
          vp = ldexp(vp, -kRenorm);
          E += kRenorm;
        }
#pragma unroll
        for (int b = 0; b < NBT; ++b) {
          s[b].x = fma(v, sx[i + 1][b].x, s[b].x);
          s[b].y = fma(v, sx[i + 1][b].y, s[b].y);
        }
      }
      const double sc = pow2(E);
#pragma unroll
      for (int b = 0; b < NBT; ++b) {
        acc[b].x = fma(s[b].x, sc, acc[b].x);
        acc[b].y = fma(s[b].y, sc, acc[b].y);
      }
    }
  }
  if (!live) return;
#pragma unroll
  for (int b = 0; b < NBT; ++b) {
    if (b0 + b >= a.nb) break;
    a.dst[(int64_t)(b0 + b) * a.ds + (int64_t)t * a.dw + (m - a.d_mlo)] =
        make_double2(acc[b].x * r.sign, acc[b].y * r.sign);
  }
}

// ---------------------------------------------------------------------------
// t -> l
// ---------------------------------------------------------------------------

constexpr int kTileLd = kSeg + 1;  // padded row of the d tile

template <int NBT>
size_t rc_t2l_smem() {
  return sizeof(double) * kRcT * kTileLd + sizeof(double2) * kRcT * NBT;
}

// grid: x = m, y = segment, z = batch chunk.  Threads generate one ring's row of
// the tile each, then contract as (degree li = tid % kSeg, half bh = tid / kSeg):
// with NBT >= 2 each half takes half of the maps over all rings of the tile;
// with NBT = 1 each half takes half of the rings, and the halves add up at the end.
template <int NBT>
__global__ void __launch_bounds__(kRcT) k_rc_t2l(RcArgs a) {
  static_assert(NBT == 1 || NBT % 2 == 0, "one map, or two map halves");
  constexpr int NH = NBT == 1 ? 1 : NBT / 2;
  constexpr bool SPLIT_T = NBT == 1;
  extern __shared__ double smem_rc[];
  double *tile = smem_rc;                                   // [kRcT][kTileLd]
  double2 *sg = (double2 *)(smem_rc + kRcT * kTileLd);      // [kRcT][NBT]
  __shared__ double2 scn[kSeg], scs[kSeg];
  __shared__ double sc2[kSeg];
  const int m = a.mlo + blockIdx.x, c = blockIdx.y;
  const RcRef r = rc_ref(a, m);
  const int amt = r.mt < 0 ? -r.mt : r.mt;
  const int l0 = amt > a.an ? amt : a.an, bl = a.bl, nl = bl - l0;
  const int lst = l0 > a.lmin ? l0 : a.lmin;
  const int nseg = nl > 0 ? (nl + kSeg - 1) / kSeg : 0;
  if (c >= nseg) return;
  const int lc = l0 + c * kSeg, n = min(kSeg, bl - lc);
  if (lc + n <= lst) return;  // every degree of the segment is below lmin: no output
  const int b0 = blockIdx.z * NBT;
  const int tid = threadIdx.x;
  for (int i = tid; i < n; i += kRcT)
    if (i >= 1) rec_coef(lc + i, r.mt, a.an, scn[i], scs[i], sc2[i]);
  const double2 *ck = a.ck + a.coff[r.mi] + (int64_t)c * a.nt;
  const int *cke = a.ck_e + a.coff[r.mi] + (int64_t)c * a.nt;
  const int li = tid % kSeg, bh = tid / kSeg;
  double2 acc[NH];
#pragma unroll
  for (int j = 0; j < NH; ++j) acc[j] = make_double2(0.0, 0.0);
  __syncthreads();
  for (int t0 = 0; t0 < a.nt; t0 += kRcT) {
    const int t = t0 + tid;
    double *row = tile + tid * kTileLd;
    double scale = 0.0;
    int E = kCkZeroExp;
    if (t < a.nt) E = cke[t];
    if (E >= -1074 - 2 * kRenorm) {
      const double2 q = a.uq[t];
      const double u = q.x;
      const double2 *cc = q.y != 0.0 ? scn : scs;
      const double2 ab = ck[t];
      double vp = ab.x, v = ab.y;
      row[0] = vp;
      if (n > 1) row[1] = v;
      for (int i = 1; i + 1 < n; ++i) {
        const double2 k = cc[i];
        const double xt = fma(k.x, u, k.y);
        const double vn = fma(xt, v, -sc2[i] * vp);
        vp = v;
        v = vn;
        if (exp_bits(v) > 1023 + kRenorm) {  // keep one scale per row: rescale what is written
          for (int j = 0; j <= i; ++j) row[j] = ldexp(row[j], -kRenorm);
          v = ldexp(v, -kRenorm);
          vp = ldexp(vp, -kRenorm);
          E += kRenorm;
        }
        row[i + 1] = v;
      }
      for (int i = n; i < kSeg; ++i) row[i] = 0.0;
      scale = pow2(E);
    } else {
      for (int i = 0; i < kSeg; ++i) row[i] = 0.0;
    }
#pragma unroll
    for (int b = 0; b < NBT; ++b) {
      double2 g = make_double2(0.0, 0.0);
      if (t < a.nt && b0 + b < a.nb && scale != 0.0) {
        g = a.src[(int64_t)(b0 + b) * a.ss + (int64_t)t * a.sw + (m - a.s_mlo)];
        g = make_double2(g.x * scale, g.y * scale);
      }
      sg[tid * NBT + b] = g;
    }
    __syncthreads();
    const int tl_end = min(kRcT, a.nt - t0);
    const int tl_lo = SPLIT_T ? bh * (kRcT / 2) : 0;
    const int tl_hi = SPLIT_T ? min(tl_end, tl_lo + kRcT / 2) : tl_end;
#pragma unroll 4
    for (int tl = tl_lo; tl < tl_hi; ++tl) {
      const double d = tile[tl * kTileLd + li];
#pragma unroll
      for (int j = 0; j < NH; ++j) {
        const double2 g = sg[tl * NBT + (SPLIT_T ? 0 : bh * NH) + j];
        acc[j].x = fma(d, g.x, acc[j].x);
        acc[j].y = fma(d, g.y, acc[j].y);
      }
    }
    __syncthreads();
  }
  if (SPLIT_T) {  // second half of the rings hands its sums to the first
    double2 *red = sg;  // free after the last tile
    if (bh == 1) red[li] = acc[0];
    __syncthreads();
    if (bh == 1) return;
    acc[0].x += red[li].x;
    acc[0].y += red[li].y;
  }
  const int l = lc + li;
  if (li >= n || l < lst) return;
  const double2 wt = weight_of(a, l);
#pragma unroll
  for (int j = 0; j < NH; ++j) {
    const int b = b0 + (SPLIT_T ? 0 : bh * NH) + j;
    if (b >= a.nb) break;
    const double2 v = make_double2(acc[j].x * r.sign, acc[j].y * r.sign);
    a.dst[(int64_t)b * a.ds + (int64_t)l * l + l + m] = cmul_(v, wt);
  }
}

// ---------------------------------------------------------------------------
// double-float variants (split-precision path on recomputed tables)
//
// The same two contractions with the per-map multiply-adds in double-float
// arithmetic on the FP32 pipe (dfarith.h), which GB300 issues at about 64
// times its FP64 rate.  The three-term recursion stays in FP64 (3 instructions
// per value, shared by all maps): in double-float its cancellation near the
// turning points cost 1e-11 of accuracy (2^-47 against 2^-53 per step over a
// 64-degree segment).  Each value is split into a double-float pair once
// (integer bit operations, dfconv.h) and multiplied into every map's partial
// sum; FP64 is otherwise left to the flush of the partial sums (two adds per
// output value and segment, or per tile of rings for t -> l).  Values are
// carried scaled by 2^-E per ring and segment as in the FP64 kernels, with a
// lower rescaling threshold (2^kRenormDf) so that they stay in the float
// range.  Coefficients (l -> t) and spectra (t -> l) enter as double-float
// scaled by the largest power of two of their block (segment or tile, per
// map).  Accumulators are renormalised after each add.
// ---------------------------------------------------------------------------

constexpr int kRenormDf = 60;

__device__ __forceinline__ float2 df_of(double v) {  // |v| within the float range
  float h, l;
  split_scaled(v, 0, h, l);
  return make_float2(h, l);
}
__device__ __forceinline__ float2 df_scale(float2 a, int k) { return make_float2(scale_pow2(a.x, k), scale_pow2(a.y, k)); }
// Rescaled recursion of one segment (double-float kernels): with v_l =
// lam_l w_l, lam_{lc} = lam_{lc+1} = 1 and lam_{l+1} = c2_l lam_{l-1}, the
// three-term step v_{l+1} = (p u + q) v_l - c2_l v_{l-1} becomes
// w_{l+1} = (p' u + q') w_l - w_{l-1} with (p', q') = (p, q) lam_l / (c2_l
// lam_{l-1}): two FP64 instructions per value instead of three.  lam depends
// on (l, m) only, so it is folded into the coefficients (l -> t) or the output
// weight (t -> l).  On entry cn / cs / c2 hold the coefficients of degrees
// lc + i, i in [1, n); on exit cn / cs the rescaled pairs and lam[i], i < n.
// Called by all threads of the block (contains barriers).
__device__ void rescale_segment(double2 *cn, double2 *cs, const double *c2, double *lam, int n) {
  __syncthreads();
  if (threadIdx.x == 0) {
    lam[0] = 1.0;
    if (n > 1) lam[1] = 1.0;
    for (int i = 1; i + 1 < n; ++i) lam[i + 1] = c2[i] * lam[i - 1];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x)
    if (i >= 1) {
      const double f = lam[i] / (c2[i] * lam[i - 1]);
      cn[i] = make_double2(cn[i].x * f, cn[i].y * f);
      cs[i] = make_double2(cs[i].x * f, cs[i].y * f);
    }
  __syncthreads();
}



template <int NBT>
__global__ void __launch_bounds__(kRcT) k_rc_l2t_df(RcArgs a) {
  __shared__ double2 scn[kSeg], scs[kSeg];
  __shared__ double sc2[kSeg], slam[kSeg];
  __shared__ double2 sxd[kSeg][NBT];  // weighted coefficients of the segment
  __shared__ float4 sx[kSeg][NBT];    // the same as double-float, scaled by 2^-sxs[b]
  __shared__ int sxm[NBT], sxs[NBT];
  const int m = a.mlo + blockIdx.x;
  const int am = m < 0 ? -m : m;
  const RcRef r = rc_ref(a, m);
  const int amt = r.mt < 0 ? -r.mt : r.mt;
  const int l0 = amt > a.an ? amt : a.an, bl = a.bl, nl = bl - l0;
  const int lst = l0 > a.lmin ? l0 : a.lmin;
  const int t = blockIdx.y * kRcT + threadIdx.x;
  const bool live = t < a.nt;
  const int b0 = blockIdx.z * NBT;
  double2 acc[NBT];
#pragma unroll
  for (int b = 0; b < NBT; ++b) acc[b] = make_double2(0.0, 0.0);
  double u = 0.0;
  bool north = true;
  if (live) {
    const double2 q = a.uq[t];
    u = q.x;
    north = q.y != 0.0;
  }
  if (nl > 0 && lst < bl) {
    const int nseg = (nl + kSeg - 1) / kSeg, c0 = (lst - l0) / kSeg;
    const double2 *ck = a.ck + a.coff[r.mi];
    const int *cke = a.ck_e + a.coff[r.mi];
    const double2 *cc = north ? scn : scs;
    for (int c = c0; c < nseg; ++c) {
      const int lc = l0 + c * kSeg, n = min(kSeg, bl - lc);
      __syncthreads();
      for (int i = threadIdx.x; i < n; i += kRcT)
        if (i >= 1) rec_coef(lc + i, r.mt, a.an, scn[i], scs[i], sc2[i]);
      if (threadIdx.x < NBT) sxm[threadIdx.x] = 0;
      rescale_segment(scn, scs, sc2, slam, n);
      for (int i = threadIdx.x; i < kSeg * NBT; i += kRcT) {
        const int kk = i / NBT, b = i % NBT, l = lc + kk;
        double2 v = make_double2(0.0, 0.0);
        if (kk < n && l >= lst && b0 + b < a.nb) {
          const int64_t base = (int64_t)(b0 + b) * a.ss + (int64_t)l * l + l;
          if (a.x_half && m < 0) {
            v = a.src[base - m];
            v.y = -v.y;
            if (am & 1) v = make_double2(-v.x, -v.y);
          } else {
            v = a.src[base + m];
          }
          const double2 wl = weight_of(a, l);
          v = cmul_(v, make_double2(wl.x * slam[kk], wl.y * slam[kk]));
        }
        sxd[kk][b] = v;
        atomicMax(&sxm[b], max(exp_bits(v.x), exp_bits(v.y)));
      }
      __syncthreads();
      if (threadIdx.x < NBT) sxs[threadIdx.x] = block_scale(sxm[threadIdx.x]);
      __syncthreads();
      for (int i = threadIdx.x; i < kSeg * NBT; i += kRcT) {
        const int kk = i / NBT, b = i % NBT;
        sx[kk][b] = dc_split(sxd[kk][b], sxs[b]);
      }
      __syncthreads();
      if (!live) continue;
      int E = cke[(int64_t)c * a.nt + t];
      if (E < -1074 - 2 * kRenorm) continue;  // the whole segment is below the double range
      const double2 ab = ck[(int64_t)c * a.nt + t];
      double vp = ab.x, v = ab.y;
      float4 sum[NBT];
      {
        const float2 dvp = df_of(vp), dv = df_of(v);
#pragma unroll
        for (int b = 0; b < NBT; ++b) {
          sum[b] = make_float4(0.f, 0.f, 0.f, 0.f);
          df_mac(sum[b], dvp, sx[0][b]);
          if (n > 1) df_mac(sum[b], dv, sx[1][b]);
        }
      }
      for (int i = 1; i + 1 < n; ++i) {
        const double2 k = cc[i];
        const double xt = fma(k.x, u, k.y);
        const double vn = fma(xt, v, -vp);  // rescaled recursion
        vp = v;
        v = vn;
        if (exp_bits(v) > 1023 + kRenormDf) {  // flush at the old scale, continue at the new one
#pragma unroll
          for (int b = 0; b < NBT; ++b) {
            const double2 f = dc_to(sum[b], E + sxs[b]);
            acc[b].x += f.x;
            acc[b].y += f.y;
            sum[b] = make_float4(0.f, 0.f, 0.f, 0.f);
          }
          v = ldexp(v, -kRenormDf);
          vp = ldexp(vp, -kRenormDf);
          E += kRenormDf;
        }
        const float2 dv = df_of(v);
#pragma unroll
        for (int b = 0; b < NBT; ++b) df_mac(sum[b], dv, sx[i + 1][b]);
      }
#pragma unroll
      for (int b = 0; b < NBT; ++b) {
        const double2 f = dc_to(sum[b], E + sxs[b]);
        acc[b].x += f.x;
        acc[b].y += f.y;
      }
    }
  }
  if (!live) return;
#pragma unroll
  for (int b = 0; b < NBT; ++b) {
    if (b0 + b >= a.nb) break;
    a.dst[(int64_t)(b0 + b) * a.ds + (int64_t)t * a.dw + (m - a.d_mlo)] =
        make_double2(acc[b].x * r.sign, acc[b].y * r.sign);
  }
}

template <int NBT>
size_t rc_t2l_df_smem() {
  return sizeof(float2) * kRcT * kTileLd + sizeof(float4) * kRcT * NBT;
}

// t -> l in double-float: the tile rows (one ring each, scaled by 2^-E_t)
// as double-float pairs; the spectra enter scaled by 2^(E_t - es[b]) with es[b]
// the largest exponent of spectrum times ring scale over the tile, so the
// sums over the tile's rings share one power of two and are flushed to FP64
// once per tile.
template <int NBT>
__global__ void __launch_bounds__(kRcT) k_rc_t2l_df(RcArgs a) {
  static_assert(NBT == 1 || NBT % 2 == 0, "one map, or two map halves");
  constexpr int NH = NBT == 1 ? 1 : NBT / 2;
  constexpr bool SPLIT_T = NBT == 1;
  extern __shared__ float2 smem_df[];
  float2 *tile = smem_df;                                  // [kRcT][kTileLd]
  float4 *sg = (float4 *)(smem_df + kRcT * kTileLd);       // [kRcT][NBT]
  __shared__ double2 scn[kSeg], scs[kSeg];
  __shared__ double sc2[kSeg], slam[kSeg];
  __shared__ int sgm[NBT];
  const int m = a.mlo + blockIdx.x, c = blockIdx.y;
  const RcRef r = rc_ref(a, m);
  const int amt = r.mt < 0 ? -r.mt : r.mt;
  const int l0 = amt > a.an ? amt : a.an, bl = a.bl, nl = bl - l0;
  const int lst = l0 > a.lmin ? l0 : a.lmin;
  const int nseg = nl > 0 ? (nl + kSeg - 1) / kSeg : 0;
  if (c >= nseg) return;
  const int lc = l0 + c * kSeg, n = min(kSeg, bl - lc);
  if (lc + n <= lst) return;  // every degree of the segment is below lmin: no output
  const int b0 = blockIdx.z * NBT;
  const int tid = threadIdx.x;
  for (int i = tid; i < n; i += kRcT)
    if (i >= 1) rec_coef(lc + i, r.mt, a.an, scn[i], scs[i], sc2[i]);
  rescale_segment(scn, scs, sc2, slam, n);
  const double2 *ck = a.ck + a.coff[r.mi] + (int64_t)c * a.nt;
  const int *cke = a.ck_e + a.coff[r.mi] + (int64_t)c * a.nt;
  const int li = tid % kSeg, bh = tid / kSeg;
  double2 acc[NH];
#pragma unroll
  for (int j = 0; j < NH; ++j) acc[j] = make_double2(0.0, 0.0);
  for (int t0 = 0; t0 < a.nt; t0 += kRcT) {
    const int t = t0 + tid;
    float2 *row = tile + tid * kTileLd;
    int E = kCkZeroExp;
    if (t < a.nt) E = cke[t];
    const bool on = E >= -1074 - 2 * kRenorm;
    if (on) {
      const double2 q = a.uq[t];
      const double u = q.x;
      const double2 *cc = q.y != 0.0 ? scn : scs;
      const double2 ab = ck[t];
      double vp = ab.x, v = ab.y;
      row[0] = df_of(vp);
      if (n > 1) row[1] = df_of(v);
      for (int i = 1; i + 1 < n; ++i) {
        const double2 k = cc[i];
        const double xt = fma(k.x, u, k.y);
        const double vn = fma(xt, v, -vp);  // rescaled recursion
        vp = v;
        v = vn;
        if (exp_bits(v) > 1023 + kRenormDf) {  // keep one scale per row: rescale what is written
          for (int j = 0; j <= i; ++j) row[j] = df_scale(row[j], -kRenormDf);
          v = ldexp(v, -kRenormDf);
          vp = ldexp(vp, -kRenormDf);
          E += kRenormDf;
        }
        row[i + 1] = df_of(v);
      }
      for (int i = n; i < kSeg; ++i) row[i] = make_float2(0.f, 0.f);
    } else {
      for (int i = 0; i < kSeg; ++i) row[i] = make_float2(0.f, 0.f);
    }
    // the spectra of this ring times 2^E, and the tile's largest exponent per map
    if (tid < NBT) sgm[tid] = -(1 << 30);
    __syncthreads();
    double2 g[NBT];
#pragma unroll
    for (int b = 0; b < NBT; ++b) {
      g[b] = make_double2(0.0, 0.0);
      if (on && b0 + b < a.nb) {
        g[b] = a.src[(int64_t)(b0 + b) * a.ss + (int64_t)t * a.sw + (m - a.s_mlo)];
        const int ex = max(exp_bits(g[b].x), exp_bits(g[b].y));
        if (ex > 0) atomicMax(&sgm[b], ex + E);
      }
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < NBT; ++b) {
      const int es = sgm[b] > -(1 << 29) ? block_scale(sgm[b]) : 0;
      sg[tid * NBT + b] = on ? dc_split(g[b], es - E) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    const int tl_end = min(kRcT, a.nt - t0);
    const int tl_lo = SPLIT_T ? bh * (kRcT / 2) : 0;
    const int tl_hi = SPLIT_T ? min(tl_end, tl_lo + kRcT / 2) : tl_end;
    float4 sum[NH];
#pragma unroll
    for (int j = 0; j < NH; ++j) sum[j] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 4
    for (int tl = tl_lo; tl < tl_hi; ++tl) {
      const float2 d = tile[tl * kTileLd + li];
#pragma unroll
      for (int j = 0; j < NH; ++j) df_mac(sum[j], d, sg[tl * NBT + (SPLIT_T ? 0 : bh * NH) + j]);
    }
#pragma unroll
    for (int j = 0; j < NH; ++j) {
      const int b = (SPLIT_T ? 0 : bh * NH) + j;
      const int es = sgm[b] > -(1 << 29) ? block_scale(sgm[b]) : 0;
      const double2 f = dc_to(sum[j], es);
      acc[j].x += f.x;
      acc[j].y += f.y;
    }
    __syncthreads();
  }
  if (SPLIT_T) {  // second half of the rings hands its sums to the first
    double2 *red = (double2 *)sg;  // free after the last tile
    if (bh == 1) red[li] = acc[0];
    __syncthreads();
    if (bh == 1) return;
    acc[0].x += red[li].x;
    acc[0].y += red[li].y;
  }
  const int l = lc + li;
  if (li >= n || l < lst) return;
  const double2 wt = weight_of(a, l);
  const double sl = r.sign * slam[li];  // the rescaled recursion's lam_l
#pragma unroll
  for (int j = 0; j < NH; ++j) {
    const int b = b0 + (SPLIT_T ? 0 : bh * NH) + j;
    if (b >= a.nb) break;
    const double2 v = make_double2(acc[j].x * sl, acc[j].y * sl);
    a.dst[(int64_t)b * a.ds + (int64_t)l * l + l + m] = cmul_(v, wt);
  }
}

// ---------------------------------------------------------------------------
// quadrature operator on ring spectra
// ---------------------------------------------------------------------------

// out[b][i][m - o_mlo] = sum_k A_m[i][k] in[b][k][m - i_mlo], i, k < nt, for the
// m in [mlo, mhi] with (m + an) even (parity 0, W_+) or odd (parity 1, W_-);
// A = W (trans = 0) or W^T (trans = 1).  Columns are the (map, m) pairs of the
// parity, each complex column two real ones.  64 x 64 output tile per CTA.
constexpr int AW_T = 64, AW_K = 16;
__global__ void __launch_bounds__(256) k_apply_w(const double *__restrict__ Wp, const double *__restrict__ Wm,
                                                 int trans, int nt, int an, int mlo, int mhi,
                                                 const double2 *__restrict__ in, int64_t is, int iw, int i_mlo,
                                                 double2 *__restrict__ out, int64_t os, int ow, int o_mlo, int nb) {
  const int par = blockIdx.z;
  const int m_first = ((mlo + an) & 1) == par ? mlo : mlo + 1;
  if (m_first > mhi) return;
  const int nmp = (mhi - m_first) / 2 + 1;  // m's of this parity
  const int ncols = 2 * nmp * nb;           // real columns
  const int row0 = blockIdx.y * AW_T, col0 = blockIdx.x * AW_T;
  if (row0 >= nt || col0 >= ncols) return;
  const double *W = par == 0 ? Wp : Wm;
  __shared__ double sA[AW_K][AW_T + 1];  // [k][row]
  __shared__ double sB[AW_K][AW_T + 1];  // [k][col]
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc[4][4] = {};
  for (int k0 = 0; k0 < nt; k0 += AW_K) {
    for (int i = threadIdx.x; i < AW_K * AW_T; i += 256) {
      // W rows are contiguous in k (trans = 0) or in the row index (trans = 1)
      const int kk = trans ? i / AW_T : i % AW_K, cc = trans ? i % AW_T : i / AW_K;
      const int k = k0 + kk;
      double av = 0.0;
      if (k < nt && row0 + cc < nt)
        av = trans ? W[(int64_t)k * nt + row0 + cc] : W[(int64_t)(row0 + cc) * nt + k];
      sA[kk][cc] = av;
    }
    for (int i = threadIdx.x; i < AW_K * AW_T; i += 256) {
      const int kk = i / AW_T, cc = i % AW_T;
      const int k = k0 + kk, col = col0 + cc;
      double bv = 0.0;
      if (k < nt && col < ncols) {
        const int pair = col >> 1, im = col & 1;
        const int b = pair / nmp, m = m_first + 2 * (pair % nmp);
        const double2 z = in[(int64_t)b * is + (int64_t)k * iw + (m - i_mlo)];
        bv = im ? z.y : z.x;
      }
      sB[kk][cc] = bv;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < AW_K; ++kk) {
      double x[4], y[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) x[i] = sA[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) y[j] = sB[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(x[i], y[j], acc[i][j]);
    }
    __syncthreads();
  }
  // columns tx*4 .. tx*4+3 are two complex columns (re, im pairs start even)
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int rr = row0 + ty * 4 + i;
    if (rr >= nt) continue;
#pragma unroll
    for (int j = 0; j < 4; j += 2) {
      const int col = col0 + tx * 4 + j;
      if (col >= ncols) continue;
      const int pair = col >> 1;
      const int b = pair / nmp, m = m_first + 2 * (pair % nmp);
      out[(int64_t)b * os + (int64_t)rr * ow + (m - o_mlo)] = make_double2(acc[i][j], acc[i][j + 1]);
    }
  }
}

// The same operator in double-float (split-precision path).  Per K-slab of
// AWD_K: W values as double-float pairs (unscaled: the operator's entries sit
// well inside the float range), each real column's slab as double-float
// scaled by its largest power of two; the slab's partial sums (renormalised
// double-float) are flushed into FP64 accumulators with that power of two.
// About 15 FP32 instructions per multiply-add against one FP64 instruction at
// 1/64 of the rate.
constexpr int AWD_K = 32;
__global__ void __launch_bounds__(256) k_apply_w_df(const double *__restrict__ Wp, const double *__restrict__ Wm,
                                                    int trans, int nt, int an, int mlo, int mhi,
                                                    const double2 *__restrict__ in, int64_t is, int iw, int i_mlo,
                                                    double2 *__restrict__ out, int64_t os, int ow, int o_mlo,
                                                    int nb) {
  const int par = blockIdx.z;
  const int m_first = ((mlo + an) & 1) == par ? mlo : mlo + 1;
  if (m_first > mhi) return;
  const int nmp = (mhi - m_first) / 2 + 1;  // m's of this parity
  const int ncols = 2 * nmp * nb;           // real columns
  const int row0 = blockIdx.y * AW_T, col0 = blockIdx.x * AW_T;
  if (row0 >= nt || col0 >= ncols) return;
  const double *W = par == 0 ? Wp : Wm;
  __shared__ float2 sA[AWD_K][AW_T + 1];  // [k][row]
  // [k][col]: first the FP64 values, then (in place, each thread converting the
  // entries it stored) their double-float pairs scaled by 2^-sBe[col]
  __shared__ float2 sB[AWD_K][AW_T + 1];
  __shared__ int sBm[AW_T], sBe[AW_T];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc[4][4] = {};
  for (int k0 = 0; k0 < nt; k0 += AWD_K) {
    if (threadIdx.x < AW_T) sBm[threadIdx.x] = 0;
    for (int i = threadIdx.x; i < AWD_K * AW_T; i += 256) {
      const int kk = trans ? i / AW_T : i % AWD_K, cc = trans ? i % AW_T : i / AWD_K;
      const int k = k0 + kk;
      double av = 0.0;
      if (k < nt && row0 + cc < nt)
        av = trans ? W[(int64_t)k * nt + row0 + cc] : W[(int64_t)(row0 + cc) * nt + k];
      sA[kk][cc] = df_of(av);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < AWD_K * AW_T; i += 256) {
      const int kk = i / AW_T, cc = i % AW_T;
      const int k = k0 + kk, col = col0 + cc;
      double bv = 0.0;
      if (k < nt && col < ncols) {
        const int pair = col >> 1, im = col & 1;
        const int b = pair / nmp, m = m_first + 2 * (pair % nmp);
        const double2 z = in[(int64_t)b * is + (int64_t)k * iw + (m - i_mlo)];
        bv = im ? z.y : z.x;
      }
      *reinterpret_cast<double *>(&sB[kk][cc]) = bv;
      atomicMax(&sBm[cc], exp_bits(bv));
    }
    __syncthreads();
    if (threadIdx.x < AW_T) sBe[threadIdx.x] = block_scale(sBm[threadIdx.x]);
    __syncthreads();
    for (int i = threadIdx.x; i < AWD_K * AW_T; i += 256) {
      const int kk = i / AW_T, cc = i % AW_T;
      sB[kk][cc] = df_split(*reinterpret_cast<const double *>(&sB[kk][cc]), sBe[cc]);
    }
    __syncthreads();
    float2 sum[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) sum[i][j] = make_float2(0.f, 0.f);
#pragma unroll 4
    for (int kk = 0; kk < AWD_K; ++kk) {
      float2 x[4], y[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) x[i] = sA[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) y[j] = sB[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) sum[i][j] = df_add_norm(sum[i][j], df_mul(x[i], y[j]));
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int e = sBe[tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i) acc[i][j] += join_scaled(sum[i][j].x, sum[i][j].y, e);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int rr = row0 + ty * 4 + i;
    if (rr >= nt) continue;
#pragma unroll
    for (int j = 0; j < 4; j += 2) {
      const int col = col0 + tx * 4 + j;
      if (col >= ncols) continue;
      const int pair = col >> 1;
      const int b = pair / nmp, m = m_first + 2 * (pair % nmp);
      out[(int64_t)b * os + (int64_t)rr * ow + (m - o_mlo)] = make_double2(acc[i][j], acc[i][j + 1]);
    }
  }
}

RcArgs rc_args(const WignerTable &tb, int n, int mlo, int lmin, const double2 *w, double wscale, bool wconj,
               int nb) {
  RcArgs a{};
  a.bl = tb.bl;
  a.nt = tb.nt;
  a.an = tb.an;
  a.tmlo = tb.mlo;
  a.n = n;
  a.coff = tb.d_coff;
  a.ck = tb.ck;
  a.ck_e = tb.ck_e;
  a.uq = tb.uq;
  a.mlo = mlo;
  a.lmin = lmin;
  a.w = w;
  a.wscale = wscale;
  a.wconj = wconj ? 1 : 0;
  a.nb = nb;
  return a;
}

// algorithmic work of one launch, as the stored path counts it (one complex x
// real MAC per (l, m, t) per map) plus the recursion (3 FP64 per value)
void rc_work(const WignerTable &tb, int mlo, int mhi, int lmin, int nb, double *flops, double *bytes) {
  double macs = 0;
  for (int m = mlo; m <= mhi; ++m) {
    const int am = m < 0 ? -m : m, l0 = std::max(am, tb.an), lst = std::max(l0, lmin);
    if (lst < tb.bl) macs += (double)(tb.bl - lst) * tb.nt;
  }
  *flops = 4.0 * macs * nb;
  *bytes = 16.0 * nb * (double)(mhi - mlo + 1) * (tb.nt + tb.bl);
}

void apply_w(const WignerTable &tb, bool trans, int mlo, int mhi, const double2 *in, int64_t is, int iw, int i_mlo,
             double2 *out, int64_t os, int ow, int o_mlo, int nb, cudaStream_t st) {
  const int nm = mhi - mlo + 1;
  const int ncols = 2 * ((nm + 1) / 2) * nb;
  KTimer kt(KC_QUAD, st, 2.0 * tb.nt * (double)tb.nt * nm * nb * 2.0, 16.0 * nb * (double)nm * tb.nt * 2.0);
  dim3 grid(ceil_div(ncols, AW_T), ceil_div(tb.nt, AW_T), 2);
  if (t_precision == 1)  // split precision: double-float multiply-adds
    k_apply_w_df<<<grid, 256, 0, st>>>(tb.W[0], tb.W[1], trans ? 1 : 0, tb.nt, tb.an, mlo, mhi, in, is, iw, i_mlo,
                                       out, os, ow, o_mlo, nb);
  else
    k_apply_w<<<grid, 256, 0, st>>>(tb.W[0], tb.W[1], trans ? 1 : 0, tb.nt, tb.an, mlo, mhi, in, is, iw, i_mlo,
                                    out, os, ow, o_mlo, nb);
  S2G_LAUNCHED();
}

template <int NBT>
void launch_l2t(const RcArgs &a, int nm, cudaStream_t st) {
  dim3 grid(nm, ceil_div(a.nt, kRcT), ceil_div(a.nb, NBT));
  k_rc_l2t<NBT><<<grid, kRcT, 0, st>>>(a);
  S2G_LAUNCHED();
}

template <int NBT>
void launch_t2l(const RcArgs &a, int nm, int maxseg, cudaStream_t st) {
  const size_t smem = rc_t2l_smem<NBT>();
  static const bool attr = [smem] {  // once per instantiation (thread-safe static initialisation)
    S2G_CUDA(cudaFuncSetAttribute(k_rc_t2l<NBT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    return true;
  }();
  (void)attr;
  dim3 grid(nm, maxseg, ceil_div(a.nb, NBT));
  k_rc_t2l<NBT><<<grid, kRcT, smem, st>>>(a);
  S2G_LAUNCHED();
}

template <int NBT>
void launch_l2t_df(const RcArgs &a, int nm, cudaStream_t st) {
  dim3 grid(nm, ceil_div(a.nt, kRcT), ceil_div(a.nb, NBT));
  k_rc_l2t_df<NBT><<<grid, kRcT, 0, st>>>(a);
  S2G_LAUNCHED();
}

template <int NBT>
void launch_t2l_df(const RcArgs &a, int nm, int maxseg, cudaStream_t st) {
  const size_t smem = rc_t2l_df_smem<NBT>();
  static const bool attr = [smem] {  // once per instantiation (thread-safe static initialisation)
    S2G_CUDA(cudaFuncSetAttribute(k_rc_t2l_df<NBT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    return true;
  }();
  (void)attr;
  dim3 grid(nm, maxseg, ceil_div(a.nb, NBT));
  k_rc_t2l_df<NBT><<<grid, kRcT, smem, st>>>(a);
  S2G_LAUNCHED();
}

}  // namespace

void contract_l2t_rc(const L2T &p, cudaStream_t st) {
  const WignerTable &tb = *p.tb;
  const int nm = p.mhi - p.mlo + 1;
  RcArgs a = rc_args(tb, p.n, p.mlo, p.lmin, p.w, p.wscale, p.wconj, p.nb);
  a.src = p.x;
  a.ss = p.xs;
  a.x_half = p.x_half ? 1 : 0;
  // Q^T x = W^T (D x): D x into a scratch of the output's layout, then W^T
  double2 *tmp = nullptr;
  if (p.use_q) {
    S2G_CUDA(cudaMallocAsync((void **)&tmp, sizeof(double2) * (size_t)p.nb * tb.nt * p.ow, st));
    a.dst = tmp;
    a.ds = (int64_t)tb.nt * p.ow;
  } else {
    a.dst = p.out;
    a.ds = p.os;
  }
  a.dw = p.ow;
  a.d_mlo = p.omlo;
  {
    double fl = 0, by = 0;
    if (timing_enabled()) rc_work(tb, p.mlo, p.mhi, p.lmin, p.nb, &fl, &by);
    // maps per CTA: the largest of 1/2/4/8 the batch fills, or the autotuned choice
    // split precision: the double-float kernels (same results to about 1e-13)
    const bool df = t_precision == 1;
    const auto run = [&](int nbc) {
      if (df) {
        switch (nbc) {
          case 8: launch_l2t_df<8>(a, nm, st); break;
          case 4: launch_l2t_df<4>(a, nm, st); break;
          case 2: launch_l2t_df<2>(a, nm, st); break;
          default: launch_l2t_df<1>(a, nm, st); break;
        }
        return;
      }
      switch (nbc) {
        case 8: launch_l2t<8>(a, nm, st); break;
        case 4: launch_l2t<4>(a, nm, st); break;
        case 2: launch_l2t<2>(a, nm, st); break;
        default: launch_l2t<1>(a, nm, st); break;
      }
    };
    static const int kCand[4] = {1, 2, 4, 8};
    const int ncand = p.nb >= 8 ? 4 : (p.nb >= 4 ? 3 : (p.nb >= 2 ? 2 : 1));
    const int c = tuned(TF_RC_L2T, tune_bucket(tb.bl), tune_bucket(p.nb), df ? 1 : 0, ncand, ncand - 1, st,
                        [&](int i) { run(kCand[i]); });
    KTimer kt(KC_RECOMPUTE, st, fl, by);
    run(kCand[c]);
  }
  if (p.use_q) {
    apply_w(tb, true, p.mlo, p.mhi, tmp, (int64_t)tb.nt * p.ow, p.ow, p.omlo, p.out, p.os, p.ow, p.omlo, p.nb, st);
    cudaFreeAsync(tmp, st);
  }
}

void contract_t2l_rc(const T2L &p, cudaStream_t st) {
  const WignerTable &tb = *p.tb;
  const int nm = p.mhi - p.mlo + 1;
  RcArgs a = rc_args(tb, p.n, p.mlo, p.lmin, p.w, p.wscale, p.wconj, p.nb);
  // Q in = D^T (W in): the quadrature on the spectra first
  double2 *tmp = nullptr;
  if (p.use_q) {
    S2G_CUDA(cudaMallocAsync((void **)&tmp, sizeof(double2) * (size_t)p.nb * tb.nt * p.iw, st));
    apply_w(tb, false, p.mlo, p.mhi, p.in, p.is, p.iw, p.imlo, tmp, (int64_t)tb.nt * p.iw, p.iw, p.imlo, p.nb, st);
    a.src = tmp;
    a.ss = (int64_t)tb.nt * p.iw;
  } else {
    a.src = p.in;
    a.ss = p.is;
  }
  a.sw = p.iw;
  a.s_mlo = p.imlo;
  a.dst = p.y;
  a.ds = p.ys;
  int maxseg = 1;
  for (int m = p.mlo; m <= p.mhi; ++m) maxseg = std::max(maxseg, tb.nseg(m < 0 ? -m : m));
  {
    double fl = 0, by = 0;
    if (timing_enabled()) rc_work(tb, p.mlo, p.mhi, p.lmin, p.nb, &fl, &by);
    // maps per CTA: the largest of 1/2/4/8/16 the batch fills, or the autotuned choice
    const bool df = t_precision == 1;  // split precision: the double-float kernels
    const auto run = [&](int nbc) {
      if (df) {
        switch (nbc) {
          case 16: launch_t2l_df<16>(a, nm, maxseg, st); break;
          case 8: launch_t2l_df<8>(a, nm, maxseg, st); break;
          case 4: launch_t2l_df<4>(a, nm, maxseg, st); break;
          case 2: launch_t2l_df<2>(a, nm, maxseg, st); break;
          default: launch_t2l_df<1>(a, nm, maxseg, st); break;
        }
        return;
      }
      switch (nbc) {
        case 16: launch_t2l<16>(a, nm, maxseg, st); break;
        case 8: launch_t2l<8>(a, nm, maxseg, st); break;
        case 4: launch_t2l<4>(a, nm, maxseg, st); break;
        case 2: launch_t2l<2>(a, nm, maxseg, st); break;
        default: launch_t2l<1>(a, nm, maxseg, st); break;
      }
    };
    static const int kCand[5] = {1, 2, 4, 8, 16};
    const int ncand = p.nb >= 16 ? 5 : (p.nb >= 8 ? 4 : (p.nb >= 4 ? 3 : (p.nb >= 2 ? 2 : 1)));
    const int c = tuned(TF_RC_T2L, tune_bucket(tb.bl), tune_bucket(p.nb), df ? 1 : 0, ncand, ncand - 1, st,
                        [&](int i) { run(kCand[i]); });
    KTimer kt(KC_RECOMPUTE, st, fl, by);
    run(kCand[c]);
  }
  if (tmp) cudaFreeAsync(tmp, st);
}

}  // namespace s2g
