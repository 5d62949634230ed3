// Split-precision contraction on tcgen05 (see mixed.h for the number format).
//
// Layout in HBM
//   Sliced table, one per (band-limit, |n|, D or Q): for each table m, for each
//   128-row tile rt, for each 64-wide K-chunk kc, for each digit slice j, a
//   16 KB panel [128 rows][64 bf16] in the 128-byte-swizzled K-major image that
//   tcgen05 reads from shared memory; rows and K are zero-padded to the panel.
//   Row exponents eA (int8) per (m, row).
//   Sliced coefficients, per call and per problem m: for each kc one 14 KB
//   panel [7 slices x 16 columns][64 bf16] (16 real columns = 8 complex maps),
//   column exponents eX (int32) per (m, column).
//
// Kernel k_contract_mx<NC>: persistent, one CTA per SM, 18 warps; NC real
// coefficient columns (16, 32 or 64) per table pass.
//   warp 0    producer: cp.async.bulk of panels into a ring of 16 KB table
//             stages (10 deep; 6 at NC = 64) and a 2-deep ring of coefficient
//             stages (7 slices x NC columns x 64 K).
//   warp 1    MMA issuer: per K-chunk and digit slice j, one 128 x N x 64
//             product (tcgen05.mma of K=16, N <= 256 each) of table slice j
//             against the first 7-j coefficient slices, written to the
//             accumulator columns of classes j..6 (N = NC (7-j)); two TMEM
//             accumulators alternate between tiles (one at NC = 64).
//   warps 2-17 epilogue: four warps per TMEM lane quarter, 16 columns each:
//             tcgen05.ld of the 7 class accumulators, double-float combine,
//             row/column exponents, sign, per-l weight, store; the
//             accumulator is released as soon as its values are in registers.
// Every wait is bounded (about 2 s); on expiry the kernel raises an error flag,
// drains its own copies and MMAs, frees TMEM and returns.
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>
#include <vector>

#include "autotune.h"
#include "common.h"
#include "dfconv.h"
#include "kernels.h"
#include "mixed.h"
#include "plan.h"
#include "timing.h"

namespace s2g {

namespace {

constexpr int kS = 7;                  // digit slices per operand
constexpr int kB0 = 6;                 // bits of the first digit (later digits: 7)
constexpr int kPK = 64;                // K per panel
constexpr int kPM = 128;               // rows per panel
constexpr int kPanelA = kPM * kPK;     // 8192 elements, 16 KB
constexpr int kMaxParts = 2;           // scales sharing one table pass
constexpr int kXST = 2;                // coefficient pipeline depth
constexpr int kEpiWarps = 16;          // four warps per TMEM lane quarter, one 16-column chunk each
constexpr int kThreads = 64 + 32 * kEpiWarps;
constexpr int kMinBl = 128;            // below this the FP64 kernel is used
constexpr long long kWaitCycles = 4000000000LL;

// NC real coefficient columns per CTA (16, 32 or 64): parts x maps x {re, im}.
// NC <= 32: two TMEM accumulators alternate between tiles; NC = 64: one
// accumulator of 448 columns, and a shallower table ring to fit shared memory.
template <int NC>
struct Cfg {
  static constexpr int kAST = NC == 64 ? 6 : 10;       // table pipeline depth
  static constexpr int kNBuf = NC == 64 ? 1 : 2;       // TMEM accumulators
  static constexpr int kPanelX = kS * NC * kPK;        // elements
  static constexpr int kAccCols = kS * NC;             // TMEM columns per accumulator
  static constexpr int kTmemCols = NC == 16 ? 256 : 512;
  static constexpr size_t kSmemA = (size_t)kAST * kPanelA * 2;
  static constexpr size_t kSmemX = (size_t)kXST * kPanelX * 2;
  static constexpr int kNumBars = 2 * kAST + 2 * kXST + 4 + 1;
  static constexpr size_t kSmemBytes = 1024 + kSmemA + kSmemX + kNumBars * 8 + 16;
};
static_assert(Cfg<64>::kSmemBytes <= 232448, "shared memory");
static_assert(Cfg<32>::kSmemBytes <= 232448, "shared memory");
static_assert(Cfg<64>::kNBuf * Cfg<64>::kAccCols <= Cfg<64>::kTmemCols, "TMEM");
static_assert(Cfg<32>::kNBuf * Cfg<32>::kAccCols <= Cfg<32>::kTmemCols, "TMEM");
static_assert(Cfg<16>::kNBuf * Cfg<16>::kAccCols <= Cfg<16>::kTmemCols, "TMEM");

struct Geom {
  int l0, nl, rows, K, nkc, nrt;
};
// Tile geometry of one m block of a table with nt theta samples: l -> t has
// rows t < nt and reduction K = l - l0; t -> l has rows l - l0 and K = t.
__host__ __device__ inline Geom geom(int bl, int nt, int an, int m, bool q) {
  Geom g;
  const int am = m < 0 ? -m : m;
  g.l0 = am > an ? am : an;
  g.nl = bl - g.l0 > 0 ? bl - g.l0 : 0;
  g.rows = q ? g.nl : nt;
  g.K = q ? nt : g.nl;
  g.nkc = g.nl > 0 ? (g.K + kPK - 1) / kPK : 0;
  g.nrt = (g.rows + kPM - 1) / kPM;  // l -> t keeps its rows (written as zeros) when nl = 0
  return g;
}

// element index of (row, col) inside a [rows][64] bf16 K-major panel with the
// 128-byte swizzle: 16-byte chunk index XOR (row mod 8), 8-row atoms of 1024 B
__host__ __device__ inline int swz(int row, int col) {
  const int chunk = (col >> 3) ^ (row & 7);
  return (row >> 3) * 512 + (row & 7) * 64 + chunk * 8 + (col & 7);
}


// Balanced digits of q = round(v 2^(48-e)), |v| < 2^e: q = sum_j d_j 2^(42-7j)
// with d_1..d_6 in [-64, 63] (base-128 digits taken from the low end) and
// d_0 in [-64, 64].  Integer arithmetic only, so the split costs no FP64 work.
__device__ __forceinline__ void int_digits(long long q, int *d) {
#pragma unroll
  for (int j = kS - 1; j >= 1; --j) {
    int r = (int)(q & 127);
    if (r >= 64) r -= 128;
    d[j] = r;
    q = (q - r) >> 7;
  }
  d[0] = (int)q;
}
__device__ __forceinline__ uint16_t bf16_of_int(int d) {
  // |d| <= 64: exact in bf16 (top half of the fp32 pattern)
  return (uint16_t)(__float_as_uint((float)d) >> 16);
}
// round(v 2^(48-e)) for |v| < 2^e, from the significand bits (no FP64 work)
__device__ __forceinline__ long long fixed48(double v, int e) {
  const uint64_t u = bits_of(v);
  const int E = (int)((u >> 52) & 0x7FF);
  if (E == 0) return 0;
  const long long M = (long long)((u & 0xFFFFFFFFFFFFFull) | (1ull << 52));
  const int sh = E - 1075 + 48 - e;  // v 2^(48-e) = M 2^sh
  long long q;
  if (sh >= 0)
    q = M << sh;  // |v| < 2^e keeps this below 2^48
  else if (sh > -64)
    q = (M + (1ll << (-sh - 1))) >> (-sh);
  else
    q = 0;
  return (u >> 63) ? -q : q;
}

// digits of v 2^-e as bf16 bit patterns
__device__ __forceinline__ void split_digits(double v, int e, uint16_t *out) {
  int d[kS];
  int_digits(fixed48(v, e), d);
#pragma unroll
  for (int j = 0; j < kS; ++j) out[j] = bf16_of_int(d[j]);
}


struct TableRefM {
  int mi;
  double sign;
};
__device__ __forceinline__ TableRefM table_ref_m(int tmlo, int n, int m) {
  TableRefM r;
  if (n > 0 || (n == 0 && m >= 0)) {
    r.mi = m - tmlo;
    r.sign = 1.0;
  } else {
    const int an = n < 0 ? -n : n;
    r.mi = -m - tmlo;
    r.sign = ((m + an) & 1) ? -1.0 : 1.0;
  }
  return r;
}

// ---------------------------------------------------------------------------
// table slicing (plan time)
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(128) k_slice_table(const double *__restrict__ T,
                                                     const int64_t *__restrict__ off, int bl, int nt,
                                                     int an, int tmlo, int q, uint16_t *__restrict__ panels,
                                                     const int64_t *__restrict__ pan_off,
                                                     int8_t *__restrict__ eA,
                                                     const int64_t *__restrict__ e_off) {
  const int mi = blockIdx.x, rt = blockIdx.y;
  const Geom g = geom(bl, nt, an, tmlo + mi, q != 0);
  if (rt >= g.nrt) return;
  const double *Tm = T + off[mi];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int kpad = g.nkc * kPK;
  for (int rr = warp; rr < kPM; rr += 4) {
    const int row = rt * kPM + rr;
    const bool live = row < g.rows;
    int mx = 0;
    if (live)
      for (int k = lane; k < g.K; k += 32) mx = max(mx, exp_field(Tm[(int64_t)row * g.K + k]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    int e = block_scale(mx);
    e = e < -126 ? -126 : (e > 126 ? 126 : e);
    if (lane == 0) eA[e_off[mi] + row] = (int8_t)e;
    for (int k = lane; k < kpad; k += 32) {
      const double v = (live && k < g.K) ? Tm[(int64_t)row * g.K + k] : 0.0;
      uint16_t dg[kS];
      split_digits(v, e, dg);
      const int kc = k / kPK;
      uint16_t *p = panels + pan_off[mi] + (int64_t)(rt * g.nkc + kc) * kS * kPanelA;
      const int idx = swz(rr, k % kPK);
#pragma unroll
      for (int j = 0; j < kS; ++j) p[(int64_t)j * kPanelA + idx] = dg[j];
    }
  }
}

// ---------------------------------------------------------------------------
// coefficient slicing (per call)
// ---------------------------------------------------------------------------

// One scale's coefficients and outputs inside a fused table pass.
struct Part {
  const double2 *src;  // l -> t: flm-like (l^2 + l + m); t -> l: spectra [t][m - s_mlo]
  int64_t ss;
  int sw, s_mlo, x_half;
  const double2 *w;  // per-l weight (l -> t: on the input; t -> l: on the output)
  double wscale;
  int wconj;
  int wkind;  // WKIND_* of w
  int lmin;
  double2 *dst;  // l -> t: spectra [t][m - d_mlo] (row width dw); t -> l: l^2 + l + m
  int64_t ds;
  int dw, d_mlo;
};

struct XArgs {
  int q;  // 0: l -> t (K = l - l0), 1: t -> l (K = t)
  int bl, nt, an, mlo, lmin;  // lmin: smallest lmin over the parts
  int nparts;
  Part part[kMaxParts];
  int nb, b0, mpp;  // maps per part in this launch: column pair cp -> part cp / mpp, map b0 + cp % mpp
  int nmp;          // problem m count
  int nkcmax, kst;  // largest K-chunk count over the problem m; staged column stride (double2)
  const int64_t *xoff;
  uint16_t *xpan;
  int *eX;
};

__device__ __forceinline__ double2 weight_of(const double2 *w, double wscale, int wconj, int l) {
  double2 v = w ? w[l] : make_double2(1.0, 0.0);
  if (wconj) v.y = -v.y;
  return make_double2(v.x * wscale, v.y * wscale);
}
// x times the part's weight at degree l (x times wscale without a weight).  A
// real or imaginary weight takes three FP64 products instead of the eight of a
// scaled complex product; the terms dropped are exact zeros, so the result is
// the same.
__device__ __forceinline__ double2 weighted(const Part &P, double2 x, int l) {
  if (!P.w) return make_double2(x.x * P.wscale, x.y * P.wscale);
  if (P.wkind == WKIND_REAL) {
    const double r = P.w[l].x * P.wscale;
    return make_double2(x.x * r, x.y * r);
  }
  if (P.wkind == WKIND_IMAG) {  // x (i r)
    const double r = (P.wconj ? -P.w[l].y : P.w[l].y) * P.wscale;
    return make_double2(-(x.y * r), x.x * r);
  }
  const double2 wt = weight_of(P.w, P.wscale, P.wconj, l);
  return make_double2(x.x * wt.x - x.y * wt.y, x.x * wt.y + x.y * wt.x);
}

// Coefficient slicing: one block per (kMG consecutive problem m, column pair
// cp = part cp / mpp, map b0 + cp % mpp).  Phase 1 stages the kMG complex
// columns in shared memory, reading the source with m as the contiguous index
// (flm-like l^2 + l + m for l -> t, spectra [t][m] for t -> l), so that a warp
// load covers 64-byte runs, and records the largest exponent field of each
// real and imaginary column.  Phase 2 writes the digit panels: 8 consecutive
// lanes build one 128-byte panel row from 8 K values each.  The FP64 values
// are read once and the panels written once.
constexpr int kMG = 4;
constexpr int kSliceThreads = 256;
// staged index of K position k: one double2 of padding per 8, so that the
// 16-byte reads of 8 lanes at K stride 8 fall in distinct banks
__host__ __device__ __forceinline__ int sv_idx(int k) { return k + (k >> 3); }

template <int NC>
__global__ void __launch_bounds__(kSliceThreads, 3) k_slice_x(XArgs a) {
  extern __shared__ double2 sv[];  // [kMG][a.kst]
  __shared__ int gl0[kMG], gnkc[kMG], gkc0[kMG], gls[kMG], gex[kMG][2];
  constexpr int PX = Cfg<NC>::kPanelX;
  const int cp = blockIdx.y, pm0 = blockIdx.x * kMG, c0 = 2 * cp;
  const int part = cp / a.mpp, b = a.b0 + cp % a.mpp;
  const bool live = part < a.nparts && b < a.nb;
  if (threadIdx.x < kMG) {
    const int pm = pm0 + threadIdx.x;
    int l0 = 0, nkc = 0, kc0 = 0, ls = 0;
    if (pm < a.nmp) {
      const Geom g = geom(a.bl, a.nt, a.an, a.mlo + pm, a.q != 0);
      l0 = g.l0;
      nkc = g.nkc;
      if (!a.q) {
        const int lst = g.l0 > a.lmin ? g.l0 : a.lmin;
        kc0 = lst >= a.bl ? g.nkc : (lst - g.l0) / kPK;
        // first degree with a value: below its part's lmin the column is zero
        ls = live && a.part[part].lmin > g.l0 ? a.part[part].lmin : g.l0;
      }
    }
    gl0[threadIdx.x] = l0;
    gnkc[threadIdx.x] = nkc;
    gkc0[threadIdx.x] = kc0;
    gls[threadIdx.x] = ls;
    gex[threadIdx.x][0] = gex[threadIdx.x][1] = 0;
  }
  for (int i = threadIdx.x; i < kMG * a.kst; i += kSliceThreads) ((int4 *)sv)[i] = make_int4(0, 0, 0, 0);
  __syncthreads();
  if (live) {
    const Part &P = a.part[part];
    const int mi = threadIdx.x % kMG;  // fixed per thread: kSliceThreads is a multiple of kMG
    const int pm = pm0 + mi, m = a.mlo + pm, am = m < 0 ? -m : m;
    const bool has = pm < a.nmp && gnkc[mi] > gkc0[mi];
    double2 *col = sv + mi * a.kst;
    int er = 0, ei = 0;
    constexpr int kStep = kSliceThreads / kMG, kU = 4;  // kU loads in flight per thread
    if (!a.q) {
      // every lane walks the same degrees, so the kMG m of one degree are adjacent
      int lb = a.bl;
      for (int i = 0; i < kMG; ++i)
        if (pm0 + i < a.nmp && gnkc[i] > gkc0[i]) lb = min(lb, gls[i]);
      const int l0 = gl0[mi], ls = gls[mi];
      const bool neg = P.x_half && m < 0;
      const int mm = neg ? -m : m;
      for (int l1 = lb + threadIdx.x / kMG; l1 < a.bl; l1 += kU * kStep) {
        double2 v[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          const int l = l1 + u * kStep;
          v[u] = make_double2(0.0, 0.0);
          if (has && l >= ls && l < a.bl) v[u] = P.src[(int64_t)b * P.ss + (int64_t)l * l + l + mm];
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          const int l = l1 + u * kStep;
          if (!has || l < ls || l >= a.bl) continue;
          double2 x = v[u];
          if (neg) {
            x.y = -x.y;
            if (am & 1) x = make_double2(-x.x, -x.y);
          }
          x = weighted(P, x, l);
          col[sv_idx(l - l0)] = x;
          er = max(er, exp_field(x.x));
          ei = max(ei, exp_field(x.y));
        }
      }
    } else if (has) {
      const double2 *src = P.src + (int64_t)b * P.ss + (m - P.s_mlo);
      for (int t1 = threadIdx.x / kMG; t1 < a.nt; t1 += kU * kStep) {
        double2 v[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          const int t = t1 + u * kStep;
          v[u] = t < a.nt ? src[(int64_t)t * P.sw] : make_double2(0.0, 0.0);
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
          const int t = t1 + u * kStep;
          if (t >= a.nt) continue;
          col[sv_idx(t)] = v[u];
          er = max(er, exp_field(v[u].x));
          ei = max(ei, exp_field(v[u].y));
        }
      }
    }
    // lanes with the same m are kMG apart
#pragma unroll
    for (int o = kMG; o < 32; o <<= 1) {
      er = max(er, __shfl_xor_sync(0xffffffffu, er, o));
      ei = max(ei, __shfl_xor_sync(0xffffffffu, ei, o));
    }
    if ((threadIdx.x & 31) < kMG) {
      atomicMax(&gex[mi][0], er);
      atomicMax(&gex[mi][1], ei);
    }
  }
  __syncthreads();
  if (threadIdx.x < kMG) {
    const int pm = pm0 + threadIdx.x;
    // |v| < 2^e for every value of the column (e = largest unbiased exponent + 1)
    const int er = block_scale(gex[threadIdx.x][0]), ei = block_scale(gex[threadIdx.x][1]);
    gex[threadIdx.x][0] = er;
    gex[threadIdx.x][1] = ei;
    if (pm < a.nmp) {
      a.eX[pm * NC + c0] = er;
      a.eX[pm * NC + c0 + 1] = ei;
    }
  }
  __syncthreads();
  const int units = kMG * a.nkcmax * 8;
  for (int u = threadIdx.x; u < units; u += kSliceThreads) {
    const int h = u & 7, rest = u >> 3;
    const int kc = rest % a.nkcmax, mi = rest / a.nkcmax;
    const int pm = pm0 + mi;
    if (pm >= a.nmp || kc < gkc0[mi] || kc >= gnkc[mi]) continue;
    uint16_t *p = a.xpan + a.xoff[pm] * (NC / 16) + (int64_t)kc * PX;
    const double *col = (const double *)(sv + mi * a.kst);
#pragma unroll 1
    for (int ri = 0; ri < 2; ++ri) {  // real part (column c0), then imaginary part (c0 + 1)
      uint32_t pk[kS][4];
      if (live) {
        const int e = gex[mi][ri];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          uint32_t d[kS];
          split_digits_fp32<kS>(col[2 * sv_idx(kc * kPK + h * 8 + q) + ri], e, d);  // dfconv.h
#pragma unroll
          for (int j = 0; j < kS; ++j) {
            if (q & 1)
              pk[j][q >> 1] |= d[j] << 16;
            else
              pk[j][q >> 1] = d[j];
          }
        }
      } else {
#pragma unroll
        for (int j = 0; j < kS; ++j)
#pragma unroll
          for (int q = 0; q < 4; ++q) pk[j][q] = 0u;
      }
#pragma unroll
      for (int j = 0; j < kS; ++j)
        *(uint4 *)(p + swz(j * NC + c0 + ri, h * 8)) = make_uint4(pk[j][0], pk[j][1], pk[j][2], pk[j][3]);
    }
  }
}

// ---------------------------------------------------------------------------
// tcgen05 / mbarrier / bulk-copy primitives
// ---------------------------------------------------------------------------

__device__ __forceinline__ uint32_t saddr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void bar_init(uint64_t *b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(saddr(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void bar_arrive(uint64_t *b) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(saddr(b))
               : "memory");
}
__device__ __forceinline__ void bar_expect_tx(uint64_t *b, uint32_t bytes) {
  asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                   saddr(b)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool bar_try(uint64_t *b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, "
      "p;\n\t}"
      : "=r"(ok)
      : "r"(saddr(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait that ignores the abort flag (draining before TMEM release).
__device__ __noinline__ bool bar_wait_timed(uint64_t *b, uint32_t parity) {
  const long long t0 = clock64();
  while (!bar_try(b, parity))
    if (clock64() - t0 > kWaitCycles) return false;
  return true;
}
// Bounded wait; false when the CTA is aborting or the wait expired (then it
// raises the CTA abort flag and the global error flag).
__device__ __noinline__ bool bar_wait(uint64_t *b, uint32_t parity, volatile int *abort_flag, int *err) {
  const long long t0 = clock64();
  for (uint32_t it = 0;; ++it) {
    if (bar_try(b, parity)) return true;
    if ((it & 255u) == 255u) {
      if (*abort_flag) return false;
      if (clock64() - t0 > kWaitCycles) {
        *abort_flag = 1;
        atomicExch(err, 1);
        return false;
      }
    }
  }
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   saddr(dst)),
               "l"(src), "r"(bytes), "r"(saddr(bar))
               : "memory");
}
__device__ __forceinline__ uint64_t sw128_desc(const void *p) {
  const uint32_t a = saddr(p);
  uint64_t d = 0;
  d |= (uint64_t)((a >> 4) & 0x3FFFu);  // start address
  d |= (uint64_t)1 << 16;               // leading byte offset (unused with 128B swizzle)
  d |= (uint64_t)(1024 >> 4) << 32;     // stride byte offset: 8-row groups 1024 B apart
  d |= (uint64_t)1 << 46;               // descriptor version
  d |= (uint64_t)2 << 61;               // 128-byte swizzle
  return d;
}
__device__ __forceinline__ uint32_t idesc_bf16(int M, int N) {
  return (1u << 4)                    // D: f32
         | (1u << 7) | (1u << 10)     // A, B: bf16
         | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);  // K-major A and B
}
__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, "
      "p;\n\t}" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(saddr(bar))
               : "memory");
}
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}


// ---------------------------------------------------------------------------
// the contraction
// ---------------------------------------------------------------------------

struct MxArgs {
  int q;  // 0: l -> t with D, 1: t -> l with Q
  const uint16_t *panels;
  const int64_t *pan_off;
  const int8_t *eA;
  const int64_t *e_off;
  int bl, nt, an, tmlo, n, mlo, lmin;  // lmin: smallest over the parts
  const uint16_t *xpan;
  const int64_t *xoff;
  const int *eX;
  const int2 *tiles;
  int ntiles;
  int nparts;
  Part part[kMaxParts];
  int nb, mpp;
  // map groups of one launch: group g holds maps [b0 + g mpp, b0 + (g + 1) mpp)
  // of every part, its coefficient panels at xpan + g xg and exponents at
  // eX + g eXg.  Work item v is tile v / ngroups of group v % ngroups, so that
  // neighbouring CTAs run the same table tile for different groups and the
  // second read of the tile's panels is served by L2.
  int b0, ngroups, eXg;
  int64_t xg;
  int *err;
};

struct TileInfo {
  int pm, m, mi, rt, kc0, nkc, l0;
  int g;  // map group
  double sign;
};
__device__ __forceinline__ TileInfo tile_info(const MxArgs &a, int v) {
  TileInfo ti;
  ti.g = v % a.ngroups;
  const int2 tl = a.tiles[v / a.ngroups];
  ti.pm = tl.x;
  ti.rt = tl.y;
  ti.m = a.mlo + ti.pm;
  const TableRefM r = table_ref_m(a.tmlo, a.n, ti.m);
  ti.mi = r.mi;
  ti.sign = r.sign;
  const Geom g = geom(a.bl, a.nt, a.an, ti.m, a.q != 0);
  ti.l0 = g.l0;
  ti.nkc = g.nkc;
  const int lst = g.l0 > a.lmin ? g.l0 : a.lmin;
  ti.kc0 = 0;
  if (!a.q) ti.kc0 = lst >= a.bl ? g.nkc : (lst - g.l0) / kPK;
  return ti;
}

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float *v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}
// the 7 class accumulators of 8 columns into registers (waits for the loads)
__device__ __forceinline__ void load_classes8(uint32_t taddr, int ncols_per_class, float (*acc)[8]) {
#pragma unroll
  for (int c = 0; c < kS; ++c) tmem_ld8(taddr + (uint32_t)(c * ncols_per_class), acc[c]);
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
// Combine the 7 class accumulators of 8 columns for this thread's row:
// S = sum_c acc_c 2^(-7c) by Horner in double-float on the FP32 pipe (the class
// values and 2^-7 scalings are exact floats), then one widening to FP64 with
// the power of two 2^(ea + eX - 12) applied while widening (dfconv.h).
__device__ __forceinline__ int ex_at(int4 e0, int4 e1, int col) {
  const int4 e = col < 4 ? e0 : e1;
  const int c = col & 3;
  return c == 0 ? e.x : (c == 1 ? e.y : (c == 2 ? e.z : e.w));
}
// eX of the 8 columns in e0 (columns 0-3) and e1 (4-7)
__device__ __forceinline__ void combine8(float (*acc)[8], int ea, int4 e0, int4 e1, double sign, double *y) {
#pragma unroll
  for (int col = 0; col < 8; ++col) {
    float hi = acc[kS - 1][col], lo = 0.0f;
#pragma unroll
    for (int c = kS - 2; c >= 0; --c) {
      hi = __fmul_rn(hi, 0.0078125f);
      lo = __fmul_rn(lo, 0.0078125f);
      const float s = __fadd_rn(acc[c][col], hi);
      const float v = __fsub_rn(s, acc[c][col]);
      float e = __fadd_rn(__fsub_rn(acc[c][col], __fsub_rn(s, v)), __fsub_rn(hi, v));
      e = __fadd_rn(e, lo);
      hi = __fadd_rn(s, e);
      lo = __fsub_rn(e, __fsub_rn(hi, s));
    }
    if (sign < 0.0) {
      hi = -hi;
      lo = -lo;
    }
    y[col] = join_scaled(hi, lo, ea + ex_at(e0, e1, col) - 2 * kB0);
  }
}

template <int NC>
__global__ void __launch_bounds__(kThreads, 1) k_contract_mx(MxArgs a) {
  constexpr int PX = Cfg<NC>::kPanelX;
  constexpr int ACC = Cfg<NC>::kAccCols;
  constexpr int TMC = Cfg<NC>::kTmemCols;
  constexpr int kAST = Cfg<NC>::kAST;
  constexpr int NBUF = Cfg<NC>::kNBuf;
  constexpr int kNumBars = Cfg<NC>::kNumBars;
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint16_t *sA = (uint16_t *)smem;
  uint16_t *sX = (uint16_t *)(smem + Cfg<NC>::kSmemA);
  uint64_t *bars = (uint64_t *)(smem + Cfg<NC>::kSmemA + Cfg<NC>::kSmemX);
  uint64_t *fullA = bars, *emptyA = bars + kAST, *fullX = bars + 2 * kAST, *emptyX = bars + 2 * kAST + kXST;
  uint64_t *tfull = bars + 2 * kAST + 2 * kXST, *tempty = tfull + 2, *mma_done = tfull + 4;
  volatile int *abort_flag = (volatile int *)(bars + kNumBars);
  uint32_t *tmem_slot = (uint32_t *)(bars + kNumBars) + 1;
  int *cons = (int *)(bars + kNumBars) + 2;  // [2]: table / coefficient stages consumed

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int i = 0; i < kAST; ++i) {
      bar_init(&fullA[i], 1);
      bar_init(&emptyA[i], 1);
    }
    for (int i = 0; i < kXST; ++i) {
      bar_init(&fullX[i], 1);
      bar_init(&emptyX[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      bar_init(&tfull[i], 1);
      bar_init(&tempty[i], 32 * kEpiWarps);
    }
    bar_init(mma_done, 1);
    *abort_flag = 0;
    cons[0] = cons[1] = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(saddr(tmem_slot)),
                 "r"(TMC)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;

  int issuedA = 0, issuedX = 0;
  if (warp == 0 && lane == 0) {
    // ---------------- producer ----------------
    bool ok = true;
    for (int t = blockIdx.x; ok && t < a.ntiles * a.ngroups; t += gridDim.x) {
      const TileInfo ti = tile_info(a, t);
      const uint16_t *pan = a.panels + a.pan_off[ti.mi] + (int64_t)ti.rt * ti.nkc * kS * kPanelA;
      const uint16_t *xp = a.xpan + ti.g * a.xg + a.xoff[ti.pm] * (NC / 16);
      for (int kc = ti.kc0; ok && kc < ti.nkc; ++kc) {
        const int xs = issuedX % kXST;
        if (!(ok = bar_wait(&emptyX[xs], ((issuedX / kXST) & 1) ^ 1, abort_flag, a.err))) break;
        bar_expect_tx(&fullX[xs], PX * 2);
        bulk_g2s(sX + (size_t)xs * PX, xp + (int64_t)kc * PX, PX * 2, &fullX[xs]);
        ++issuedX;
        for (int j = 0; j < kS; ++j) {
          const int as = issuedA % kAST;
          if (!(ok = bar_wait(&emptyA[as], ((issuedA / kAST) & 1) ^ 1, abort_flag, a.err))) break;
          bar_expect_tx(&fullA[as], kPanelA * 2);
          bulk_g2s(sA + (size_t)as * kPanelA, pan + ((int64_t)kc * kS + j) * kPanelA, kPanelA * 2, &fullA[as]);
          ++issuedA;
        }
      }
    }
  } else if (warp == 1 && lane == 0) {
    // ---------------- MMA issuer ----------------
    int ca = 0, cx = 0, ti_n = 0;
    bool ok = true, any = false;
    for (int t = blockIdx.x; ok && t < a.ntiles * a.ngroups; t += gridDim.x, ++ti_n) {
      const TileInfo ti = tile_info(a, t);
      const int ab = ti_n % NBUF;
      if (!(ok = bar_wait(&tempty[ab], ((ti_n / NBUF) & 1) ^ 1, abort_flag, a.err))) break;
      tc_fence_after();
      const uint32_t d0 = tmem + (uint32_t)(ab * ACC);
      if (ti.kc0 >= ti.nkc) {
        bar_arrive(&tfull[ab]);  // nothing to accumulate: the epilogue writes zeros
        continue;
      }
      for (int kc = ti.kc0; ok && kc < ti.nkc; ++kc) {
        const int xs = cx % kXST;
        if (!(ok = bar_wait(&fullX[xs], (cx / kXST) & 1, abort_flag, a.err))) break;
        tc_fence_after();
        const uint64_t bdesc = sw128_desc(sX + (size_t)xs * PX);
        for (int j = 0; j < kS; ++j) {
          const int as = ca % kAST;
          if (!(ok = bar_wait(&fullA[as], (ca / kAST) & 1, abort_flag, a.err))) break;
          tc_fence_after();
          const uint64_t adesc = sw128_desc(sA + (size_t)as * kPanelA);
          // B rows [0, NC (7 - j)) -> accumulator columns NC j + row, in MMAs of N <= 256
          const int ntot = NC * (kS - j);
          for (int off = 0; off < ntot; off += 256) {
            const int n = ntot - off < 256 ? ntot - off : 256;
            const uint32_t idesc = idesc_bf16(kPM, n);
            // 8-row atoms of 128 B: a row offset of `off` moves the start by off * 128 B
            const uint64_t bd = bdesc + (uint64_t)(off * 8);
#pragma unroll
            for (int k = 0; k < kPK / 16; ++k) {
              // K advance of 16 bf16 = 32 bytes inside the swizzle atom
              mma_bf16(d0 + (uint32_t)(NC * j + off), adesc + (uint64_t)(2 * k), bd + (uint64_t)(2 * k), idesc,
                       (kc == ti.kc0 && j == 0 && k == 0) ? 0u : 1u);
            }
          }
          any = true;
          mma_commit(&emptyA[as]);
          ++ca;
        }
        if (!ok) break;
        mma_commit(&emptyX[xs]);
        ++cx;
      }
      if (!ok) break;
      mma_commit(&tfull[ab]);
    }
    cons[0] = ca;
    cons[1] = cx;
    if (any) {  // every MMA of this thread has completed before TMEM is released
      mma_commit(mma_done);
      if (!bar_wait_timed(mma_done, 0)) atomicExch(a.err, 2);
    }
  } else if (warp >= 2) {
    // ---------------- epilogue ----------------
    // warp -> TMEM lane quarter (warp mod 4, the quarter it may address) and one
    // 16-column chunk pi, read as two 8-column halves; the accumulator is
    // handed back right after the second half is in registers, before it is
    // combined and stored, so that the next tile's MMAs wait as little as possible
    const int quarter = warp & 3;
    const int pi = (warp - 2) / 4;
    const int rr = quarter * 32 + lane;
    int ti_n = 0;
    for (int t = blockIdx.x; t < a.ntiles * a.ngroups; t += gridDim.x, ++ti_n) {
      const TileInfo ti = tile_info(a, t);
      const int ab = ti_n % NBUF;
      const bool live = ti.kc0 < ti.nkc;
      // the row and column exponents do not depend on the accumulator: read
      // them before waiting, so that their latency is not spent holding TMEM
      int ea = 0;
      int4 ex4[4];
      if (pi < NC / 16 && live) {
        ea = (int)a.eA[a.e_off[ti.mi] + ti.rt * kPM + rr];
        const int4 *ep = (const int4 *)(a.eX + ti.g * a.eXg + ti.pm * NC + pi * 16);
#pragma unroll
        for (int q = 0; q < 4; ++q) ex4[q] = ep[q];
      }
      // warp-uniform outcome: tcgen05.ld below is .sync.aligned
      if (!__all_sync(0xffffffffu, bar_wait(&tfull[ab], (ti_n / NBUF) & 1, abort_flag, a.err))) break;
      tc_fence_after();
      if (pi >= NC / 16 || !live) {  // no columns here, or nothing accumulated: release at once
        tc_fence_before();
        bar_arrive(&tempty[ab]);
        if (pi >= NC / 16) continue;
      }
      const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(ab * ACC);
      const int t_row = ti.rt * kPM + rr;
      const int l = ti.l0 + ti.rt * kPM + rr;
#pragma unroll 1
      for (int hh = 0; hh < 2; ++hh) {
        const int c0 = pi * 16 + hh * 8;  // first column of this half
        double y[8];
        if (live) {
          float acc[kS][8];
          load_classes8(taddr + (uint32_t)c0, NC, acc);
          if (hh == 1) {  // every column of this warp is in registers: hand the accumulator back
            tc_fence_before();
            bar_arrive(&tempty[ab]);
          }
          combine8(acc, ea, hh ? ex4[2] : ex4[0], hh ? ex4[3] : ex4[1], ti.sign, y);
        } else {
#pragma unroll
          for (int col = 0; col < 8; ++col) y[col] = 0.0;
        }
        // column pair cp = c0 / 2 + bb: part cp / mpp, map b0 + cp % mpp
#pragma unroll
        for (int bb = 0; bb < 4; ++bb) {
          const int cp = c0 / 2 + bb;
          const int part = cp / a.mpp;
          const int b = a.b0 + ti.g * a.mpp + cp % a.mpp;
          if (part >= a.nparts || b >= a.nb) continue;
          const Part &P = a.part[part];
          if (!a.q) {
            if (t_row < a.nt)
              P.dst[(int64_t)b * P.ds + (int64_t)t_row * P.dw + (ti.m - P.d_mlo)] =
                  make_double2(y[2 * bb], y[2 * bb + 1]);
          } else {
            const int lst = ti.l0 > P.lmin ? ti.l0 : P.lmin;
            if (l >= lst && l < a.bl) {
              const double yr = y[2 * bb], yi = y[2 * bb + 1];
              P.dst[(int64_t)b * P.ds + (int64_t)l * l + l + ti.m] = weighted(P, make_double2(yr, yi), l);
            }
          }
        }
      }
    }
  }

  // producer: on abort, wait (bounded) for its own copies still in flight
  __syncthreads();
  if (warp == 0 && lane == 0 && *abort_flag) {
    const long long t0 = clock64();
    for (int i = cons[0]; i < issuedA; ++i)
      while (!bar_try(&fullA[i % kAST], (i / kAST) & 1) && clock64() - t0 < kWaitCycles) {
      }
    for (int i = cons[1]; i < issuedX; ++i)
      while (!bar_try(&fullX[i % kXST], (i / kXST) & 1) && clock64() - t0 < kWaitCycles) {
      }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 1)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMC) : "memory");
}

// ---------------------------------------------------------------------------
// host side: sliced-table cache, tile lists, launches
// ---------------------------------------------------------------------------

struct TileList {
  int2 *d_tiles = nullptr;
  int ntiles = 0;
  int64_t *d_xoff = nullptr;
  int64_t x_elems = 0;
  int64_t work_entries = 0;  // table entries streamed per launch (all tiles)
};

struct SlicedTable {
  int bl = 0, nt = 0, an = 0, mlo = 0, nm = 0;
  bool q = false;
  uint16_t *panels = nullptr;
  int8_t *eA = nullptr;
  int64_t *d_pan_off = nullptr, *d_e_off = nullptr;
  size_t bytes = 0;
  std::map<std::tuple<int, int, int, int>, TileList> lists;  // (n, mlo, mhi, lmin)
};

std::mutex g_mx_mu;
std::map<std::tuple<int, int, int, int>, std::unique_ptr<SlicedTable>> g_sliced;  // (bl, an, ss, q)
size_t g_mx_bytes = 0;
int *g_err = nullptr;

template <class T>
T *dev_alloc(size_t n, size_t *acc) {
  void *p = nullptr;
  S2G_CUDA(cudaMalloc(&p, sizeof(T) * (n ? n : 1)));
  *acc += sizeof(T) * (n ? n : 1);
  return (T *)p;
}

SlicedTable &sliced(const WignerTable &tb, bool q, cudaStream_t st) {
  auto key = std::make_tuple(tb.bl, tb.an, tb.ss, q ? 1 : 0);
  auto it = g_sliced.find(key);
  if (it != g_sliced.end()) return *it->second;
  auto s = std::make_unique<SlicedTable>();
  s->bl = tb.bl;
  s->nt = tb.nt;
  s->an = tb.an;
  s->mlo = tb.mlo;
  s->nm = tb.nm;
  s->q = q;
  std::vector<int64_t> po(tb.nm), eo(tb.nm);
  int64_t ptot = 0, etot = 0;
  for (int mi = 0; mi < tb.nm; ++mi) {
    const Geom g = geom(tb.bl, tb.nt, tb.an, tb.mlo + mi, q);
    po[mi] = ptot;
    eo[mi] = etot;
    ptot += (int64_t)g.nrt * g.nkc * kS * kPanelA;
    etot += (int64_t)g.nrt * kPM;
  }
  size_t by = 0;
  s->panels = dev_alloc<uint16_t>((size_t)ptot, &by);
  s->eA = dev_alloc<int8_t>((size_t)etot, &by);
  s->d_pan_off = dev_alloc<int64_t>(tb.nm, &by);
  s->d_e_off = dev_alloc<int64_t>(tb.nm, &by);
  S2G_CUDA(cudaMemcpyAsync(s->d_pan_off, po.data(), sizeof(int64_t) * tb.nm, cudaMemcpyHostToDevice, st));
  S2G_CUDA(cudaMemcpyAsync(s->d_e_off, eo.data(), sizeof(int64_t) * tb.nm, cudaMemcpyHostToDevice, st));
  int nrt_max = (std::max(tb.bl, tb.nt) + kPM - 1) / kPM;
  dim3 grid(tb.nm, nrt_max);
  k_slice_table<<<grid, 128, 0, st>>>(q ? tb.Q : tb.D, tb.d_off, tb.bl, tb.nt, tb.an, tb.mlo, q ? 1 : 0,
                                      s->panels, s->d_pan_off, s->eA, s->d_e_off);
  S2G_LAUNCHED();
  S2G_CUDA(cudaStreamSynchronize(st));
  s->bytes = by;
  g_mx_bytes += by;
  SlicedTable &ref = *s;
  g_sliced.emplace(key, std::move(s));
  return ref;
}

const TileList &tile_list(SlicedTable &s, int n, int mlo, int mhi, int lmin, cudaStream_t st) {
  auto key = std::make_tuple(n, mlo, mhi, lmin);
  auto it = s.lists.find(key);
  if (it != s.lists.end()) return it->second;
  TileList L;
  std::vector<int2> tiles;
  std::vector<int64_t> xoff(mhi - mlo + 1);
  int64_t xe = 0, work = 0;
  for (int m = mlo; m <= mhi; ++m) {
    const Geom g = geom(s.bl, s.nt, s.an, m, s.q);
    xoff[m - mlo] = xe;
    xe += (int64_t)g.nkc * Cfg<16>::kPanelX;
    if (g.nl <= 0) continue;
    const int lst = g.l0 > lmin ? g.l0 : lmin;
    int rt0 = 0, kc0 = 0;
    if (s.q) {
      if (lst >= s.bl) continue;
      rt0 = (lst - g.l0) / kPM;
    } else {
      kc0 = lst >= s.bl ? g.nkc : (lst - g.l0) / kPK;
    }
    for (int rt = rt0; rt < g.nrt; ++rt) {
      tiles.push_back(make_int2(m - mlo, rt));
      work += (int64_t)(g.nkc - kc0) * kPK * kPM;
    }
  }
  size_t by = 0;
  L.ntiles = (int)tiles.size();
  L.d_tiles = dev_alloc<int2>(tiles.size(), &by);
  L.d_xoff = dev_alloc<int64_t>(xoff.size(), &by);
  L.x_elems = xe;
  L.work_entries = work;
  if (!tiles.empty())
    S2G_CUDA(cudaMemcpyAsync(L.d_tiles, tiles.data(), sizeof(int2) * tiles.size(), cudaMemcpyHostToDevice, st));
  S2G_CUDA(cudaMemcpyAsync(L.d_xoff, xoff.data(), sizeof(int64_t) * xoff.size(), cudaMemcpyHostToDevice, st));
  S2G_CUDA(cudaStreamSynchronize(st));
  g_mx_bytes += by;
  s.bytes += by;
  return s.lists.emplace(key, L).first->second;
}

int num_sms() {
  static const int n = [] {
    int dev = 0, v = 0;
    S2G_CUDA(cudaGetDevice(&dev));
    S2G_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev));
    return v;
  }();
  return n;
}

int *error_flag() {
  if (!g_err) {
    S2G_CUDA(cudaMalloc(&g_err, sizeof(int)));
    S2G_CUDA(cudaMemset(g_err, 0, sizeof(int)));
  }
  return g_err;
}

struct Problem {
  bool q;
  const WignerTable *tb;
  int n, mlo, mhi;
  int nparts;
  Part part[kMaxParts];
  int nb;
};

template <int NC>
void run_mixed(const Problem &p, cudaStream_t st, int gpl_max) {
  static const bool attr = [] {  // once per instantiation (thread-safe static initialisation)
    S2G_CUDA(cudaFuncSetAttribute(k_contract_mx<NC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)Cfg<NC>::kSmemBytes));
    return true;
  }();
  (void)attr;
  int lmin = p.part[0].lmin;
  for (int i = 1; i < p.nparts; ++i) lmin = std::min(lmin, p.part[i].lmin);
  SlicedTable *s;
  const TileList *L;
  int *err;
  {
    std::lock_guard<std::mutex> lk(g_mx_mu);
    s = &sliced(*p.tb, p.q, st);
    L = &tile_list(*s, p.n, p.mlo, p.mhi, lmin, st);
    err = error_flag();
  }
  const int nmp = p.mhi - p.mlo + 1;
  const int mpp = NC / (2 * p.nparts);  // maps per part per launch
  int nkcmax = 0;
  for (int pm = 0; pm < nmp; ++pm) nkcmax = std::max(nkcmax, geom(p.tb->bl, p.tb->nt, p.tb->an, p.mlo + pm, p.q).nkc);
  const size_t slice_smem = sizeof(double2) * kMG * (size_t)sv_idx(nkcmax * kPK);
  constexpr int kSliceSmemMax = 232448 - 1024;  // the opt-in maximum less the static arrays
  S2G_REQUIRE(slice_smem <= (size_t)kSliceSmemMax, ERR_INVALID,
              "coefficient slicing: K too large for shared-memory staging");
  static const bool attr_x = [] {
    S2G_CUDA(cudaFuncSetAttribute(k_slice_x<NC>, cudaFuncAttributeMaxDynamicSharedMemorySize, kSliceSmemMax));
    return true;
  }();
  (void)attr_x;
  const int ngroups = (p.nb + mpp - 1) / mpp;
  // map groups run up to gpl_max at a time in one launch (their tiles
  // interleaved, the table read once from HBM and again from L2)
  const int gpl = ngroups < gpl_max ? ngroups : gpl_max;
  // coefficient panels: the tile list's offsets count 16-column panels; an
  // NC-column panel is NC/16 times larger, so offsets scale by NC/16
  const int64_t x_elems = L->x_elems * (NC / 16);
  uint16_t *xpan = nullptr;
  int *eX = nullptr;
  const int64_t *xoff = L->d_xoff;
  S2G_CUDA(cudaMallocAsync((void **)&xpan, sizeof(uint16_t) * (size_t)(x_elems ? x_elems * gpl : 1), st));
  S2G_CUDA(cudaMallocAsync((void **)&eX, sizeof(int) * (size_t)nmp * NC * gpl, st));
  const double entries = (double)L->work_entries;
  for (int g0 = 0; g0 < ngroups; g0 += gpl) {
    const int ng = ngroups - g0 < gpl ? ngroups - g0 : gpl;
    double fl = 0, by = 0;
    for (int g = g0; g < g0 + ng; ++g) {
      const int b0 = g * mpp;
      const int nbg = p.nb - b0 < mpp ? p.nb - b0 : mpp;
      double xby = 0;
      if (timing_enabled()) {
        fl += 4.0 * entries * nbg * p.nparts;
        by += entries * 2.0 * kS + (double)x_elems * 2.0 + 16.0 * nbg * p.nparts * (double)p.tb->nt * nmp;
        xby = (double)x_elems * 2.0 * (1.0 + 8.0 / (2.0 * kS));  // panels written + FP64 values read
      }
      XArgs xa{};
      xa.q = p.q ? 1 : 0;
      xa.bl = p.tb->bl;
      xa.nt = p.tb->nt;
      xa.an = p.tb->an;
      xa.mlo = p.mlo;
      xa.lmin = lmin;
      xa.nparts = p.nparts;
      for (int i = 0; i < p.nparts; ++i) xa.part[i] = p.part[i];
      xa.nb = p.nb;
      xa.b0 = b0;
      xa.mpp = mpp;
      xa.xoff = xoff;
      xa.xpan = xpan + (int64_t)(g - g0) * x_elems;
      xa.eX = eX + (int64_t)(g - g0) * nmp * NC;
      xa.nmp = nmp;
      xa.nkcmax = nkcmax;
      xa.kst = sv_idx(nkcmax * kPK);
      KTimer kx(KC_SLICE, st, 0.0, xby);
      k_slice_x<NC><<<dim3((nmp + kMG - 1) / kMG, NC / 2), kSliceThreads, slice_smem, st>>>(xa);
      S2G_LAUNCHED();
    }
    if (L->ntiles == 0) continue;
    KTimer kt(KC_MIXED, st, fl, by);
    MxArgs ma{};
    ma.q = p.q ? 1 : 0;
    ma.panels = s->panels;
    ma.pan_off = s->d_pan_off;
    ma.eA = s->eA;
    ma.e_off = s->d_e_off;
    ma.bl = p.tb->bl;
    ma.nt = p.tb->nt;
    ma.an = p.tb->an;
    ma.tmlo = p.tb->mlo;
    ma.n = p.n;
    ma.mlo = p.mlo;
    ma.lmin = lmin;
    ma.xpan = xpan;
    ma.xoff = xoff;
    ma.eX = eX;
    ma.tiles = L->d_tiles;
    ma.ntiles = L->ntiles;
    ma.nparts = p.nparts;
    for (int i = 0; i < p.nparts; ++i) ma.part[i] = p.part[i];
    ma.nb = p.nb;
    ma.mpp = mpp;
    ma.b0 = g0 * mpp;
    ma.ngroups = ng;
    ma.xg = x_elems;
    ma.eXg = nmp * NC;
    ma.err = err;
    const int nwork = L->ntiles * ng;
    const int grid = nwork < num_sms() ? nwork : num_sms();
    k_contract_mx<NC><<<grid, kThreads, Cfg<NC>::kSmemBytes, st>>>(ma);
    S2G_LAUNCHED();
  }
  cudaFreeAsync(xpan, st);
  cudaFreeAsync(eX, st);
}

// Columns per table pass (2 (re, im) x maps x parts) and map groups per launch.
// Built-in: the smallest of 16 / 32 / 64 columns that holds the whole batch
// (larger batches loop over map groups), 4 groups per launch.  With tuning
// on, the candidates below are timed per (band-limit bucket, column bucket,
// direction) and the fastest kept.
void run_problem(const Problem &p, cudaStream_t st) {
  struct Shape {
    int nc, gpl;
  };
  static const Shape kCand[7] = {{16, 1}, {16, 4}, {32, 1}, {32, 4}, {64, 1}, {64, 2}, {64, 4}};
  const int cols = 2 * p.nb * p.nparts;
  const int def = cols <= 16 ? 1 : (cols <= 32 ? 3 : 6);
  // a candidate narrower than one part's two columns cannot hold a map
  const int first = 2 * p.nparts > 16 ? (2 * p.nparts > 32 ? 4 : 2) : 0;
  const auto run = [&](const Shape &sh) {
    if (sh.nc == 16)
      run_mixed<16>(p, st, sh.gpl);
    else if (sh.nc == 32)
      run_mixed<32>(p, st, sh.gpl);
    else
      run_mixed<64>(p, st, sh.gpl);
  };
  const int c = tuned(TF_MIXED, tune_bucket(p.tb->bl), tune_bucket(cols), p.q ? 1 : 0, 7 - first, def - first, st,
                      [&](int i) { run(kCand[first + i]); });
  run(kCand[first + c]);
}

Part part_of(const L2T &a) {
  Part P{};
  P.src = a.x;
  P.ss = a.xs;
  P.x_half = a.x_half ? 1 : 0;
  P.w = a.w;
  P.wscale = a.wscale;
  P.wconj = a.wconj ? 1 : 0;
  P.wkind = a.wkind;
  P.lmin = a.lmin;
  P.dst = a.out;
  P.ds = a.os;
  P.dw = a.ow;
  P.d_mlo = a.omlo;
  return P;
}

Part part_of(const T2L &a) {
  Part P{};
  P.src = a.in;
  P.ss = a.is;
  P.sw = a.iw;
  P.s_mlo = a.imlo;
  P.w = a.w;
  P.wscale = a.wscale;
  P.wconj = a.wconj ? 1 : 0;
  P.wkind = a.wkind;
  P.lmin = a.lmin;
  P.dst = a.y;
  P.ds = a.ys;
  return P;
}

template <class A>
bool same_problem(const A &x, const A &y) {
  return x.tb == y.tb && x.n == y.n && x.use_q == y.use_q && x.mlo == y.mlo && x.mhi == y.mhi && x.nb == y.nb;
}

}  // namespace

bool contract_l2t_mixed(const L2T *a, int nparts, cudaStream_t st) {
  if (nparts < 1 || nparts > kMaxParts) return false;
  if (a[0].use_q || a[0].tb->bl < kMinBl || a[0].nb <= 0 || a[0].mhi < a[0].mlo) return false;
  for (int i = 1; i < nparts; ++i)
    if (!same_problem(a[0], a[i])) return false;
  Problem p{};
  p.q = false;
  p.tb = a[0].tb;
  p.n = a[0].n;
  p.mlo = a[0].mlo;
  p.mhi = a[0].mhi;
  p.nb = a[0].nb;
  p.nparts = nparts;
  for (int i = 0; i < nparts; ++i) p.part[i] = part_of(a[i]);
  run_problem(p, st);
  return true;
}

bool contract_t2l_mixed(const T2L *a, int nparts, cudaStream_t st) {
  if (nparts < 1 || nparts > kMaxParts) return false;
  if (!a[0].use_q || a[0].tb->bl < kMinBl || a[0].nb <= 0 || a[0].mhi < a[0].mlo) return false;
  for (int i = 1; i < nparts; ++i)
    if (!same_problem(a[0], a[i])) return false;
  Problem p{};
  p.q = true;
  p.tb = a[0].tb;
  p.n = a[0].n;
  p.mlo = a[0].mlo;
  p.mhi = a[0].mhi;
  p.nb = a[0].nb;
  p.nparts = nparts;
  for (int i = 0; i < nparts; ++i) p.part[i] = part_of(a[i]);
  run_problem(p, st);
  return true;
}

void release_sliced_tables() {
  std::lock_guard<std::mutex> lk(g_mx_mu);
  for (auto &kv : g_sliced) {
    SlicedTable &s = *kv.second;
    cudaFree(s.panels);
    cudaFree(s.eA);
    cudaFree(s.d_pan_off);
    cudaFree(s.d_e_off);
    for (auto &l : s.lists) {
      cudaFree(l.second.d_tiles);
      cudaFree(l.second.d_xoff);
    }
  }
  g_sliced.clear();
  g_mx_bytes = 0;
}

size_t sliced_table_bytes() {
  std::lock_guard<std::mutex> lk(g_mx_mu);
  return g_mx_bytes;
}

int mixed_error_flag_read_and_clear() {
  std::lock_guard<std::mutex> lk(g_mx_mu);
  if (!g_err) return 0;
  int v = 0;
  S2G_CUDA(cudaMemcpy(&v, g_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (v) S2G_CUDA(cudaMemset(g_err, 0, sizeof(int)));
  return v;
}

}  // namespace s2g
