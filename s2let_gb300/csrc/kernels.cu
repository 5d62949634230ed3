// Transform kernels, FP64 path.
//
//  k_ring      batched Bluestein DFT of rings (length 2bl-1 on MW, 2bl on MWSS
//              sampling) in shared memory: chirp premultiply, radix-2 DIT FFT of the padded length,
//              pointwise multiply by the chirp-kernel spectrum, DIF inverse FFT,
//              chirp postmultiply.  Two real rings share one complex FFT.
//  k_contract  per-m Legendre/Wigner contraction against the cached d-tables,
//              tiled through shared memory (table tiles loaded coalesced along
//              their contiguous axis, coefficient tiles broadcast).
//  k_gamma_*   DFT over the 2N-1 gamma samples of the rotation group.
//  k_merge     harmonic tiling merge (lmn -> lm) fused over scales/directions.
#include <cooperative_groups.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <map>
#include <mutex>
#include <type_traits>

#include "autotune.h"
#include "common.h"
#include "dfarith.h"
#include "dfconv.h"
#include <cstdlib>

#include "kernels.h"
#include "mixed.h"
#include "recompute.h"
#include "timing.h"

namespace s2g {

namespace {

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cmulc(double2 a, double2 b) {  // a * conj(b)
  return make_double2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
__device__ __forceinline__ double2 conj2(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 add2(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 sub2(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 scl2(double2 a, double s) { return make_double2(a.x * s, a.y * s); }
__device__ __forceinline__ int brev(int k, int logP) {
  return logP == 0 ? 0 : (int)(__brev((unsigned)k) >> (32 - logP));
}

// ---------------------------------------------------------------------------
// Ring DFT (Bluestein)
// ---------------------------------------------------------------------------

struct RingArgs {
  const void *rings;
  double2 *rings_out;  // inverse: output rings (as double2 or double)
  int64_t ring_stride;  // between rings of one map
  int64_t map_stride;   // between maps
  int rpm;              // rings per map
  const double2 *spec_in;
  double2 *spec_out;
  int64_t spec_stride;      // between spectra of one map
  int64_t spec_map_stride;  // between maps (spectra of ring r at spec_base(r))
  int spec_rpm;             // spectra per map
  int herm;                 // complex inverse: m < 0 taken as conj of m > 0 (real-valued ring)
  int sw, mlo;
  int nrings, bl, K, P, logP;
  const double2 *chirp, *bhat, *tw;
  const float4 *chirp_df, *bhat_df, *tw_df;
};

namespace cg = cooperative_groups;

// One launch of ring DFTs fused with the gamma DFT (k_ring_inverse_gamma_df,
// k_gamma_ring_forward_df): NN <= kFuseMaxNN n-components per ring.
constexpr int kFuseMaxNN = 8;
constexpr int kFuseMaxTw = 128;
struct GammaFuse {
  const double2 *G;  // synthesis input: spectrum of component k of ring (b, t) at G + b gms + k gks + t W
  double2 *Gout;     // analysis output, the same addressing (all m from -(bl-1))
  int64_t gms, gks;
  int W, nt;
  int herm_k;  // real signals: the component with n = 0 (m >= 0 stored, at offset bl-1), else -1
  void *fw;    // gamma slice g of ring (b, t) at fw + b fms + g npx + t K (double, or double2 unless real)
  int64_t fms, npx;
  int ng, real;
  float4 tw[kFuseMaxTw];  // [g NN + k] double-float twiddles with their normalisation
};

// element offset of ring r (rings of a map are ring_stride apart, maps map_stride)
__device__ __forceinline__ int64_t ring_base(const RingArgs &a, int r) {
  return (int64_t)(r / a.rpm) * a.map_stride + (int64_t)(r % a.rpm) * a.ring_stride;
}
__device__ __forceinline__ int64_t spec_base(const RingArgs &a, int r) {
  return (int64_t)(r / a.spec_rpm) * a.spec_map_stride + (int64_t)(r % a.spec_rpm) * a.spec_stride;
}

// In-place transforms on the shared buffer.
__device__ void fft_dit(double2 *buf, const double2 *__restrict__ tw, int P, int logP) {
  for (int s = 1; s <= logP; ++s) {
    const int half = 1 << (s - 1);
    for (int i = threadIdx.x; i < P / 2; i += blockDim.x) {
      const int j = i & (half - 1);
      const int i0 = ((i >> (s - 1)) << s) + j, i1 = i0 + half;
      const double2 w = __ldg(&tw[j << (logP - s)]);
      const double2 u = buf[i0], v = cmul(buf[i1], w);
      buf[i0] = add2(u, v);
      buf[i1] = sub2(u, v);
    }
    __syncthreads();
  }
}
__device__ void ifft_dif(double2 *buf, const double2 *__restrict__ tw, int P, int logP) {
  for (int s = logP; s >= 1; --s) {
    const int half = 1 << (s - 1);
    for (int i = threadIdx.x; i < P / 2; i += blockDim.x) {
      const int j = i & (half - 1);
      const int i0 = ((i >> (s - 1)) << s) + j, i1 = i0 + half;
      const double2 w = conj2(__ldg(&tw[j << (logP - s)]));
      const double2 u = buf[i0], v = buf[i1];
      buf[i0] = add2(u, v);
      buf[i1] = cmul(sub2(u, v), w);
    }
    __syncthreads();
  }
}

// Bluestein core: buf holds a_j (bit-reversed positions) on entry; on exit
// buf[brev(k)] holds P * y_k where y = a (*) chirp-kernel.
__device__ void bluestein_core(double2 *buf, const RingArgs &a) {
  __syncthreads();
  fft_dit(buf, a.tw, a.P, a.logP);
  for (int k = threadIdx.x; k < a.P; k += blockDim.x) buf[k] = cmul(buf[k], __ldg(&a.bhat[k]));
  __syncthreads();
  ifft_dif(buf, a.tw, a.P, a.logP);
}

template <bool REAL>
__global__ void __launch_bounds__(512) k_ring_forward(RingArgs a) {
  extern __shared__ double2 buf[];
  const int K = a.K, P = a.P, logP = a.logP;
  const int r0 = REAL ? 2 * blockIdx.x : blockIdx.x;
  const bool has1 = REAL && (r0 + 1 < a.nrings);
  for (int j = threadIdx.x; j < P; j += blockDim.x) {
    double2 z = make_double2(0.0, 0.0);
    if (j < K) {
      if (REAL) {
        z.x = ((const double *)a.rings)[ring_base(a, r0) + j];
        if (has1) z.y = ((const double *)a.rings)[ring_base(a, r0 + 1) + j];
      } else {
        z = ((const double2 *)a.rings)[ring_base(a, r0) + j];
      }
      z = cmulc(z, __ldg(&a.chirp[j]));  // x_j conj(c_j)
    }
    buf[brev(j, logP)] = z;
  }
  bluestein_core(buf, a);
  const double inv = 1.0 / (double)P;
  if (!REAL) {
    double2 *out = a.spec_out + spec_base(a, r0);
    for (int c = threadIdx.x; c < a.sw; c += blockDim.x) {
      const int m = a.mlo + c;
      const int k = ((m % K) + K) % K;
      out[c] = scl2(cmulc(buf[brev(k, logP)], __ldg(&a.chirp[k])), inv);
    }
  } else {
    double2 *out0 = a.spec_out + spec_base(a, r0);
    for (int m = threadIdx.x; m < a.sw; m += blockDim.x) {
      const int km = (K - m) % K;
      const double2 zm = scl2(cmulc(buf[brev(m, logP)], __ldg(&a.chirp[m])), inv);
      const double2 zk = scl2(cmulc(buf[brev(km, logP)], __ldg(&a.chirp[km])), inv);
      const double2 zc = conj2(zk);
      // A = (Z_m + conj Z_{-m})/2,  B = (Z_m - conj Z_{-m})/(2i)
      out0[m] = make_double2(0.5 * (zm.x + zc.x), 0.5 * (zm.y + zc.y));
      if (has1) {
        const double2 d = sub2(zm, zc);
        out0[a.spec_stride + m] = make_double2(0.5 * d.y, -0.5 * d.x);
      }
    }
  }
}

template <bool REAL>
__global__ void __launch_bounds__(512) k_ring_inverse(RingArgs a) {
  extern __shared__ double2 buf[];
  const int K = a.K, P = a.P, logP = a.logP, bl = a.bl;
  const int r0 = REAL ? 2 * blockIdx.x : blockIdx.x;
  const bool has1 = REAL && (r0 + 1 < a.nrings);
  const double2 *s0 = a.spec_in + spec_base(a, r0);
  for (int j = threadIdx.x; j < P; j += blockDim.x) {
    double2 z = make_double2(0.0, 0.0);
    if (j < K) {
      const int m = (j < bl) ? j : j - K;  // frequency of DFT bin j
      if (REAL) {
        const int am = m < 0 ? -m : m;
        if (am < a.sw) {
          double2 A = s0[am];
          double2 B = has1 ? s0[a.spec_stride + am] : make_double2(0.0, 0.0);
          if (m < 0) {
            A = conj2(A);
            B = conj2(B);
          }
          z = make_double2(A.x - B.y, A.y + B.x);  // A + i B
        }
      } else {
        const int c = m - a.mlo;
        if (c >= 0 && c < a.sw)
          z = s0[c];
        else if (a.herm && m < 0 && -m - a.mlo < a.sw)
          z = conj2(s0[-m - a.mlo]);
      }
      // inverse DFT = conj(forward(conj z)):  a_j = conj(z_j) conj(c_j)
      z = conj2(cmul(z, __ldg(&a.chirp[j])));
    }
    buf[brev(j, logP)] = z;
  }
  bluestein_core(buf, a);
  const double inv = 1.0 / (double)P;
  for (int p = threadIdx.x; p < K; p += blockDim.x) {
    // f_p = conj(conj(c_p) y_p) = c_p conj(y_p)
    const double2 y = scl2(buf[brev(p, logP)], inv);
    const double2 f = cmul(__ldg(&a.chirp[p]), conj2(y));
    if (REAL) {
      ((double *)a.rings_out)[ring_base(a, r0) + p] = f.x;
      if (has1) ((double *)a.rings_out)[ring_base(a, r0 + 1) + p] = f.y;
    } else {
      a.rings_out[ring_base(a, r0) + p] = f;
    }
  }
}

// ---------------------------------------------------------------------------
// Ring DFT in double-float arithmetic (split-precision path)
//
// Values are unevaluated sums hi + lo of two floats (48-bit significand, unit
// roundoff 2^-48, error-free transformations of Dekker/Knuth: two-sum,
// two-product by FMA).  Every operation is an explicit round-to-nearest
// intrinsic so that no multiply-add is contracted.  The same Bluestein steps
// as the FP64 kernels run on the FP32 pipe; each ring (pair) is scaled by a
// power of two first so that the float exponent range never limits accuracy.
//
// Sums and products are left unnormalised (no fast-two-sum after the error
// term is accumulated): hi + lo still equals the value to within the rounding
// of lo, and |lo| grows by at most ulp(hi)/2 plus the inputs' lo per
// operation, so after k operations it stays below k 2^-24 of the block's
// magnitude and its own rounding below k 2^-48.  Normwise this costs about a
// factor 2 in the error of a 4096-point transform (6.6e-15 -> 1.4e-14, l2,
// emulated on the CPU) for 22 % fewer FP32 instructions per butterfly; the
// FP64 widening at the end accepts any hi/lo split.
// ---------------------------------------------------------------------------

// Stages are paired (radix 2^2): one pass over shared memory and one barrier
// per two radix-2 stages; a leftover single stage when log2 P is odd.
//
// Shared-memory layout: element i of the P = 2^lg point buffer (16-byte
// complex double-float values, no padding) lives at swz(i) = i ^ X(i), where
// X(i) XORs bits 3-4 of i into bits 1-2, bits 3-5 into bits 0-2 and bits
// lg-3..lg-1 into bits 0-2 (the last term only for lg > 6).  X depends only on
// bits >= 3 and sets only bits 0-2, so swz is a bijection and its own inverse,
// and it is linear over GF(2): swz(a ^ b) = swz(a) ^ swz(b).  Every access
// pattern below (bit-reversed scatter and gather, the radix-2^2 passes at every
// span, stride-4 and linear sweeps) then touches 8 distinct 16-byte bank groups
// per quarter warp for P >= 256 (checked by enumerating the patterns on the
// CPU), without the 1/8 padding a skewed layout needs: a 4096-point buffer
// takes 64 KB, which leaves room in L1 for the twiddle table.
struct Swz {
  int top;  // lg - 3 when lg > 6, else 31 (the term vanishes for non-negative i)
};
__device__ __forceinline__ Swz swz_of(int logP) { return Swz{logP > 6 ? logP - 3 : 31}; }
__device__ __forceinline__ int swz(int i, Swz z) {
  return i ^ ((i >> 2) & 6) ^ ((i >> 3) & 7) ^ ((i >> z.top) & 7);
}
__device__ __forceinline__ float4 dc_mul_mi(float4 a) { return make_float4(a.z, a.w, -a.x, -a.y); }  // a * (-i)
__device__ __forceinline__ float4 dc_mul_pi(float4 a) { return make_float4(-a.z, -a.w, a.x, a.y); }  // a * (+i)

// Read-only table loads with an L1 eviction priority: the twiddle table is
// read by every pass of every ring on the SM (kept: evict_last); the chirp and
// the chirp-kernel spectrum are read once per ring (evict_first).
__device__ __forceinline__ float4 ld_keep(const float4 *p) {
  float4 v;
  asm("ld.global.nc.L1::evict_last.v4.f32 {%0, %1, %2, %3}, [%4];"
      : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
      : "l"(p));
  return v;
}
__device__ __forceinline__ float4 ld_once(const float4 *p) {
  float4 v;
  asm("ld.global.nc.L1::evict_first.v4.f32 {%0, %1, %2, %3}, [%4];"
      : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
      : "l"(p));
  return v;
}

// bit-reversed input, natural output, forward transform (w = e^{-2 pi i k / P}).
// The input is zero-padded past P/2 (the Bluestein sequences have K <= P/2
// values), i.e. zero at every odd bit-reversed position, and the first two
// stages have unit twiddles: that pass is a 4-point DFT of (a0, 0, a2, 0).
// In every pass the four points p0 + c h (c < 4) differ from p0 only in bits
// that are zero in p0, so their buffer slots are swz(p0) ^ swz(c h).
__device__ void fft_dit_df(float4 *buf, const float4 *__restrict__ tw, int P, int logP) {
  const Swz z = swz_of(logP);
  for (int i = threadIdx.x; i < P / 4; i += blockDim.x) {
    const int b = swz(4 * i, z);
    const float4 a0 = buf[b], a2 = buf[b ^ 2], a2m = dc_mul_mi(a2);
    buf[b] = dc_add(a0, a2);
    buf[b ^ 2] = dc_sub(a0, a2);
    buf[b ^ 1] = dc_add(a0, a2m);
    buf[b ^ 3] = dc_sub(a0, a2m);
  }
  __syncthreads();
  int s = 3;
  for (; s + 1 <= logP; s += 2) {
    const int h = 1 << (s - 1);
    const int q1 = swz(h, z), q2 = swz(2 * h, z), q3 = swz(3 * h, z);
    for (int i = threadIdx.x; i < P / 4; i += blockDim.x) {
      const int jp = i & (h - 1);
      const int b = swz(((i >> (s - 1)) << (s + 1)) + jp, z);
      const float4 w1 = ld_keep(&tw[jp << (logP - s)]);
      const float4 w2 = ld_keep(&tw[jp << (logP - s - 1)]);
      const float4 a0 = buf[b], a1 = buf[b ^ q1], a2 = buf[b ^ q2], a3 = buf[b ^ q3];
      const float4 t1 = dc_mul(a1, w1), t3 = dc_mul(a3, w1);
      const float4 b0 = dc_add(a0, t1), b1 = dc_sub(a0, t1), b2 = dc_add(a2, t3), b3 = dc_sub(a2, t3);
      const float4 u2 = dc_mul(b2, w2), u3 = dc_mul_mi(dc_mul(b3, w2));
      buf[b] = dc_add(b0, u2);
      buf[b ^ q2] = dc_sub(b0, u2);
      buf[b ^ q1] = dc_add(b1, u3);
      buf[b ^ q3] = dc_sub(b1, u3);
    }
    __syncthreads();
  }
  if (s == logP) {
    const int half = 1 << (s - 1);
    const int qh = swz(half, z);
    for (int i = threadIdx.x; i < P / 2; i += blockDim.x) {
      const int j = i & (half - 1);
      const int b = swz(((i >> (s - 1)) << s) + j, z);
      const float4 w = ld_keep(&tw[j << (logP - s)]);
      const float4 u = buf[b], v = dc_mul(buf[b ^ qh], w);
      buf[b] = dc_add(u, v);
      buf[b ^ qh] = dc_sub(u, v);
    }
    __syncthreads();
  }
}
// natural input, bit-reversed output, unnormalised inverse transform.  Only
// the outputs at even bit-reversed positions (natural index < P/2) are
// produced: the Bluestein result needs K <= P/2 of them.  The last pass has
// unit twiddles.
__device__ void ifft_dif_df(float4 *buf, const float4 *__restrict__ tw, int P, int logP) {
  const Swz z = swz_of(logP);
  int s = logP;
  for (; s >= 3; s -= 2) {
    const int h = 1 << (s - 2);
    const int q1 = swz(h, z), q2 = swz(2 * h, z), q3 = swz(3 * h, z);
    for (int i = threadIdx.x; i < P / 4; i += blockDim.x) {
      const int jp = i & (h - 1);
      const int b = swz(((i >> (s - 2)) << s) + jp, z);
      const float4 c2 = ld_keep(&tw[jp << (logP - s)]);
      const float4 c1 = ld_keep(&tw[jp << (logP - s + 1)]);
      const float4 a0 = buf[b], a1 = buf[b ^ q1], a2 = buf[b ^ q2], a3 = buf[b ^ q3];
      const float4 b0 = dc_add(a0, a2), b1 = dc_add(a1, a3);
      const float4 b2 = dc_mulc(dc_sub(a0, a2), c2), b3 = dc_mul_pi(dc_mulc(dc_sub(a1, a3), c2));
      buf[b] = dc_add(b0, b1);
      buf[b ^ q1] = dc_mulc(dc_sub(b0, b1), c1);
      buf[b ^ q2] = dc_add(b2, b3);
      buf[b ^ q3] = dc_mulc(dc_sub(b2, b3), c1);
    }
    __syncthreads();
  }
  if (s == 2) {  // stages 2 and 1, unit twiddles, even outputs only
    for (int i = threadIdx.x; i < P / 4; i += blockDim.x) {
      const int b = swz(4 * i, z);
      const float4 a0 = buf[b], a1 = buf[b ^ 1], a2 = buf[b ^ 2], a3 = buf[b ^ 3];
      buf[b] = dc_add(dc_add(a0, a2), dc_add(a1, a3));
      buf[b ^ 2] = dc_add(dc_sub(a0, a2), dc_mul_pi(dc_sub(a1, a3)));
    }
    __syncthreads();
  } else if (s == 1) {
    for (int i = threadIdx.x; i < P / 2; i += blockDim.x) {
      const int b = swz(2 * i, z);
      buf[b] = dc_add(buf[b], buf[b ^ 1]);
    }
    __syncthreads();
  }
}
// pointwise product with the chirp-kernel spectrum (every slot, any order)
__device__ __forceinline__ void kernel_multiply_df(float4 *buf, const float4 *__restrict__ bhat, int P, int logP) {
  const Swz z = swz_of(logP);
  for (int k = threadIdx.x; k < P; k += blockDim.x) {
    const int b = swz(k, z);
    buf[b] = dc_mul(buf[b], ld_once(&bhat[k]));
  }
  __syncthreads();
}
// buffer slot of bit-reversed position k
__device__ __forceinline__ int slot_brev(int k, int logP) { return swz(brev(k, logP), swz_of(logP)); }

// block-wide max of an int (blockDim.x <= 1024)
__device__ int block_max_int(int v) {
  __shared__ int redi[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) redi[threadIdx.x >> 5] = v;
  __syncthreads();
  int m = 0;
  for (int i = 0; i < (int)((blockDim.x + 31) >> 5); ++i) m = max(m, redi[i]);
  return m;
}
__device__ __forceinline__ int emax2(int m, double2 z) { return max(m, max(exp_field(z.x), exp_field(z.y))); }

template <bool REAL>
__global__ void __launch_bounds__(512, 3) k_ring_forward_df(RingArgs a) {
  extern __shared__ float4 bufd[];
  const int K = a.K, P = a.P, logP = a.logP;
  const int r0 = REAL ? 2 * blockIdx.x : blockIdx.x;
  const bool has1 = REAL && (r0 + 1 < a.nrings);
  int em = 0;
  for (int j = threadIdx.x; j < K; j += blockDim.x) {
    if (REAL) {
      em = max(em, exp_field(((const double *)a.rings)[ring_base(a, r0) + j]));
      if (has1) em = max(em, exp_field(((const double *)a.rings)[ring_base(a, r0 + 1) + j]));
    } else {
      em = emax2(em, ((const double2 *)a.rings)[ring_base(a, r0) + j]);
    }
  }
  const int e = block_scale(block_max_int(em));
  for (int j = threadIdx.x; j < P; j += blockDim.x) {
    float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    if (j < K) {
      double2 v;
      if (REAL) {
        v.x = ((const double *)a.rings)[ring_base(a, r0) + j];
        v.y = has1 ? ((const double *)a.rings)[ring_base(a, r0 + 1) + j] : 0.0;
      } else {
        v = ((const double2 *)a.rings)[ring_base(a, r0) + j];
      }
      z = dc_mulc(dc_split(v, e), ld_once(&a.chirp_df[j]));
    }
    bufd[slot_brev(j, logP)] = z;
  }
  __syncthreads();
  fft_dit_df(bufd, a.tw_df, P, logP);
  kernel_multiply_df(bufd, a.bhat_df, P, logP);
  ifft_dif_df(bufd, a.tw_df, P, logP);
  const int eo = e - logP;  // undo the ring scaling and the 1/P of the unnormalised transforms
  if (!REAL) {
    double2 *out = a.spec_out + spec_base(a, r0);
    for (int c = threadIdx.x; c < a.sw; c += blockDim.x) {
      const int m = a.mlo + c;
      const int k = ((m % K) + K) % K;
      out[c] = dc_to(dc_mulc(bufd[slot_brev(k, logP)], ld_once(&a.chirp_df[k])), eo);
    }
  } else {
    double2 *out0 = a.spec_out + spec_base(a, r0);
    for (int m = threadIdx.x; m < a.sw; m += blockDim.x) {
      const int km = (K - m) % K;
      const float4 zm = dc_mulc(bufd[slot_brev(m, logP)], ld_once(&a.chirp_df[m]));
      const float4 zc = dc_conj(dc_mulc(bufd[slot_brev(km, logP)], ld_once(&a.chirp_df[km])));
      // A = (Z_m + conj Z_{-m})/2,  B = (Z_m - conj Z_{-m})/(2i)
      const double2 s = dc_to(dc_add(zm, zc), eo - 1);
      out0[m] = s;
      if (has1) {
        const double2 d = dc_to(dc_sub(zm, zc), eo - 1);
        out0[a.spec_stride + m] = make_double2(d.y, -d.x);
      }
    }
  }
}

template <bool REAL>
__global__ void __launch_bounds__(512, 3) k_ring_inverse_df(RingArgs a) {
  extern __shared__ float4 bufd[];
  const int K = a.K, P = a.P, logP = a.logP, bl = a.bl;
  const int r0 = REAL ? 2 * blockIdx.x : blockIdx.x;
  const bool has1 = REAL && (r0 + 1 < a.nrings);
  const double2 *s0 = a.spec_in + spec_base(a, r0);
  int em = 0;
  for (int c = threadIdx.x; c < a.sw; c += blockDim.x) {
    em = emax2(em, s0[c]);
    if (has1) em = emax2(em, s0[a.spec_stride + c]);
  }
  const int e = block_scale(block_max_int(em));
  for (int j = threadIdx.x; j < P; j += blockDim.x) {
    float4 zz = make_float4(0.f, 0.f, 0.f, 0.f);
    if (j < K) {
      const int m = (j < bl) ? j : j - K;
      if (REAL) {
        const int am = m < 0 ? -m : m;
        if (am < a.sw) {
          float4 A = dc_split(s0[am], e);
          float4 B = has1 ? dc_split(s0[a.spec_stride + am], e) : make_float4(0.f, 0.f, 0.f, 0.f);
          if (m < 0) {
            A = dc_conj(A);
            B = dc_conj(B);
          }
          // A + i B
          zz = dmk(df_add(dre(A), df_neg(dim_(B))), df_add(dim_(A), dre(B)));
        }
      } else {
        const int c = m - a.mlo;
        if (c >= 0 && c < a.sw)
          zz = dc_split(s0[c], e);
        else if (a.herm && m < 0 && -m - a.mlo < a.sw)
          zz = dc_conj(dc_split(s0[-m - a.mlo], e));
      }
    }
    float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
    // inverse DFT = conj(forward(conj z)):  a_j = conj(z_j) conj(c_j)
    if (j < K) v = dc_conj(dc_mul(zz, ld_once(&a.chirp_df[j])));
    bufd[slot_brev(j, logP)] = v;
  }
  __syncthreads();
  fft_dit_df(bufd, a.tw_df, P, logP);
  kernel_multiply_df(bufd, a.bhat_df, P, logP);
  ifft_dif_df(bufd, a.tw_df, P, logP);
  const int eo = e - logP;
  for (int p = threadIdx.x; p < K; p += blockDim.x) {
    // f_p = c_p conj(y_p)
    const double2 f = dc_to(dc_mul(ld_once(&a.chirp_df[p]), dc_conj(bufd[slot_brev(p, logP)])), eo);
    if (REAL) {
      ((double *)a.rings_out)[ring_base(a, r0) + p] = f.x;
      if (has1) ((double *)a.rings_out)[ring_base(a, r0 + 1) + p] = f.y;
    } else {
      a.rings_out[ring_base(a, r0) + p] = f;
    }
  }
}

RingArgs ring_args(const RingFFT &rf, int bl, int nrings) {
  RingArgs a{};
  a.spec_rpm = 1 << 30;  // single-level spectrum addressing unless set
  a.spec_map_stride = 0;
  a.K = rf.K;
  a.P = rf.P;
  a.logP = rf.logP;
  a.bl = bl;
  a.nrings = nrings;
  a.chirp = rf.chirp;
  a.bhat = rf.bhat;
  a.tw = rf.tw;
  a.chirp_df = rf.chirp_df;
  a.bhat_df = rf.bhat_df;
  a.tw_df = rf.tw_df;
  return a;
}

int ring_threads(int P) { return P / 2 >= 512 ? 512 : (P / 2 >= 32 ? P / 2 : 32); }

// ---------------------------------------------------------------------------
// Contractions
// ---------------------------------------------------------------------------

constexpr int CT_M = 128;  // rows (t or l) per CTA
constexpr int CT_K = 32;   // reduction tile
// split precision: batches of at most this many maps contract in double-float
// on the FP64 tables instead of streaming the tensor path's digit panels
// (s2let_gpu_set_df_max_maps, initially S2LET_GPU_DF_MAX_MAPS or 1; 0 keeps
// every batch on the tensor path)
std::atomic<int> g_df_max_maps{[] {
  const char *e = getenv("S2LET_GPU_DF_MAX_MAPS");
  const int x = e ? atoi(e) : 1;
  return (x >= 0 && x <= 4) ? x : 1;
}()};
int df_max_maps() { return g_df_max_maps.load(); }

struct TableRef {
  int mi;       // m index inside the table
  double sign;  // (-1)^{m+|n|} when read through the n -> -n mirror
};
__device__ __forceinline__ TableRef table_ref(int mlo_table, int n, int m) {
  TableRef r;
  if (n > 0 || (n == 0 && m >= 0)) {
    r.mi = m - mlo_table;
    r.sign = 1.0;
  } else {
    const int an = n < 0 ? -n : n;
    r.mi = -m - mlo_table;
    r.sign = ((m + an) & 1) ? -1.0 : 1.0;
  }
  return r;
}

struct ContractArgs {
  const double *table;
  const float2 *table_df;  // double-float copy of table (same offsets), or null
  const int64_t *off;
  int bl, nt, an, tmlo, n, mlo, lmin;  // nt: theta samples of the table
  const double2 *w;
  double wscale;
  int wconj;
  // l->t: x source / spectra dest;  t->l: spectra source / y dest
  const double2 *src;
  int64_t ss;
  int sw_or_xL;  // t->l: spectrum row width; l->t: x band-limit
  int s_mlo;     // t->l: m of spectrum column 0
  int x_half;
  double2 *dst;
  int64_t ds;
  int dw, d_mlo;  // l->t: spectrum row width / m of column 0
  int nb;
  // double-float kernel: a second part on the same table and m range (another
  // scale of the same band-limit and n) with its own source, destination,
  // weights and lmin, contracted in the same pass over the table
  int nparts;
  const double2 *src2;
  double2 *dst2;
  const double2 *w2;
  int lmin2;
};

__device__ __forceinline__ double2 weight_at(const ContractArgs &a, int l) {
  double2 w = a.w ? a.w[l] : make_double2(1.0, 0.0);
  if (a.wconj) w.y = -w.y;
  return scl2(w, a.wscale);
}

// MODE 0: l->t with D (A[t][l] = D[t][l-l0])     MODE 1: l->t with Q^T (A[t][l] = Q[l-l0][t])
// MODE 2: t->l with Q (A[l][t] = Q[l-l0][t])     MODE 3: t->l with D^T (A[l][t] = D[t][l-l0])
template <int MODE, int NBT>
__global__ void __launch_bounds__(CT_M) k_contract(ContractArgs a) {
  __shared__ double sA[CT_M][CT_K + 1];
  __shared__ double2 sX[CT_K][NBT];
  const int m = a.mlo + blockIdx.x;
  const int am = m < 0 ? -m : m;
  const int l0 = am > a.an ? am : a.an;
  const int bl = a.bl;
  const int nl = bl - l0;
  const int lst = l0 > a.lmin ? l0 : a.lmin;
  constexpr bool L2T = (MODE == 0 || MODE == 1);
  // l -> t with no admissible l still writes its (zero) output rows
  if (!L2T && lst >= bl) return;
  const TableRef tr = table_ref(a.tmlo, a.n, m);
  const double *T = (lst < bl) ? a.table + a.off[tr.mi] : a.table;
  const int b0 = blockIdx.z * NBT;
  const int r = threadIdx.x;
  // rows of this CTA
  const int row0 = blockIdx.y * CT_M;
  const int nt = a.nt;
  const int rows_total = L2T ? nt : (bl - lst);
  if (row0 >= rows_total) return;
  const int kbeg = L2T ? lst : 0, kend = L2T ? bl : nt;  // reduction range (l for L2T, t for T2L)

  double2 acc[NBT];
#pragma unroll
  for (int b = 0; b < NBT; ++b) acc[b] = make_double2(0.0, 0.0);

  for (int k0 = kbeg; k0 < kend; k0 += CT_K) {
    // coefficient tile
    for (int i = threadIdx.x; i < CT_K * NBT; i += CT_M) {
      const int kk = i / NBT, b = i % NBT, k = k0 + kk;
      double2 v = make_double2(0.0, 0.0);
      if (k < kend && b0 + b < a.nb) {
        if (L2T) {  // x(l = k, m) * w(l)
          const int64_t base = (int64_t)(b0 + b) * a.ss + (int64_t)k * k + k;
          if (a.x_half && m < 0) {
            v = conj2(a.src[base - m]);
            if (am & 1) v = scl2(v, -1.0);
          } else {
            v = a.src[base + m];
          }
          v = cmul(v, weight_at(a, k));
        } else {  // spectrum(t = k, m)
          v = a.src[(int64_t)(b0 + b) * a.ss + (int64_t)k * a.sw_or_xL + (m - a.s_mlo)];
        }
      }
      sX[kk][b] = v;
    }
    // table tile sA[row][kk]
    if (MODE == 0 || MODE == 2) {
      // contiguous along the reduction axis: D[t][l-l0] (MODE 0) or Q[l-l0][t] (MODE 2)
      for (int i = threadIdx.x; i < CT_M * CT_K; i += CT_M) {
        const int rr = i / CT_K, kk = i % CT_K;
        const int row = row0 + rr, k = k0 + kk;
        double v = 0.0;
        if (row < rows_total && k < kend) {
          if (MODE == 0)
            v = T[(int64_t)row * nl + (k - l0)];
          else
            v = T[(int64_t)(lst + row - l0) * nt + k];
        }
        sA[rr][kk] = v;
      }
    } else {
      // contiguous along the row axis: Q[l-l0][t] read as A[t][l] (MODE 1),
      // D[t][l-l0] read as A[l][t] (MODE 3)
      for (int i = threadIdx.x; i < CT_M * CT_K; i += CT_M) {
        const int kk = i / CT_M, rr = i % CT_M;
        const int row = row0 + rr, k = k0 + kk;
        double v = 0.0;
        if (row < rows_total && k < kend) {
          if (MODE == 1)
            v = T[(int64_t)(k - l0) * nt + row];
          else
            v = T[(int64_t)k * nl + (lst + row - l0)];
        }
        sA[rr][kk] = v;
      }
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < CT_K; ++kk) {
      const double av = sA[r][kk];
#pragma unroll
      for (int b = 0; b < NBT; ++b) {
        const double2 x = sX[kk][b];
        acc[b].x = fma(av, x.x, acc[b].x);
        acc[b].y = fma(av, x.y, acc[b].y);
      }
    }
    __syncthreads();
  }
  const int row = row0 + r;
  if (row >= rows_total) return;
#pragma unroll
  for (int b = 0; b < NBT; ++b) {
    if (b0 + b >= a.nb) break;
    double2 v = scl2(acc[b], tr.sign);
    if (L2T) {
      a.dst[(int64_t)(b0 + b) * a.ds + (int64_t)row * a.dw + (m - a.d_mlo)] = v;
    } else {
      const int l = lst + row;
      v = cmul(v, weight_at(a, l));
      a.dst[(int64_t)(b0 + b) * a.ds + (int64_t)l * l + l + m] = v;
    }
  }
}

// The same contractions in double-float on the FP32 pipe (split-precision
// path: every contraction the tensor-core kernel does not take, and batches of
// at most df_max_maps() maps, for which streaming the tables' 7 bf16 digit
// panels (14 B per entry) costs more than reading 8 B per entry and
// multiplying in double-float).
//
// A CTA owns one m and up to 128 output rows.  It first splits its coefficient
// columns (maps x parts; a second part is another scale on the same table)
// over the whole reduction range into double-float pairs in shared memory,
// one power-of-two scale per column (|x| 2^-e < 1).  Table values (|d| <= 1)
// come from the double-float copy of the table (df_table) or are split from
// FP64 as they are read (df_split_unit).  Products are summed as in Ogita,
// Rump and Oishi's Dot2 (SIAM J. Sci. Comput. 26, 2005): a float sum s carried
// by TwoSum, its rounding errors and the products' low parts gathered in a
// second float c, so that s + c is the sum as if computed in twice the working
// precision; (s + c) 2^e is widened to FP64 once per output.
//   MODE 1, 3 (table contiguous along the output rows): one thread per row,
//   each step of the reduction a coalesced warp-wide row of the table.
//   MODE 0, 2 (table contiguous along the reduction axis): groups of DFC_LPR
//   lanes along the reduction axis, one row per group and several rows per
//   lane, the next step's table loads issued before the current step's
//   arithmetic; the groups' partial sums are reduced by butterfly shuffles.

// v (|v| <= 1 or zero) as hi + lo: the top 24 and next 23 significand bits
// (truncated: |hi + lo - v| < 2^-46 |v|); |v| < 2^-103 gives 0
__device__ __forceinline__ float2 df_split_unit(double v) {
  const uint32_t wl = (uint32_t)__double2loint(v), wh = (uint32_t)__double2hiint(v);
  const uint32_t mag = wh & 0x7FFFFFFFu;
  const uint32_t eb = mag - 0x38000000u;  // float exponent field at bits 20..27
  const uint32_t hb = __funnelshift_l(wl, eb, 3) | (wh & 0x80000000u);
  const uint32_t base = (hb & 0xFF800000u) - (23u << 23);
  const uint32_t lb = base | ((wl >> 6) & 0x7FFFFFu);
  const bool ok = mag >= 0x39800000u;  // double exponent >= 1023 - 103
  const float hi = __uint_as_float(hb);
  const float lo = __fsub_rn(__uint_as_float(lb), __uint_as_float(base));
  return ok ? make_float2(hi, lo) : make_float2(0.0f, 0.0f);
}

// table value as a double-float pair: split as read (FP64 table) or stored split
__device__ __forceinline__ float2 unit_df(double v) { return df_split_unit(v); }
__device__ __forceinline__ float2 unit_df(float2 v) { return v; }

// Dot2 step: (s, c) += a * x, a and x double-float reals
__device__ __forceinline__ void dot2_mac(float &s, float &c, float2 av, float xh, float xl) {
  const float p = __fmul_rn(av.x, xh);
  const float q = __fmaf_rn(av.x, xh, -p);
  const float t = __fadd_rn(s, p);
  const float v = __fsub_rn(t, s);
  const float r = __fadd_rn(__fsub_rn(s, __fsub_rn(t, v)), __fsub_rn(p, v));
  s = t;
  c = __fadd_rn(c, __fadd_rn(q, r));
  c = __fmaf_rn(av.x, xl, c);
  c = __fmaf_rn(av.y, xh, c);
}
// (s, c) += (s2, c2), symmetric in its two operands: TwoSum's error r is
// exact and c + c2 commutes, so both lanes of a butterfly step get the same
// bits (the lane that stores a sum then does not matter)
__device__ __forceinline__ void dot2_add(float &s, float &c, float s2, float c2) {
  const float t = __fadd_rn(s, s2);
  const float v = __fsub_rn(t, s);
  const float r = __fadd_rn(__fsub_rn(s, __fsub_rn(t, v)), __fsub_rn(s2, v));
  s = t;
  c = __fadd_rn(__fadd_rn(c, c2), r);
}

// complex product with explicit roundings: every instantiation of the
// double-float kernel (maps per CTA, table element type) rounds the same way,
// so that launch shapes chosen by the autotuner give identical bits
__device__ __forceinline__ double2 cmul_rn(double2 a, double2 b) {
  return make_double2(__fma_rn(a.x, b.x, __dmul_rn(-a.y, b.y)), __fma_rn(a.x, b.y, __dmul_rn(a.y, b.x)));
}
__device__ __forceinline__ double2 weight_at_part(const ContractArgs &a, int p, int l) {
  const double2 *wp = p ? a.w2 : a.w;
  double2 w = wp ? wp[l] : make_double2(1.0, 0.0);
  if (a.wconj) w.y = -w.y;
  return make_double2(__dmul_rn(w.x, a.wscale), __dmul_rn(w.y, a.wscale));
}

// coefficient k of map b of part p for column m (x(l = k, m) w(l) for l->t,
// spectrum(t = k, m) for t->l)
template <bool L2T>
__device__ __forceinline__ double2 contract_coef(const ContractArgs &a, int p, int m, int am, int k, int b) {
  const double2 *src = p ? a.src2 : a.src;
  if (L2T) {
    const int64_t base = (int64_t)b * a.ss + (int64_t)k * k + k;
    double2 v;
    if (a.x_half && m < 0) {
      v = conj2(src[base - m]);
      if (am & 1) v = scl2(v, -1.0);
    } else {
      v = src[base + m];
    }
    return cmul_rn(v, weight_at_part(a, p, k));
  }
  return src[(int64_t)b * a.ss + (int64_t)k * a.sw_or_xL + (m - a.s_mlo)];
}

// output of map b of part p at row (t for l->t, l - lst for t->l); t->l rows
// below the part's first degree lstp are not written
template <bool L2T>
__device__ __forceinline__ void contract_store(const ContractArgs &a, int p, int b, int m, int row, int lst,
                                               int lstp, double2 v) {
  double2 *dst = p ? a.dst2 : a.dst;
  if (L2T) {
    dst[(int64_t)b * a.ds + (int64_t)row * a.dw + (m - a.d_mlo)] = v;
  } else {
    const int l = lst + row;
    if (l < lstp) return;
    dst[(int64_t)b * a.ds + (int64_t)l * l + l + m] = cmul_rn(v, weight_at_part(a, p, l));
  }
}

constexpr int DFC_R = 8;    // rows per lane (MODE 0, 2; half that from 4 maps per CTA)
constexpr int DFC_LPR = 8;  // lanes per row (MODE 0, 2)

template <int MODE, int NBT, class E>
__global__ void __launch_bounds__(CT_M) k_contract_df(ContractArgs a) {
  extern __shared__ float4 sx[];  // [k - kbeg][b]
  __shared__ int sxm[NBT];
  const int m = a.mlo + blockIdx.x;
  const int am = m < 0 ? -m : m;
  const int l0 = am > a.an ? am : a.an;
  const int bl = a.bl;
  const int nl = bl - l0;
  // columns: NBT = maps per CTA x parts (column c: part c / mpc, map b0 + c % mpc)
  const int np = a.nparts == 2 ? 2 : 1;
  const int mpc = NBT / np;
  const int lmin_u = (np == 2 && a.lmin2 < a.lmin) ? a.lmin2 : a.lmin;
  const int lst = l0 > lmin_u ? l0 : lmin_u;  // first degree of any part
  constexpr bool L2T = (MODE == 0 || MODE == 1);
  if (!L2T && lst >= bl) return;
  const TableRef tr = table_ref(a.tmlo, a.n, m);
  const E *T0;
  if constexpr (std::is_same<E, double>::value)
    T0 = a.table;
  else
    T0 = a.table_df;
  const E *T = (lst < bl) ? T0 + a.off[tr.mi] : T0;
  const int b0 = blockIdx.z * mpc;
  const int row0 = blockIdx.y * CT_M;
  const int nt = a.nt;
  const int rows_total = L2T ? nt : (bl - lst);
  if (row0 >= rows_total) return;
  const int kbeg = L2T ? lst : 0, kend = L2T ? bl : nt;
  const int K = kend > kbeg ? kend - kbeg : 0;

  // coefficient columns: per-column scale, then the double-float split.  The
  // stride CT_M is a multiple of NBT, so each thread serves one column.  l->t
  // coefficients below a part's first degree are zero.
  const int bt = threadIdx.x % NBT;
  const int pt = bt / mpc, mt = b0 + bt % mpc;
  const bool bon = mt < a.nb;
  const int lpt = pt ? a.lmin2 : a.lmin;
  const int lst_t = l0 > lpt ? l0 : lpt;
  // The weighted FP64 values go to the same 16-byte slots first and are split
  // in place once the column scale is known (each slot by the thread that
  // wrote it), so the FP64 weighting runs once per coefficient.
  if (threadIdx.x < NBT) sxm[threadIdx.x] = 0;
  __syncthreads();
  double2 *sxd = reinterpret_cast<double2 *>(sx);
  int emax = 0;
  for (int i = threadIdx.x; i < K * NBT; i += CT_M) {
    const int k = kbeg + i / NBT;
    double2 v = make_double2(0.0, 0.0);
    if (bon && !(L2T && k < lst_t)) v = contract_coef<L2T>(a, pt, m, am, k, mt);
    sxd[i] = v;
    emax = max(emax, max(exp_field(v.x), exp_field(v.y)));
  }
  atomicMax(&sxm[bt], emax);
  __syncthreads();
  const int es = block_scale(sxm[bt]);
  for (int i = threadIdx.x; i < K * NBT; i += CT_M) sx[i] = dc_split(sxd[i], es);
  __syncthreads();
  int eo[NBT];
#pragma unroll
  for (int b = 0; b < NBT; ++b) eo[b] = block_scale(sxm[b]);

  if (MODE == 1 || MODE == 3) {
    const int row = row0 + threadIdx.x;
    if (row >= rows_total) return;
    // 32-bit element offsets from the CTA's table block
    const uint32_t tstride = MODE == 1 ? (uint32_t)nt : (uint32_t)nl;
    const uint32_t t0 = MODE == 1 ? (uint32_t)(kbeg - l0) * tstride + (uint32_t)row
                                  : (uint32_t)kbeg * tstride + (uint32_t)(lst + row - l0);
    float sre[NBT], cre[NBT], sim[NBT], cim[NBT];
#pragma unroll
    for (int b = 0; b < NBT; ++b) sre[b] = cre[b] = sim[b] = cim[b] = 0.f;
    int k = 0;
    for (; k + 8 <= K; k += 8) {
      E tv[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) tv[j] = T[t0 + (uint32_t)(k + j) * tstride];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const float2 av = unit_df(tv[j]);
#pragma unroll
        for (int b = 0; b < NBT; ++b) {
          const float4 x = sx[(k + j) * NBT + b];
          dot2_mac(sre[b], cre[b], av, x.x, x.y);
          dot2_mac(sim[b], cim[b], av, x.z, x.w);
        }
      }
    }
    for (; k < K; ++k) {
      const float2 av = unit_df(T[t0 + (uint32_t)k * tstride]);
#pragma unroll
      for (int b = 0; b < NBT; ++b) {
        const float4 x = sx[k * NBT + b];
        dot2_mac(sre[b], cre[b], av, x.x, x.y);
        dot2_mac(sim[b], cim[b], av, x.z, x.w);
      }
    }
#pragma unroll
    for (int c = 0; c < NBT; ++c) {
      const int p = c / mpc, b = b0 + c % mpc;
      if (b >= a.nb) continue;
      const int lp = p ? a.lmin2 : a.lmin;
      const double2 v =
          scl2(make_double2(join_scaled(sre[c], cre[c], eo[c]), join_scaled(sim[c], cim[c], eo[c])), tr.sign);
      contract_store<L2T>(a, p, b, m, row, lst, l0 > lp ? l0 : lp, v);
    }
    return;
  }

  // MODE 0, 2: groups of DFC_LPR lanes along the reduction axis, one row per
  // group and DFC_R rows per lane; the next step's table values are loaded
  // before the current step's arithmetic
  constexpr int R = NBT <= 2 ? DFC_R : DFC_R / 2;
  constexpr int GPW = 32 / DFC_LPR;  // row groups per warp
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int sub = lane % DFC_LPR, grp = lane / DFC_LPR;
  const uint32_t rs = MODE == 0 ? (uint32_t)nl : (uint32_t)nt;  // table row stride
  for (int g = 0; g < 32; g += GPW * R) {
    const int rbase = row0 + warp * 32 + g;
    if (rbase >= rows_total) break;
    // rows of this lane: rbase + grp + GPW i (past the end: the last row, not stored)
    uint32_t roff[R];
#pragma unroll
    for (int i = 0; i < R; ++i) {
      const int row = min(rbase + grp + GPW * i, rows_total - 1);
      roff[i] = MODE == 0 ? (uint32_t)row * rs + (uint32_t)(kbeg - l0) : (uint32_t)(lst + row - l0) * rs;
    }
    float sre[R][NBT], cre[R][NBT], sim[R][NBT], cim[R][NBT];
#pragma unroll
    for (int i = 0; i < R; ++i)
#pragma unroll
      for (int b = 0; b < NBT; ++b) sre[i][b] = cre[i][b] = sim[i][b] = cim[i][b] = 0.f;
    // loads past the reduction range re-read its last entry (the value is not
    // used); an empty range (l -> t with no admissible l) reads nothing
    E cur[R] = {};
    if (K > 0)
#pragma unroll
      for (int i = 0; i < R; ++i) cur[i] = T[roff[i] + (uint32_t)min(sub, K - 1)];
    for (int k = sub; k < K + sub; k += DFC_LPR) {
      const uint32_t kn = (uint32_t)min(k + DFC_LPR, K - 1);
      E nxt[R];
#pragma unroll
      for (int i = 0; i < R; ++i) nxt[i] = T[roff[i] + kn];
      if (k < K) {
        float4 x[NBT];
#pragma unroll
        for (int b = 0; b < NBT; ++b) x[b] = sx[k * NBT + b];
#pragma unroll
        for (int i = 0; i < R; ++i) {
          const float2 av = unit_df(cur[i]);
#pragma unroll
          for (int b = 0; b < NBT; ++b) {
            dot2_mac(sre[i][b], cre[i][b], av, x[b].x, x[b].y);
            dot2_mac(sim[i][b], cim[i][b], av, x[b].z, x[b].w);
          }
        }
      }
#pragma unroll
      for (int i = 0; i < R; ++i) cur[i] = nxt[i];
    }
#pragma unroll
    for (int i = 0; i < R; ++i) {
#pragma unroll
      for (int b = 0; b < NBT; ++b) {
#pragma unroll
        for (int off = DFC_LPR / 2; off >= 1; off >>= 1) {
          const float s2 = __shfl_xor_sync(0xFFFFFFFFu, sre[i][b], off);
          const float c2 = __shfl_xor_sync(0xFFFFFFFFu, cre[i][b], off);
          const float t2 = __shfl_xor_sync(0xFFFFFFFFu, sim[i][b], off);
          const float d2 = __shfl_xor_sync(0xFFFFFFFFu, cim[i][b], off);
          dot2_add(sre[i][b], cre[i][b], s2, c2);
          dot2_add(sim[i][b], cim[i][b], t2, d2);
        }
      }
      // lane sub = c of each group stores column c of the group's row
      const int row = rbase + grp + GPW * i;
      if (sub < NBT && row < rows_total) {
#pragma unroll
        for (int c = 0; c < NBT; ++c) {
          const int p = c / mpc, b = b0 + c % mpc;
          if (c != sub || b >= a.nb) continue;
          const int lp = p ? a.lmin2 : a.lmin;
          const double2 v = scl2(make_double2(join_scaled(sre[i][c], cre[i][c], eo[c]),
                                              join_scaled(sim[i][c], cim[i][c], eo[c])),
                                 tr.sign);
          contract_store<L2T>(a, p, b, m, row, lst, l0 > lp ? l0 : lp, v);
        }
      }
    }
  }
}

// algorithmic work of one contraction launch: one complex x real MAC (4 flops)
// per (l, m, t) per map; bytes = table entries read once + coefficient/spectrum I/O
void contract_work(const ContractArgs &a, int nm, double *flops, double *bytes, double *table_bytes = nullptr) {
  double macs = 0, tab = 0, io = 0;
  for (int i = 0; i < nm; ++i) {
    const int m = a.mlo + i, am = m < 0 ? -m : m;
    const int l0 = am > a.an ? am : a.an, lst = l0 > a.lmin ? l0 : a.lmin;
    const int nl = a.bl - lst;
    if (nl <= 0) continue;
    macs += (double)nl * a.nt;
    tab += (double)nl * a.nt;
    io += (double)nl + a.nt;
  }
  *flops = 4.0 * macs * a.nb;
  *bytes = 8.0 * tab + 16.0 * io * a.nb;
  if (table_bytes) *table_bytes = 8.0 * tab;
}

constexpr size_t kDfcSmemMax = 200 * 1024;

template <int MODE, int NBT, class E>
void launch_contract_df_e(dim3 grid, size_t smem, const ContractArgs &a, cudaStream_t st) {
  static bool attr = [] {
    S2G_CUDA(cudaFuncSetAttribute(k_contract_df<MODE, NBT, E>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)kDfcSmemMax));
    return true;
  }();
  (void)attr;
  k_contract_df<MODE, NBT, E><<<grid, CT_M, smem, st>>>(a);
}
template <int MODE, int NBT>
void launch_contract_df(dim3 grid, size_t smem, const ContractArgs &a, cudaStream_t st) {
  if (a.table_df)
    launch_contract_df_e<MODE, NBT, float2>(grid, smem, a, st);
  else
    launch_contract_df_e<MODE, NBT, double>(grid, smem, a, st);
}

// Double-float copies of stored Wigner tables for the double-float
// contractions (same layout and offsets, hi + lo per entry: the same 8 bytes
// as FP64, no splitting in the contraction loop).  Built on first use per
// table while the device keeps kDftReserve bytes free after the copy, else
// the contraction splits the FP64 values as it reads them.
constexpr size_t kDftReserve = size_t(4) << 30;
std::mutex g_dft_mu;
std::map<const double *, float2 *> g_dft;
size_t g_dft_bytes = 0;
std::atomic<int> g_split_tables{1};

__global__ void k_split_table(const double *__restrict__ in, float2 *__restrict__ out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = df_split(in[i], 0);
}

const float2 *df_table(const WignerTable &tb, bool q, cudaStream_t st) {
  const double *src = q ? tb.Q : tb.D;
  if (!src || !g_split_tables.load()) return nullptr;
  std::lock_guard<std::mutex> lk(g_dft_mu);
  auto it = g_dft.find(src);
  if (it != g_dft.end()) return it->second;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  S2G_CUDA(cudaStreamIsCapturing(st, &cap));
  if (cap != cudaStreamCaptureStatusNone) return nullptr;  // no allocation inside a graph capture
  const int64_t n = tb.elems();
  const size_t by = sizeof(float2) * (size_t)(n > 0 ? n : 1);
  size_t fr = 0, tot = 0;
  S2G_CUDA(cudaMemGetInfo(&fr, &tot));
  if (fr < by + kDftReserve) return nullptr;
  float2 *p = nullptr;
  S2G_CUDA(cudaMalloc(&p, by));
  const int64_t blocks = std::min<int64_t>(ceil_div(n > 0 ? n : 1, 256), 152 * 16);
  k_split_table<<<(unsigned)blocks, 256, 0, st>>>(src, p, n);
  S2G_LAUNCHED();
  S2G_CUDA(cudaStreamSynchronize(st));
  g_dft.emplace(src, p);
  g_dft_bytes += by;
  return p;
}

template <int MODE>
void launch_contract_nbt(const ContractArgs &a, int nm, int rows, int nbt, cudaStream_t st) {
  dim3 grid(nm, ceil_div(rows, CT_M), ceil_div(a.nb, nbt));
  if (t_precision == 1) {  // split precision: the double-float kernel
    // shared memory: the split coefficient columns over the reduction range
    const int kmax = a.bl > a.nt ? a.bl : a.nt;
    while (nbt > 1 && (size_t)kmax * nbt * sizeof(float4) > kDfcSmemMax) nbt /= 2;
    S2G_REQUIRE((size_t)kmax * sizeof(float4) <= kDfcSmemMax, ERR_UNSUPPORTED,
                "reduction range too long for the double-float contraction");
    grid.z = ceil_div(a.nb, nbt);
    const size_t smem = (size_t)kmax * nbt * sizeof(float4);
    switch (nbt) {
      case 8: launch_contract_df<MODE, 8>(grid, smem, a, st); break;
      case 4: launch_contract_df<MODE, 4>(grid, smem, a, st); break;
      case 2: launch_contract_df<MODE, 2>(grid, smem, a, st); break;
      default: launch_contract_df<MODE, 1>(grid, smem, a, st); break;
    }
    S2G_LAUNCHED();
    return;
  }
  switch (nbt) {
  case 8: k_contract<MODE, 8><<<grid, CT_M, 0, st>>>(a); break;
  case 4: k_contract<MODE, 4><<<grid, CT_M, 0, st>>>(a); break;
  case 2: k_contract<MODE, 2><<<grid, CT_M, 0, st>>>(a); break;
  default: k_contract<MODE, 1><<<grid, CT_M, 0, st>>>(a); break;
  }
  S2G_LAUNCHED();
}

// maps per CTA: the largest power of two up to 8 that the batch fills, or the
// autotuned choice among those (per mode, band-limit bucket and batch bucket)
template <int MODE>
void launch_contract(const ContractArgs &a, int nm, int rows, cudaStream_t st) {
  static const int kCand[4] = {1, 2, 4, 8};
  const int ncand = a.nb >= 8 ? 4 : (a.nb >= 4 ? 3 : (a.nb >= 2 ? 2 : 1));
  const int c = tuned(TF_CONTRACT, MODE + 4 * t_precision, tune_bucket(a.bl), tune_bucket(a.nb), ncand, ncand - 1,
                      st, [&](int i) { launch_contract_nbt<MODE>(a, nm, rows, kCand[i], st); });
  double fl = 0, by = 0;
  if (timing_enabled()) contract_work(a, nm, &fl, &by);
  KTimer kt(KC_CONTRACT, st, fl, by);
  launch_contract_nbt<MODE>(a, nm, rows, kCand[c], st);
}

// two parts on one table (double-float kernel, split precision): columns =
// 2 parts x nb maps, one pass over the table
template <int MODE>
void launch_contract_df_pair(const ContractArgs &a, int nm, int rows, cudaStream_t st) {
  const int nbt = 2 * a.nb;
  const int kmax = a.bl > a.nt ? a.bl : a.nt;
  const size_t smem = (size_t)kmax * nbt * sizeof(float4);
  S2G_REQUIRE(a.nb >= 1 && a.nb <= 4 && smem <= kDfcSmemMax, ERR_UNSUPPORTED,
              "double-float contraction of two parts: at most 4 maps");
  double fl = 0, by = 0;
  if (timing_enabled()) {
    ContractArgs b = a;
    b.lmin = a.lmin2;
    double f1 = 0, b1 = 0, t1 = 0;
    contract_work(a, nm, &fl, &by);
    contract_work(b, nm, &f1, &b1, &t1);
    fl += f1;
    by += b1 - t1;  // the table is read once for both parts
  }
  KTimer kt(KC_CONTRACT, st, fl, by);
  const dim3 grid(nm, ceil_div(rows, CT_M), 1);
  switch (nbt) {
    case 8: launch_contract_df<MODE, 8>(grid, smem, a, st); break;
    case 4: launch_contract_df<MODE, 4>(grid, smem, a, st); break;
    default: launch_contract_df<MODE, 2>(grid, smem, a, st); break;
  }
  S2G_LAUNCHED();
}

// ---------------------------------------------------------------------------
// gamma DFTs
// ---------------------------------------------------------------------------

// e^{i n_k gamma_g} for all (g, k) of one call, gamma_g = 2 pi g / ng
constexpr int kMaxGammaTw = 512;

// NN = number of n values (compile time, so that the per-n values live in registers)
template <int NN>
__global__ void k_gamma_synth(const double2 *__restrict__ G, double2 *__restrict__ spec,
                              const int *__restrict__ ns, int ng, int bl, int nt, int nb, int real, double c) {
  __shared__ double2 tw[kMaxGammaTw];  // tw[g * NN + k]
  for (int i = threadIdx.x; i < ng * NN; i += blockDim.x) {
    const int g = i / NN, k = i % NN;
    double sn, cs;
    sincospi(2.0 * (double)((ns[k] * g) % ng) / (double)ng, &sn, &cs);
    tw[i] = make_double2(cs, sn);
  }
  __syncthreads();
  const int W = 2 * bl - 1;
  const int sw = real ? bl : W, smlo = real ? 0 : -(bl - 1);
  const int64_t total = (int64_t)nb * nt * sw;
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const int col = (int)(gid % sw);
  const int t = (int)((gid / sw) % nt);
  const int b = (int)(gid / ((int64_t)sw * nt));
  const int m = smlo + col;
  const int64_t gb = (int64_t)b * NN * nt * W;
  // real signals: the -n term is conj of G_n at -m, folded in as
  // e G_n(m) + conj(e) conj(G_n(-m)) = e.re (G + H) + i e.im (G - H),  H = conj(G_n(-m))
  double2 S[NN], D[NN];
#pragma unroll
  for (int k = 0; k < NN; ++k) {
    const double2 *Gk = G + gb + (int64_t)k * nt * W + (int64_t)t * W;
    const double2 gv = Gk[m + bl - 1];
    const double2 gm = (real && ns[k] > 0) ? conj2(Gk[-m + bl - 1]) : make_double2(0.0, 0.0);
    S[k] = add2(gv, gm);
    D[k] = sub2(gv, gm);
  }
  double2 *out = spec + (int64_t)b * ng * nt * sw + (int64_t)t * sw + col;
  for (int g = 0; g < ng; ++g) {
    double2 acc = make_double2(0.0, 0.0);
#pragma unroll
    for (int k = 0; k < NN; ++k) {
      const double2 e = tw[g * NN + k];
      // e.re * S + i e.im * D
      acc.x = fma(e.x, S[k].x, fma(-e.y, D[k].y, acc.x));
      acc.y = fma(e.x, S[k].y, fma(e.y, D[k].x, acc.y));
    }
    out[(int64_t)g * nt * sw] = scl2(acc, c);
  }
}

template <int NN>
__global__ void k_gamma_anal(const double2 *__restrict__ spec, double2 *__restrict__ G,
                             const int *__restrict__ ns, int ng, int bl, int nt, int nb, int real, double c) {
  __shared__ double2 tw[kMaxGammaTw];  // tw[g * NN + k] = e^{-i n_k gamma_g}
  for (int i = threadIdx.x; i < ng * NN; i += blockDim.x) {
    const int g = i / NN, k = i % NN;
    double sn, cs;
    sincospi(2.0 * (double)((ns[k] * g) % ng) / (double)ng, &sn, &cs);
    tw[i] = make_double2(cs, -sn);
  }
  __syncthreads();
  const int W = 2 * bl - 1;
  const int sw = real ? bl : W, smlo = real ? 0 : -(bl - 1);
  const int64_t total = (int64_t)nb * nt * W;
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= total) return;
  const int col = (int)(gid % W);
  const int t = (int)((gid / W) % nt);
  const int b = (int)(gid / ((int64_t)W * nt));
  const int m = col - (bl - 1);
  double2 acc[NN];
#pragma unroll
  for (int k = 0; k < NN; ++k) acc[k] = make_double2(0.0, 0.0);
  const double2 *sg = spec + (int64_t)b * ng * nt * sw + (int64_t)t * sw;
  for (int g = 0; g < ng; ++g, sg += (int64_t)nt * sw) {
    double2 s;
    if (real)
      s = m >= 0 ? sg[m] : conj2(sg[-m]);
    else
      s = sg[m - smlo];
#pragma unroll
    for (int k = 0; k < NN; ++k) {
      const double2 e = tw[g * NN + k];
      acc[k].x = fma(e.x, s.x, fma(-e.y, s.y, acc[k].x));
      acc[k].y = fma(e.x, s.y, fma(e.y, s.x, acc[k].y));
    }
  }
#pragma unroll
  for (int k = 0; k < NN; ++k) G[((int64_t)b * NN + k) * nt * W + (int64_t)t * W + col] = scl2(acc[k], c);
}

// gamma DFT on pixels: between the n-components F_n(t, p) (complex, one ring
// per (n, t)) and the gamma slices f_g(t, p) of the f_wav layout.  The phi DFT
// commutes with it, so the ring DFTs can run on the nn n-components instead of
// the ng = 2N-1 gamma slices.
//   synthesis: f_g = c sum_n e^{i n gamma_g} F_n  (real signals: n > 0 stand for
//              the +-n pair, 2 Re(e^{i n gamma_g} F_n); n = 0 adds Re F_0)
//   analysis:  F_n = c sum_g e^{-i n gamma_g} f_g
template <int NN>
__global__ void k_gamma_px_synth(const double2 *__restrict__ F, void *__restrict__ out, int64_t out_ms,
                                 const int *__restrict__ ns, int ng, int64_t npx, int nb, int real, double c) {
  __shared__ double2 tw[kMaxGammaTw];  // tw[g * NN + k] = e^{i n_k gamma_g} (x2 for n_k > 0, real)
  for (int i = threadIdx.x; i < ng * NN; i += blockDim.x) {
    const int g = i / NN, k = i % NN;
    double sn, cs;
    sincospi(2.0 * (double)((ns[k] * g) % ng) / (double)ng, &sn, &cs);
    const double f = (real && ns[k] != 0) ? 2.0 : 1.0;
    tw[i] = make_double2(f * cs, f * sn);
  }
  __syncthreads();
  const int64_t total = (int64_t)nb * npx;
  // grid-stride: a few blocks per SM, so the twiddle table above is built once per block
  for (int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; gid < total;
       gid += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(gid / npx);
    const int64_t px = gid - (int64_t)b * npx;
    double2 v[NN];
#pragma unroll
    for (int k = 0; k < NN; ++k) v[k] = F[((int64_t)b * NN + k) * npx + px];
    for (int g = 0; g < ng; ++g) {
      double re = 0.0, im = 0.0;
#pragma unroll
      for (int k = 0; k < NN; ++k) {
        const double2 e = tw[g * NN + k];
        re = fma(e.x, v[k].x, fma(-e.y, v[k].y, re));
        if (!real) im = fma(e.x, v[k].y, fma(e.y, v[k].x, im));
      }
      const int64_t o = (int64_t)b * out_ms + (int64_t)g * npx + px;
      if (real)
        ((double *)out)[o] = re * c;
      else
        ((double2 *)out)[o] = make_double2(re * c, im * c);
    }
  }
}

template <int NN>
__global__ void k_gamma_px_anal(const void *__restrict__ in, int64_t in_ms, double2 *__restrict__ F,
                                const int *__restrict__ ns, int ng, int64_t npx, int nb, int real, double c) {
  __shared__ double2 tw[kMaxGammaTw];  // tw[g * NN + k] = e^{-i n_k gamma_g}
  for (int i = threadIdx.x; i < ng * NN; i += blockDim.x) {
    const int g = i / NN, k = i % NN;
    double sn, cs;
    sincospi(2.0 * (double)((ns[k] * g) % ng) / (double)ng, &sn, &cs);
    tw[i] = make_double2(cs, -sn);
  }
  __syncthreads();
  const int64_t total = (int64_t)nb * npx;
  // grid-stride: a few blocks per SM, so the twiddle table above is built once per block
  for (int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; gid < total;
       gid += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(gid / npx);
    const int64_t px = gid - (int64_t)b * npx;
    double2 acc[NN];
#pragma unroll
    for (int k = 0; k < NN; ++k) acc[k] = make_double2(0.0, 0.0);
    if (real) {
      for (int g = 0; g < ng; ++g) {
        const double f = ((const double *)in)[(int64_t)b * in_ms + (int64_t)g * npx + px];
#pragma unroll
        for (int k = 0; k < NN; ++k) {
          const double2 e = tw[g * NN + k];
          acc[k].x = fma(e.x, f, acc[k].x);
          acc[k].y = fma(e.y, f, acc[k].y);
        }
      }
    } else {
      for (int g = 0; g < ng; ++g) {
        const double2 f = ((const double2 *)in)[(int64_t)b * in_ms + (int64_t)g * npx + px];
#pragma unroll
        for (int k = 0; k < NN; ++k) {
          const double2 e = tw[g * NN + k];
          acc[k].x = fma(e.x, f.x, fma(-e.y, f.y, acc[k].x));
          acc[k].y = fma(e.x, f.y, fma(e.y, f.x, acc[k].y));
        }
      }
    }
#pragma unroll
    for (int k = 0; k < NN; ++k) F[((int64_t)b * NN + k) * npx + px] = scl2(acc[k], c);
  }
}

// The same gamma DFTs in double-float arithmetic on the FP32 pipe (split-
// precision path): each pixel's inputs are rescaled by a power of two taken
// from their largest exponent field, the twiddles (times the normalisation c,
// times 2 for the real +-n pairs) are double-float constants, and each output
// costs one FP64 add to widen.

template <int NN>
__global__ void k_gamma_px_synth_df(const double2 *__restrict__ F, void *__restrict__ out, int64_t out_ms,
                                    const int *__restrict__ ns, int ng, int64_t npx, int nb, int real, double c) {
  __shared__ float4 tw[kMaxGammaTw];  // c e^{i n_k gamma_g} (x2 for n_k > 0, real)
  for (int i = threadIdx.x; i < ng * NN; i += blockDim.x) {
    const int g = i / NN, k = i % NN;
    double sn, cs;
    sincospi(2.0 * (double)((ns[k] * g) % ng) / (double)ng, &sn, &cs);
    const double f = ((real && ns[k] != 0) ? 2.0 : 1.0) * c;
    float2 re, im;
    split_scaled(f * cs, 0, re.x, re.y);
    split_scaled(f * sn, 0, im.x, im.y);
    tw[i] = dmk(re, im);
  }
  __syncthreads();
  const int64_t total = (int64_t)nb * npx;
  // grid-stride: a few blocks per SM, so the twiddle table above is built once per block
  for (int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; gid < total;
       gid += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(gid / npx);
    const int64_t px = gid - (int64_t)b * npx;
    double2 v[NN];
    int em = 0;
#pragma unroll
    for (int k = 0; k < NN; ++k) {
      v[k] = F[((int64_t)b * NN + k) * npx + px];
      em = max(em, max(exp_field(v[k].x), exp_field(v[k].y)));
    }
    const int e = block_scale(em);
    float4 z[NN];
#pragma unroll
    for (int k = 0; k < NN; ++k) z[k] = dc_split(v[k], e);
    for (int g = 0; g < ng; ++g) {
      float2 re = make_float2(0.f, 0.f), im = make_float2(0.f, 0.f);
#pragma unroll
      for (int k = 0; k < NN; ++k) {
        const float4 w = tw[g * NN + k];
        re = df_add(re, df_dot2(dre(w), dre(z[k]), df_neg(dim_(w)), dim_(z[k])));
        if (!real) im = df_add(im, df_dot2(dre(w), dim_(z[k]), dim_(w), dre(z[k])));
      }
      const int64_t o = (int64_t)b * out_ms + (int64_t)g * npx + px;
      if (real)
        ((double *)out)[o] = join_scaled(re.x, re.y, e);
      else
        ((double2 *)out)[o] = make_double2(join_scaled(re.x, re.y, e), join_scaled(im.x, im.y, e));
    }
  }
}

template <int NN>
__global__ void k_gamma_px_anal_df(const void *__restrict__ in, int64_t in_ms, double2 *__restrict__ F,
                                   const int *__restrict__ ns, int ng, int64_t npx, int nb, int real, double c) {
  __shared__ float4 tw[kMaxGammaTw];  // c e^{-i n_k gamma_g}
  for (int i = threadIdx.x; i < ng * NN; i += blockDim.x) {
    const int g = i / NN, k = i % NN;
    double sn, cs;
    sincospi(2.0 * (double)((ns[k] * g) % ng) / (double)ng, &sn, &cs);
    float2 re, im;
    split_scaled(c * cs, 0, re.x, re.y);
    split_scaled(-c * sn, 0, im.x, im.y);
    tw[i] = dmk(re, im);
  }
  __syncthreads();
  const int64_t total = (int64_t)nb * npx;
  // grid-stride: a few blocks per SM, so the twiddle table above is built once per block
  for (int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; gid < total;
       gid += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(gid / npx);
    const int64_t px = gid - (int64_t)b * npx;
    float4 acc[NN];
#pragma unroll
    for (int k = 0; k < NN; ++k) acc[k] = make_float4(0.f, 0.f, 0.f, 0.f);
    const int64_t base = (int64_t)b * in_ms + px;
    int em = 0;
    for (int g = 0; g < ng; ++g) {
      if (real) {
        em = max(em, exp_field(((const double *)in)[base + (int64_t)g * npx]));
      } else {
        const double2 f = ((const double2 *)in)[base + (int64_t)g * npx];
        em = max(em, max(exp_field(f.x), exp_field(f.y)));
      }
    }
    const int e = block_scale(em);
    for (int g = 0; g < ng; ++g) {
      if (real) {
        const float2 f = df_split(((const double *)in)[base + (int64_t)g * npx], e);
#pragma unroll
        for (int k = 0; k < NN; ++k) {
          const float4 w = tw[g * NN + k];
          acc[k] = dmk(df_add(dre(acc[k]), df_mul(dre(w), f)), df_add(dim_(acc[k]), df_mul(dim_(w), f)));
        }
      } else {
        const float4 f = dc_split(((const double2 *)in)[base + (int64_t)g * npx], e);
#pragma unroll
        for (int k = 0; k < NN; ++k) acc[k] = dc_add(acc[k], dc_mul(tw[g * NN + k], f));
      }
    }
#pragma unroll
    for (int k = 0; k < NN; ++k) F[((int64_t)b * NN + k) * npx + px] = dc_to(acc[k], e);
  }
}

// ---------------------------------------------------------------------------
// Ring DFTs and gamma DFT in one launch (split-precision path)
//
// The n-components F_k(t, p) (k < NN) of one theta-ring are transformed by a
// thread-block cluster of NN CTAs, one per component, each with the padded
// Bluestein buffer of the single-ring kernels (3 CTAs per SM, as there).  The
// gamma DFT exchanges values between the components of a pixel through
// distributed shared memory, so the n-components never go to HBM:
//   synthesis: each CTA runs the inverse ring DFT of its component and leaves
//              F_k(p) (double-float) in its buffer; after a cluster barrier
//              each CTA computes the gamma slices f_g(p) of its share of the
//              pixels from all NN buffers and writes them to f_wav.
//   analysis:  each CTA reads the gamma slices of its share of the pixels,
//              forms every component F_k(p), premultiplies by the chirp and
//              stores it into CTA k's buffer; after a cluster barrier each CTA
//              runs the forward ring DFT of its component and writes its
//              spectrum.
// One power-of-two scale per ring, the largest over the cluster (exchanged
// through shared memory before the transforms), so the components combine
// without rescaling.
// ---------------------------------------------------------------------------

__device__ __forceinline__ int cluster_max_int(cg::cluster_group &cl, int *slot, int v, int nn) {
  const int m = block_max_int(v);
  if (threadIdx.x == 0) *slot = m;
  cl.sync();
  int r = 0;
  for (int j = 0; j < nn; ++j) r = max(r, *cl.map_shared_rank(slot, j));
  return r;
}

template <int NN, bool REAL>
__global__ void __launch_bounds__(512, 3) k_ring_inverse_gamma_df(RingArgs a, GammaFuse gf) {
  extern __shared__ float4 bufd[];
  __shared__ int s_em, s_e;
  cg::cluster_group cl = cg::this_cluster();
  const int k = (int)cl.block_rank();
  const int r = blockIdx.x / NN;
  const int b = r / gf.nt, t = r - b * gf.nt;
  const int K = a.K, P = a.P, logP = a.logP, bl = a.bl;
  const bool herm = (k == gf.herm_k);
  const int sw = herm ? bl : gf.W, mlo = herm ? 0 : -(bl - 1);
  const double2 *s0 = gf.G + (int64_t)b * gf.gms + (int64_t)k * gf.gks + (int64_t)t * gf.W + (herm ? bl - 1 : 0);
  int em = 0;
  for (int c = threadIdx.x; c < sw; c += blockDim.x) em = emax2(em, s0[c]);
  const int e = block_scale(cluster_max_int(cl, &s_em, em, NN));
  if (threadIdx.x == 0) s_e = e;  // read back after the transforms: fewer live registers in them
  for (int j = threadIdx.x; j < P; j += blockDim.x) {
    float4 zz = make_float4(0.f, 0.f, 0.f, 0.f);
    if (j < K) {
      const int m = (j < bl) ? j : j - K;
      const int c = m - mlo;
      if (c >= 0 && c < sw)
        zz = dc_split(s0[c], e);
      else if (herm && m < 0 && -m < sw)
        zz = dc_conj(dc_split(s0[-m], e));
      zz = dc_conj(dc_mul(zz, ld_once(&a.chirp_df[j])));
    }
    bufd[slot_brev(j, logP)] = zz;
  }
  __syncthreads();
  fft_dit_df(bufd, a.tw_df, P, logP);
  kernel_multiply_df(bufd, a.bhat_df, P, logP);
  ifft_dif_df(bufd, a.tw_df, P, logP);
  // F_k(p) = c_p conj(y_p), in place (p -> brev(p) is one-to-one)
  for (int p = threadIdx.x; p < K; p += blockDim.x) {
    const int i = slot_brev(p, logP);
    bufd[i] = dc_mul(ld_once(&a.chirp_df[p]), dc_conj(bufd[i]));
  }
  cl.sync();
  // gamma slices of this CTA's share of the pixels
  const int eo = s_e - logP;
  const int kk = (int)cl.block_rank(), rr = blockIdx.x / NN;
  const int bb = rr / gf.nt, tt = rr - bb * gf.nt;
  const int chunk = (K + NN - 1) / NN;
  const int p1 = min(K, (kk + 1) * chunk);
  const int64_t obase = (int64_t)bb * gf.fms + (int64_t)tt * K;
  // gamma_g and gamma_{ng-g} have conjugate twiddles: with w = C + i S,
  //   real:    f_g = A - B, f_{ng-g} = A + B, A = sum_k C Re z_k, B = sum_k S Im z_k
  //   complex: f_g = U + i V, f_{ng-g} = U - i V, U = sum_k C z_k, V = sum_k S z_k
  for (int p = kk * chunk + threadIdx.x; p < p1; p += blockDim.x) {
    const int i = slot_brev(p, logP);
    float4 z[NN];
#pragma unroll
    for (int j = 0; j < NN; ++j) z[j] = *cl.map_shared_rank(bufd + i, j);
    for (int g = 0; 2 * g <= gf.ng; ++g) {
      const int g2 = gf.ng - g;  // the conjugate partner (g = 0 and g2 == g have none)
      const int64_t o = obase + (int64_t)g * gf.npx + p, o2 = obase + (int64_t)g2 * gf.npx + p;
      const bool pair = g > 0 && g2 != g;
      if (REAL) {
        float2 A = make_float2(0.f, 0.f), B = make_float2(0.f, 0.f);
#pragma unroll
        for (int j = 0; j < NN; ++j) {
          const float4 w = gf.tw[g * NN + j];
          A = df_add(A, df_mul(dre(w), dre(z[j])));
          B = df_add(B, df_mul(dim_(w), dim_(z[j])));
        }
        const float2 f1 = df_add(A, df_neg(B));
        ((double *)gf.fw)[o] = join_scaled(f1.x, f1.y, eo);
        if (pair) {
          const float2 f2 = df_add(A, B);
          ((double *)gf.fw)[o2] = join_scaled(f2.x, f2.y, eo);
        }
      } else {
        float4 U = make_float4(0.f, 0.f, 0.f, 0.f), V = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int j = 0; j < NN; ++j) {
          const float4 w = gf.tw[g * NN + j];
          U = dmk(df_add(dre(U), df_mul(dre(w), dre(z[j]))), df_add(dim_(U), df_mul(dre(w), dim_(z[j]))));
          V = dmk(df_add(dre(V), df_mul(dim_(w), dre(z[j]))), df_add(dim_(V), df_mul(dim_(w), dim_(z[j]))));
        }
        const float4 iV = dc_mul_pi(V);
        const float4 f1 = dc_add(U, iV);
        ((double2 *)gf.fw)[o] = dc_to(f1, eo);
        if (pair) ((double2 *)gf.fw)[o2] = dc_to(dc_sub(U, iV), eo);
      }
    }
  }
  cl.sync();  // peers read this buffer until here
}

template <int NN, bool REAL>
__global__ void __launch_bounds__(512, 3) k_gamma_ring_forward_df(RingArgs a, GammaFuse gf) {
  extern __shared__ float4 bufd[];
  __shared__ int s_em, s_e;
  cg::cluster_group cl = cg::this_cluster();
  const int k = (int)cl.block_rank();
  const int r = blockIdx.x / NN;
  const int b = r / gf.nt, t = r - b * gf.nt;
  const int K = a.K, P = a.P, logP = a.logP;
  const int chunk = (K + NN - 1) / NN;
  const int p0 = k * chunk, p1 = min(K, p0 + chunk);
  const int64_t ibase = (int64_t)b * gf.fms + (int64_t)t * K;
  int em = 0;
  for (int p = p0 + threadIdx.x; p < p1; p += blockDim.x)
    for (int g = 0; g < gf.ng; ++g) {
      const int64_t o = ibase + (int64_t)g * gf.npx + p;
      if (REAL)
        em = max(em, exp_field(((const double *)gf.fw)[o]));
      else
        em = emax2(em, ((const double2 *)gf.fw)[o]);
    }
  const int e = block_scale(cluster_max_int(cl, &s_em, em, NN));
  if (threadIdx.x == 0) s_e = e;  // read back after the transforms: fewer live registers in them
  // the zero padding of this CTA's own buffer
  for (int j = K + threadIdx.x; j < P; j += blockDim.x) bufd[slot_brev(j, logP)] = make_float4(0.f, 0.f, 0.f, 0.f);
  // gamma_g and gamma_{ng-g} have conjugate twiddles w = C + i S and C - i S:
  // each pair contributes C (f_g + f_{ng-g}) + i S (f_g - f_{ng-g})
  for (int p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
    float4 acc[NN];
#pragma unroll
    for (int j = 0; j < NN; ++j) acc[j] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int g = 0; 2 * g <= gf.ng; ++g) {
      const int g2 = gf.ng - g;
      const bool pair = g > 0 && g2 != g;
      const int64_t o = ibase + (int64_t)g * gf.npx + p, o2 = ibase + (int64_t)g2 * gf.npx + p;
      if (REAL) {
        const float2 fa = df_split(((const double *)gf.fw)[o], e);
        const float2 fb = pair ? df_split(((const double *)gf.fw)[o2], e) : make_float2(0.f, 0.f);
        const float2 Pp = df_add(fa, fb), Q = df_add(fa, df_neg(fb));
#pragma unroll
        for (int j = 0; j < NN; ++j) {
          const float4 w = gf.tw[g * NN + j];
          acc[j] = dmk(df_add(dre(acc[j]), df_mul(dre(w), Pp)), df_add(dim_(acc[j]), df_mul(dim_(w), Q)));
        }
      } else {
        const float4 fa = dc_split(((const double2 *)gf.fw)[o], e);
        const float4 fb = pair ? dc_split(((const double2 *)gf.fw)[o2], e) : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 Pp = dc_add(fa, fb), Q = dc_sub(fa, fb);
#pragma unroll
        for (int j = 0; j < NN; ++j) {
          const float4 w = gf.tw[g * NN + j];
          // C P + i S Q
          const float2 re = df_add(df_mul(dre(w), dre(Pp)), df_neg(df_mul(dim_(w), dim_(Q))));
          const float2 im = df_add(df_mul(dre(w), dim_(Pp)), df_mul(dim_(w), dre(Q)));
          acc[j] = dc_add(acc[j], dmk(re, im));
        }
      }
    }
    const float4 ch = ld_once(&a.chirp_df[p]);
    const int i = slot_brev(p, logP);
#pragma unroll
    for (int j = 0; j < NN; ++j) *cl.map_shared_rank(bufd + i, j) = dc_mulc(acc[j], ch);
  }
  cl.sync();  // every component's buffer is complete
  fft_dit_df(bufd, a.tw_df, P, logP);
  kernel_multiply_df(bufd, a.bhat_df, P, logP);
  ifft_dif_df(bufd, a.tw_df, P, logP);
  const int eo = s_e - logP;
  const int kk = (int)cl.block_rank(), rr = blockIdx.x / NN;
  const int bb = rr / gf.nt, tt = rr - bb * gf.nt;
  double2 *out = gf.Gout + (int64_t)bb * gf.gms + (int64_t)kk * gf.gks + (int64_t)tt * gf.W;
  for (int c = threadIdx.x; c < gf.W; c += blockDim.x) {
    const int m = c - (a.bl - 1);
    const int q = ((m % K) + K) % K;
    out[c] = dc_to(dc_mulc(bufd[slot_brev(q, logP)], ld_once(&a.chirp_df[q])), eo);
  }
}

// ---------------------------------------------------------------------------
// lmn -> lm merge
// ---------------------------------------------------------------------------

__global__ void k_merge(double2 *__restrict__ flm, int L, int64_t fs, const double2 *__restrict__ z,
                        int64_t zs, const MergePair *__restrict__ pairs, int npairs,
                        const double2 *__restrict__ wts, const double2 *__restrict__ zscal, int64_t zss,
                        int bl_scal, int real, int accumulate, int nb) {
  const int64_t L2 = (int64_t)L * L;
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= nb * L2) return;
  const int b = (int)(gid / L2);
  const int i = (int)(gid % L2);
  int l2 = (int)sqrt((double)i);
  while (l2 * l2 > i) --l2;
  while ((l2 + 1) * (l2 + 1) <= i) ++l2;
  const int m = i - l2 * l2 - l2;
  if (real && m < 0) return;
  double2 acc = accumulate ? flm[(int64_t)b * fs + i] : make_double2(0.0, 0.0);
  const double2 *zb = z + (int64_t)b * zs;
  for (int p = 0; p < npairs; ++p) {
    const MergePair pr = pairs[p];
    if (l2 >= pr.bl || l2 < pr.lmin) continue;
    const int an = pr.n < 0 ? -pr.n : pr.n;
    if (l2 < an) continue;
    const double2 *zp = zb + pr.off;
    const int64_t li = (int64_t)l2 * l2 + l2;
    acc = add2(acc, cmul(wts[pr.woff + l2], zp[li + m]));
    if (real && pr.n > 0) {
      double2 v = cmul(conj2(zp[li - m]), wts[pr.woff + pr.bl + l2]);
      if ((m + pr.n) & 1) v = scl2(v, -1.0);
      acc = add2(acc, v);
    }
  }
  if (zscal && l2 < bl_scal) acc = add2(acc, zscal[(int64_t)b * zss + i]);
  flm[(int64_t)b * fs + i] = acc;
}

__global__ void k_symmetrize(double2 *flm, int L, int64_t fs, int nb) {
  const int64_t L2 = (int64_t)L * L;
  const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= nb * L2) return;
  const int b = (int)(gid / L2);
  const int i = (int)(gid % L2);
  int l = (int)sqrt((double)i);
  while (l * l > i) --l;
  while ((l + 1) * (l + 1) <= i) ++l;
  const int m = i - l * l - l;
  if (m <= 0) return;
  double2 v = conj2(flm[(int64_t)b * fs + i]);
  if (m & 1) v = scl2(v, -1.0);
  flm[(int64_t)b * fs + l * l + l - m] = v;
}

// FP32 storage: `rows` rows of n values, row r at src + r ss and dst + r ds
// (elements); widening is exact, narrowing rounds to nearest.
__global__ void k_widen_rows(const float *__restrict__ src, int64_t ss, double *__restrict__ dst, int64_t ds,
                             int64_t n, int rows) {
  const int64_t total = (int64_t)rows * n;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / n, c = i - r * n;
    dst[r * ds + c] = (double)src[r * ss + c];
  }
}
__global__ void k_narrow_rows(const double *__restrict__ src, int64_t ss, float *__restrict__ dst, int64_t ds,
                              int64_t n, int rows) {
  const int64_t total = (int64_t)rows * n;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = i / n, c = i - r * n;
    dst[r * ds + c] = __double2float_rn(src[r * ss + c]);
  }
}

__global__ void k_scale_copy(const double *x, double *y, int64_t n, double s) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = x[i] * s;
}

// y[b * ys + i] = a x[b * xs + i] + c y[b * ys + i], i < n, b < nb
__global__ void k_axpby(const double *x, int64_t xs, double *y, int64_t ys, int64_t n, int nb, double a, double c) {
  const int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n * nb) return;
  const int64_t b = g / n, i = g - b * n;
  y[b * ys + i] = fma(a, x[b * xs + i], c * y[b * ys + i]);
}

}  // namespace

// ===========================================================================
// wrappers
// ===========================================================================

namespace {

// Shared memory of the ring kernels: one P-point buffer of 16-byte values.
// The double-float kernels (3 CTAs per SM) ask for a carveout just large
// enough for three buffers, so that the rest of the SM's L1 keeps the twiddle
// table (32 KB at P = 4096).
void ring_smem_attrs(const void *kernel, size_t smem, bool df) {
  if (smem > 48 * 1024) S2G_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (df) {
    constexpr double kMaxSmemPerSm = 228.0 * 1024.0;
    const int pct = std::min(100, (int)std::ceil(100.0 * 3.0 * (double)(smem + 2048) / kMaxSmemPerSm) + 1);
    S2G_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, pct));
  }
}

template <class KF>
void launch_ring(KF kernel, const RingArgs &a, int nblk, int P, cudaStream_t st, bool df = false) {
  const size_t smem = sizeof(double2) * (size_t)P;
  ring_smem_attrs((const void *)kernel, smem, df);
  kernel<<<nblk, ring_threads(P), smem, st>>>(a);
  S2G_LAUNCHED();
}

// Work model of one Bluestein transform of padded length P (for the timing
// report): the split path counts double-float FP32 instructions (32 per
// element per radix-2 stage and FFT with unnormalised adds of 8 and complex
// multiplies of 32 instructions, less the pruned first and last passes; 32
// for the kernel-spectrum multiply and 64 K / P for the two chirps); the FP64
// path counts 5 P log2 P flop per FFT.
double ring_work(const RingArgs &a, int nblk) {
  const double P = a.P, lg = a.logP;
  if (t_precision == 1) return (double)nblk * P * (64.0 * lg - 56.0 + 64.0 * a.K / P);
  return (double)nblk * (10.0 * P * lg + 6.0 * P + 12.0 * a.K);
}

void run_ring_forward(const RingArgs &a, int nrings, bool real, cudaStream_t st) {
  const int nblk = real ? (nrings + 1) / 2 : nrings;
  KTimer kt(KC_RING, st, timing_enabled() ? ring_work(a, nblk) : 0.0,
            (double)nrings * a.K * (real ? 8.0 : 16.0) + (double)nrings * a.sw * 16.0);
  if (t_precision == 1) {
    if (real)
      launch_ring(k_ring_forward_df<true>, a, nblk, a.P, st, true);
    else
      launch_ring(k_ring_forward_df<false>, a, nblk, a.P, st, true);
  } else if (real) {
    launch_ring(k_ring_forward<true>, a, nblk, a.P, st);
  } else {
    launch_ring(k_ring_forward<false>, a, nblk, a.P, st);
  }
}

void run_ring_inverse(const RingArgs &a, int nrings, bool real, cudaStream_t st) {
  const int nblk = real ? (nrings + 1) / 2 : nrings;
  KTimer kt(KC_RING, st, timing_enabled() ? ring_work(a, nblk) : 0.0,
            (double)nrings * a.K * (real ? 8.0 : 16.0) + (double)nrings * a.sw * 16.0);
  if (t_precision == 1) {
    if (real)
      launch_ring(k_ring_inverse_df<true>, a, nblk, a.P, st, true);
    else
      launch_ring(k_ring_inverse_df<false>, a, nblk, a.P, st, true);
  } else if (real) {
    launch_ring(k_ring_inverse<true>, a, nblk, a.P, st);
  } else {
    launch_ring(k_ring_inverse<false>, a, nblk, a.P, st);
  }
}

// Twiddles of the fused gamma DFT: synthesis c e^{i n_k gamma_g} (x2 for
// n_k != 0 on real signals, which stand for the +-n pair), analysis
// c e^{-i n_k gamma_g}; gamma_g = 2 pi g / ng, as double-float pairs.
void fuse_twiddles(GammaFuse &gf, const std::vector<int> &ns, int ng, bool real, double c, bool synth) {
  const int nn = (int)ns.size();
  for (int g = 0; g < ng; ++g)
    for (int k = 0; k < nn; ++k) {
      const long double x = 2.0L * (long double)((ns[k] * g) % ng) / (long double)ng;  // angle / pi
      const long double pi = 3.141592653589793238462643383279502884L;
      const double f = synth ? ((real && ns[k] != 0) ? 2.0 * c : c) : c;
      const double re = (double)(f * cosl(pi * x)), im = (double)((synth ? f : -f) * sinl(pi * x));
      const float rh = (float)re, ih = (float)im;
      gf.tw[g * nn + k] = make_float4(rh, (float)(re - (double)rh), ih, (float)(im - (double)ih));
    }
}

template <class KF>
void launch_fused(KF kernel, const RingArgs &a, const GammaFuse &gf, int nrings, int nn, cudaStream_t st) {
  const size_t smem = sizeof(float4) * (size_t)a.P;
  ring_smem_attrs((const void *)kernel, smem, true);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(nrings * nn));
  cfg.blockDim = dim3(ring_threads(a.P));
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)nn;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  S2G_CUDA(cudaLaunchKernelEx(&cfg, kernel, a, gf));
  S2G_LAUNCHED();
}

}  // namespace

namespace {
// Whether a cluster of nn CTAs of the fused kernels (P-point buffers) can be
// resident on this GPU: asked once per (nn, P) of the device in use.
bool cluster_fits(int nn, int P) {
  static std::mutex mu;
  static std::map<std::pair<int, int>, bool> known;
  std::lock_guard<std::mutex> lk(mu);
  const auto key = std::make_pair(nn, P);
  auto it = known.find(key);
  if (it != known.end()) return it->second;
  const void *kern = nullptr;
  switch (nn) {
    case 2: kern = (const void *)k_ring_inverse_gamma_df<2, false>; break;
    case 3: kern = (const void *)k_ring_inverse_gamma_df<3, false>; break;
    case 4: kern = (const void *)k_ring_inverse_gamma_df<4, false>; break;
    case 5: kern = (const void *)k_ring_inverse_gamma_df<5, false>; break;
    case 6: kern = (const void *)k_ring_inverse_gamma_df<6, false>; break;
    case 7: kern = (const void *)k_ring_inverse_gamma_df<7, false>; break;
    default: kern = (const void *)k_ring_inverse_gamma_df<8, false>; break;
  }
  const size_t smem = sizeof(float4) * (size_t)P;
  ring_smem_attrs(kern, smem, true);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)nn);
  cfg.blockDim = dim3(ring_threads(P));
  cfg.dynamicSmemBytes = smem;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)nn;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int nclusters = 0;
  const cudaError_t e = cudaOccupancyMaxActiveClusters(&nclusters, kern, &cfg);
  if (e != cudaSuccess) cudaGetLastError();  // a refusal only means: not fusable here
  const bool ok = e == cudaSuccess && nclusters > 0;
  known[key] = ok;
  return ok;
}
}  // namespace

bool ring_gamma_fusable(int nn, int ng, int bl, int ss) {
  if (t_precision != 1 || nn < 2 || nn > kFuseMaxNN || ng * nn > kFuseMaxTw) return false;
  return cluster_fits(nn, ring_fft(grid_ring_len(bl, ss)).P);
}

void ring_inverse_gamma(const double2 *G, int64_t gms, int64_t gks, const std::vector<int> &ns, int ng, bool real,
                        double c, void *fw, int64_t fms, int nb, int bl, int ss, cudaStream_t st) {
  const int nn = (int)ns.size();
  S2G_REQUIRE(ring_gamma_fusable(nn, ng, bl, ss), ERR_UNSUPPORTED, "fused ring/gamma DFT: unsupported shape");
  const int nt = grid_rings(bl, ss), nrings = nb * nt;
  if (nrings <= 0) return;
  const RingFFT &rf = ring_fft(grid_ring_len(bl, ss));
  RingArgs a = ring_args(rf, bl, nrings);
  GammaFuse gf{};
  gf.G = G;
  gf.gms = gms;
  gf.gks = gks;
  gf.W = 2 * bl - 1;
  gf.nt = nt;
  gf.herm_k = -1;
  for (int k = 0; k < nn; ++k)
    if (real && ns[k] == 0) gf.herm_k = k;
  gf.fw = fw;
  gf.fms = fms;
  gf.npx = (int64_t)nt * a.K;
  gf.ng = ng;
  gf.real = real ? 1 : 0;
  fuse_twiddles(gf, ns, ng, real, c, true);
  const double px = (double)nrings * a.K;
  KTimer kt(KC_RING, st, timing_enabled() ? ring_work(a, nrings * nn) + px * ng * nn * (real ? 24.0 : 48.0) : 0.0,
            (double)nrings * nn * gf.W * 16.0 + px * ng * (real ? 8.0 : 16.0));
  switch (nn) {
#define S2G_FUSE(N)                                                              \
  case N:                                                                        \
    if (real)                                                                    \
      launch_fused(k_ring_inverse_gamma_df<N, true>, a, gf, nrings, N, st);     \
    else                                                                         \
      launch_fused(k_ring_inverse_gamma_df<N, false>, a, gf, nrings, N, st);    \
    break;
    S2G_FUSE(2) S2G_FUSE(3) S2G_FUSE(4) S2G_FUSE(5) S2G_FUSE(6) S2G_FUSE(7) S2G_FUSE(8)
#undef S2G_FUSE
    default: break;
  }
}

void gamma_ring_forward(const void *fw, int64_t fms, const std::vector<int> &ns, int ng, bool real, double c,
                        double2 *Gout, int64_t gms, int64_t gks, int nb, int bl, int ss, cudaStream_t st) {
  const int nn = (int)ns.size();
  S2G_REQUIRE(ring_gamma_fusable(nn, ng, bl, ss), ERR_UNSUPPORTED, "fused ring/gamma DFT: unsupported shape");
  const int nt = grid_rings(bl, ss), nrings = nb * nt;
  if (nrings <= 0) return;
  const RingFFT &rf = ring_fft(grid_ring_len(bl, ss));
  RingArgs a = ring_args(rf, bl, nrings);
  GammaFuse gf{};
  gf.Gout = Gout;
  gf.gms = gms;
  gf.gks = gks;
  gf.W = 2 * bl - 1;
  gf.nt = nt;
  gf.herm_k = -1;
  gf.fw = const_cast<void *>(fw);
  gf.fms = fms;
  gf.npx = (int64_t)nt * a.K;
  gf.ng = ng;
  gf.real = real ? 1 : 0;
  fuse_twiddles(gf, ns, ng, real, c, false);
  const double px = (double)nrings * a.K;
  KTimer kt(KC_RING, st, timing_enabled() ? ring_work(a, nrings * nn) + px * ng * nn * (real ? 24.0 : 48.0) : 0.0,
            (double)nrings * nn * gf.W * 16.0 + px * ng * (real ? 8.0 : 16.0));
  switch (nn) {
#define S2G_FUSE(N)                                                              \
  case N:                                                                        \
    if (real)                                                                    \
      launch_fused(k_gamma_ring_forward_df<N, true>, a, gf, nrings, N, st);     \
    else                                                                         \
      launch_fused(k_gamma_ring_forward_df<N, false>, a, gf, nrings, N, st);    \
    break;
    S2G_FUSE(2) S2G_FUSE(3) S2G_FUSE(4) S2G_FUSE(5) S2G_FUSE(6) S2G_FUSE(7) S2G_FUSE(8)
#undef S2G_FUSE
    default: break;
  }
}

namespace {

}  // namespace

void ring_forward(const void *rings, int64_t ring_stride, int64_t map_stride, int rpm, double2 *spec,
                  int64_t spec_stride, int sw, int mlo, int nrings, int bl, int ss, bool real, cudaStream_t st) {
  if (nrings <= 0) return;
  const RingFFT &rf = ring_fft(grid_ring_len(bl, ss));
  RingArgs a = ring_args(rf, bl, nrings);
  a.rings = rings;
  a.ring_stride = ring_stride;
  a.map_stride = map_stride;
  a.rpm = rpm;
  a.spec_out = spec;
  a.spec_stride = spec_stride;
  a.sw = sw;
  a.mlo = mlo;
  run_ring_forward(a, nrings, real, st);
}

void ring_inverse(const double2 *spec, int64_t spec_stride, int sw, int mlo, void *rings,
                  int64_t ring_stride, int64_t map_stride, int rpm, int nrings, int bl, int ss, bool real,
                  cudaStream_t st) {
  if (nrings <= 0) return;
  const RingFFT &rf = ring_fft(grid_ring_len(bl, ss));
  RingArgs a = ring_args(rf, bl, nrings);
  a.spec_in = spec;
  a.spec_stride = spec_stride;
  a.sw = sw;
  a.mlo = mlo;
  a.rings_out = (double2 *)rings;
  a.ring_stride = ring_stride;
  a.map_stride = map_stride;
  a.rpm = rpm;
  run_ring_inverse(a, nrings, real, st);
}

void ring_forward_c(const double2 *rings, int64_t ring_stride, int64_t map_stride, int rpm, double2 *spec,
                    int64_t spec_stride, int64_t spec_map_stride, int spec_rpm, int sw, int mlo, int nrings, int bl,
                    int ss, cudaStream_t st) {
  if (nrings <= 0) return;
  const RingFFT &rf = ring_fft(grid_ring_len(bl, ss));
  RingArgs a = ring_args(rf, bl, nrings);
  a.rings = rings;
  a.ring_stride = ring_stride;
  a.map_stride = map_stride;
  a.rpm = rpm;
  a.spec_out = spec;
  a.spec_stride = spec_stride;
  a.spec_map_stride = spec_map_stride;
  a.spec_rpm = spec_rpm;
  a.sw = sw;
  a.mlo = mlo;
  run_ring_forward(a, nrings, false, st);
}

void ring_inverse_c(const double2 *spec, int64_t spec_stride, int64_t spec_map_stride, int spec_rpm, int sw,
                    int mlo, bool herm, double2 *rings, int64_t ring_stride, int64_t map_stride, int rpm, int nrings,
                    int bl, int ss, cudaStream_t st) {
  if (nrings <= 0) return;
  const RingFFT &rf = ring_fft(grid_ring_len(bl, ss));
  RingArgs a = ring_args(rf, bl, nrings);
  a.spec_in = spec;
  a.spec_stride = spec_stride;
  a.spec_map_stride = spec_map_stride;
  a.spec_rpm = spec_rpm;
  a.herm = herm ? 1 : 0;
  a.sw = sw;
  a.mlo = mlo;
  a.rings_out = rings;
  a.ring_stride = ring_stride;
  a.map_stride = map_stride;
  a.rpm = rpm;
  run_ring_inverse(a, nrings, false, st);
}

void release_df_tables() {
  std::lock_guard<std::mutex> lk(g_dft_mu);
  for (auto &kv : g_dft) cudaFree(kv.second);
  g_dft.clear();
  g_dft_bytes = 0;
}
size_t df_table_bytes() {
  std::lock_guard<std::mutex> lk(g_dft_mu);
  return g_dft_bytes;
}
void set_split_tables(int on) { g_split_tables.store(on ? 1 : 0); }
int get_split_tables() { return g_split_tables.load(); }
void set_df_max_maps(int maps) { g_df_max_maps.store(maps); }
int get_df_max_maps() { return g_df_max_maps.load(); }

void contract_l2t(const L2T &p, cudaStream_t st) {
  if (p.nb <= 0 || p.mhi < p.mlo) return;
  if (p.tb->rc) {
    contract_l2t_rc(p, st);
    return;
  }
  if (t_precision == 1 && p.nb > df_max_maps() && contract_l2t_mixed(&p, 1, st)) return;
  ContractArgs a{};
  a.table = p.use_q ? p.tb->Q : p.tb->D;
  if (t_precision == 1) a.table_df = df_table(*p.tb, p.use_q, st);
  a.off = p.tb->d_off;
  a.bl = p.tb->bl;
  a.nt = p.tb->nt;
  a.an = p.tb->an;
  a.tmlo = p.tb->mlo;
  a.n = p.n;
  a.mlo = p.mlo;
  a.lmin = p.lmin;
  a.w = p.w;
  a.wscale = p.wscale;
  a.wconj = p.wconj;
  a.src = p.x;
  a.ss = p.xs;
  a.sw_or_xL = p.xL;
  a.x_half = p.x_half;
  a.dst = p.out;
  a.ds = p.os;
  a.dw = p.ow;
  a.d_mlo = p.omlo;
  a.nb = p.nb;
  const int nm = p.mhi - p.mlo + 1;
  if (p.use_q)
    launch_contract<1>(a, nm, a.nt, st);
  else
    launch_contract<0>(a, nm, a.nt, st);
}

void contract_t2l(const T2L &p, cudaStream_t st) {
  if (p.nb <= 0 || p.mhi < p.mlo) return;
  if (p.tb->rc) {
    contract_t2l_rc(p, st);
    return;
  }
  if (t_precision == 1 && p.nb > df_max_maps() && contract_t2l_mixed(&p, 1, st)) return;
  ContractArgs a{};
  a.table = p.use_q ? p.tb->Q : p.tb->D;
  if (t_precision == 1) a.table_df = df_table(*p.tb, p.use_q, st);
  a.off = p.tb->d_off;
  a.bl = p.tb->bl;
  a.nt = p.tb->nt;
  a.an = p.tb->an;
  a.tmlo = p.tb->mlo;
  a.n = p.n;
  a.mlo = p.mlo;
  a.lmin = p.lmin;
  a.w = p.w;
  a.wscale = p.wscale;
  a.wconj = p.wconj;
  a.src = p.in;
  a.ss = p.is;
  a.sw_or_xL = p.iw;
  a.s_mlo = p.imlo;
  a.dst = p.y;
  a.ds = p.ys;
  a.nb = p.nb;
  const int nm = p.mhi - p.mlo + 1;
  if (p.use_q)
    launch_contract<2>(a, nm, a.bl, st);
  else
    launch_contract<3>(a, nm, a.bl, st);
}

// split precision, two scales of one band-limit and n on a stored table, a
// batch the double-float kernel takes: both parts in one pass over the table
bool df_pair_l2t(const L2T *a, cudaStream_t st) {
  const L2T &p = a[0], &q = a[1];
  if (p.tb != q.tb || p.tb->rc || p.use_q != q.use_q || p.n != q.n || p.mlo != q.mlo || p.mhi != q.mhi ||
      p.xs != q.xs || p.xL != q.xL || p.x_half != q.x_half || p.wscale != q.wscale || p.wconj != q.wconj ||
      p.os != q.os || p.ow != q.ow || p.omlo != q.omlo || p.nb != q.nb || p.nb > 4 || p.nb < 1 || p.mhi < p.mlo)
    return false;
  ContractArgs c{};
  c.table = p.use_q ? p.tb->Q : p.tb->D;
  c.table_df = df_table(*p.tb, p.use_q, st);
  c.off = p.tb->d_off;
  c.bl = p.tb->bl;
  c.nt = p.tb->nt;
  c.an = p.tb->an;
  c.tmlo = p.tb->mlo;
  c.n = p.n;
  c.mlo = p.mlo;
  c.lmin = p.lmin;
  c.w = p.w;
  c.wscale = p.wscale;
  c.wconj = p.wconj;
  c.src = p.x;
  c.ss = p.xs;
  c.sw_or_xL = p.xL;
  c.x_half = p.x_half;
  c.dst = p.out;
  c.ds = p.os;
  c.dw = p.ow;
  c.d_mlo = p.omlo;
  c.nb = p.nb;
  c.nparts = 2;
  c.src2 = q.x;
  c.dst2 = q.out;
  c.w2 = q.w;
  c.lmin2 = q.lmin;
  const int nm = p.mhi - p.mlo + 1;
  if (p.use_q)
    launch_contract_df_pair<1>(c, nm, c.nt, st);
  else
    launch_contract_df_pair<0>(c, nm, c.nt, st);
  return true;
}

bool df_pair_t2l(const T2L *a, cudaStream_t st) {
  const T2L &p = a[0], &q = a[1];
  if (p.tb != q.tb || p.tb->rc || p.use_q != q.use_q || p.n != q.n || p.mlo != q.mlo || p.mhi != q.mhi ||
      p.is != q.is || p.iw != q.iw || p.imlo != q.imlo || p.wscale != q.wscale || p.wconj != q.wconj ||
      p.ys != q.ys || p.nb != q.nb || p.nb > 4 || p.nb < 1 || p.mhi < p.mlo)
    return false;
  ContractArgs c{};
  c.table = p.use_q ? p.tb->Q : p.tb->D;
  c.table_df = df_table(*p.tb, p.use_q, st);
  c.off = p.tb->d_off;
  c.bl = p.tb->bl;
  c.nt = p.tb->nt;
  c.an = p.tb->an;
  c.tmlo = p.tb->mlo;
  c.n = p.n;
  c.mlo = p.mlo;
  c.lmin = p.lmin;
  c.w = p.w;
  c.wscale = p.wscale;
  c.wconj = p.wconj;
  c.src = p.in;
  c.ss = p.is;
  c.sw_or_xL = p.iw;
  c.s_mlo = p.imlo;
  c.dst = p.y;
  c.ds = p.ys;
  c.nb = p.nb;
  c.nparts = 2;
  c.src2 = q.in;
  c.dst2 = q.y;
  c.w2 = q.w;
  c.lmin2 = q.lmin;
  const int nm = p.mhi - p.mlo + 1;
  if (p.use_q)
    launch_contract_df_pair<2>(c, nm, c.bl, st);
  else
    launch_contract_df_pair<3>(c, nm, c.bl, st);
  return true;
}

void contract_l2t_group(const L2T *a, int n, cudaStream_t st) {
  if (n <= 0) return;
  if (t_precision == 1 && n <= 2 && !a[0].tb->rc) {
    if (a[0].nb > df_max_maps()) {
      if (contract_l2t_mixed(a, n, st)) return;
    } else if (n == 2 && df_pair_l2t(a, st)) {
      return;
    }
  }
  for (int i = 0; i < n; ++i) contract_l2t(a[i], st);
}

void contract_t2l_group(const T2L *a, int n, cudaStream_t st) {
  if (n <= 0) return;
  if (t_precision == 1 && n <= 2 && !a[0].tb->rc) {
    if (a[0].nb > df_max_maps()) {
      if (contract_t2l_mixed(a, n, st)) return;
    } else if (n == 2 && df_pair_t2l(a, st)) {
      return;
    }
  }
  for (int i = 0; i < n; ++i) contract_t2l(a[i], st);
}

void gamma_synthesis(const double2 *G, double2 *spec, const int *ns, int nn, int ng, int bl, int ss, int nb,
                     bool real, double c, cudaStream_t st) {
  S2G_REQUIRE(nn >= 1 && nn <= 16 && ng * nn <= kMaxGammaTw, ERR_UNSUPPORTED, "more than 16 directions per scale");
  const int sw = real ? bl : 2 * bl - 1, nt = grid_rings(bl, ss);
  const int64_t total = (int64_t)nb * nt * sw;
  if (total <= 0) return;
  KTimer kt(KC_GAMMA, st, 0.0, (double)nb * nt * ((real ? 2.0 : 1.0) * nn + ng) * sw * 16.0);
  const unsigned grid = (unsigned)ceil_div(total, 256);
  switch (nn) {
#define S2G_GS(N) \
  case N: k_gamma_synth<N><<<grid, 256, 0, st>>>(G, spec, ns, ng, bl, nt, nb, real, c); break;
    S2G_GS(1) S2G_GS(2) S2G_GS(3) S2G_GS(4) S2G_GS(5) S2G_GS(6) S2G_GS(7) S2G_GS(8)
    S2G_GS(9) S2G_GS(10) S2G_GS(11) S2G_GS(12) S2G_GS(13) S2G_GS(14) S2G_GS(15) S2G_GS(16)
#undef S2G_GS
    default: break;
  }
  S2G_LAUNCHED();
}

void gamma_analysis(const double2 *spec, double2 *G, const int *ns, int nn, int ng, int bl, int ss, int nb,
                    bool real, double c, cudaStream_t st) {
  S2G_REQUIRE(nn >= 1 && nn <= 16 && ng * nn <= kMaxGammaTw, ERR_UNSUPPORTED, "more than 16 directions per scale");
  const int nt = grid_rings(bl, ss);
  const int64_t total = (int64_t)nb * nt * (2 * bl - 1);
  if (total <= 0) return;
  const int sw = real ? bl : 2 * bl - 1;
  KTimer kt(KC_GAMMA, st, 0.0, (double)nb * nt * ((double)ng * sw + (double)nn * (2 * bl - 1)) * 16.0);
  const unsigned grid = (unsigned)ceil_div(total, 256);
  switch (nn) {
#define S2G_GA(N) \
  case N: k_gamma_anal<N><<<grid, 256, 0, st>>>(spec, G, ns, ng, bl, nt, nb, real, c); break;
    S2G_GA(1) S2G_GA(2) S2G_GA(3) S2G_GA(4) S2G_GA(5) S2G_GA(6) S2G_GA(7) S2G_GA(8)
    S2G_GA(9) S2G_GA(10) S2G_GA(11) S2G_GA(12) S2G_GA(13) S2G_GA(14) S2G_GA(15) S2G_GA(16)
#undef S2G_GA
    default: break;
  }
  S2G_LAUNCHED();
}

// blocks for a grid-stride pixel gamma kernel: as many as are resident at
// once (one wave), fewer for small inputs
static unsigned gamma_px_grid(int64_t total, const void *kernel) {
  static const int nsm = [] {
    int dev = 0, n = 0;
    S2G_CUDA(cudaGetDevice(&dev));
    S2G_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
    return n;
  }();
  static std::mutex mu;
  static std::map<const void *, int> per_sm;
  int blocks;
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = per_sm.find(kernel);
    if (it == per_sm.end()) {
      int b = 0;
      S2G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, 256, 0));
      it = per_sm.emplace(kernel, b > 0 ? b : 1).first;
    }
    blocks = it->second;
  }
  const int64_t want = ceil_div(total, 256), cap = (int64_t)nsm * blocks;
  return (unsigned)(want < cap ? want : cap);
}

void gamma_px_synthesis(const double2 *F, void *out, int64_t out_ms, const int *ns, int nn, int ng, int bl,
                        int ss, int nb, bool real, double c, cudaStream_t st) {
  S2G_REQUIRE(nn >= 1 && nn <= 16 && ng * nn <= kMaxGammaTw, ERR_UNSUPPORTED, "more than 16 directions per scale");
  const int64_t npx = (int64_t)grid_rings(bl, ss) * grid_ring_len(bl, ss);
  const int64_t total = (int64_t)nb * npx;
  if (total <= 0) return;
  KTimer kt(KC_GAMMA, st, 0.0, (double)total * (16.0 * nn + (real ? 8.0 : 16.0) * ng));
  switch (nn) {
#define S2G_GPS(N)                                                                                    \
  case N:                                                                                             \
    if (t_precision == 1)                                                                             \
      k_gamma_px_synth_df<N><<<gamma_px_grid(total, (const void *)k_gamma_px_synth_df<N>), 256, 0, st>>>( \
          F, out, out_ms, ns, ng, npx, nb, real, c);                                                  \
    else                                                                                              \
      k_gamma_px_synth<N><<<gamma_px_grid(total, (const void *)k_gamma_px_synth<N>), 256, 0, st>>>(       \
          F, out, out_ms, ns, ng, npx, nb, real, c);                                                  \
    break;
    S2G_GPS(1) S2G_GPS(2) S2G_GPS(3) S2G_GPS(4) S2G_GPS(5) S2G_GPS(6) S2G_GPS(7) S2G_GPS(8)
    S2G_GPS(9) S2G_GPS(10) S2G_GPS(11) S2G_GPS(12) S2G_GPS(13) S2G_GPS(14) S2G_GPS(15) S2G_GPS(16)
#undef S2G_GPS
    default: break;
  }
  S2G_LAUNCHED();
}

void gamma_px_analysis(const void *in, int64_t in_ms, double2 *F, const int *ns, int nn, int ng, int bl, int ss,
                       int nb, bool real, double c, cudaStream_t st) {
  S2G_REQUIRE(nn >= 1 && nn <= 16 && ng * nn <= kMaxGammaTw, ERR_UNSUPPORTED, "more than 16 directions per scale");
  const int64_t npx = (int64_t)grid_rings(bl, ss) * grid_ring_len(bl, ss);
  const int64_t total = (int64_t)nb * npx;
  if (total <= 0) return;
  KTimer kt(KC_GAMMA, st, 0.0, (double)total * (16.0 * nn + (real ? 8.0 : 16.0) * ng));
  switch (nn) {
#define S2G_GPA(N)                                                                                  \
  case N:                                                                                           \
    if (t_precision == 1)                                                                           \
      k_gamma_px_anal_df<N><<<gamma_px_grid(total, (const void *)k_gamma_px_anal_df<N>), 256, 0, st>>>( \
          in, in_ms, F, ns, ng, npx, nb, real, c);                                                  \
    else                                                                                            \
      k_gamma_px_anal<N><<<gamma_px_grid(total, (const void *)k_gamma_px_anal<N>), 256, 0, st>>>(       \
          in, in_ms, F, ns, ng, npx, nb, real, c);                                                  \
    break;
    S2G_GPA(1) S2G_GPA(2) S2G_GPA(3) S2G_GPA(4) S2G_GPA(5) S2G_GPA(6) S2G_GPA(7) S2G_GPA(8)
    S2G_GPA(9) S2G_GPA(10) S2G_GPA(11) S2G_GPA(12) S2G_GPA(13) S2G_GPA(14) S2G_GPA(15) S2G_GPA(16)
#undef S2G_GPA
    default: break;
  }
  S2G_LAUNCHED();
}


void merge_lmn(double2 *flm, int L, int64_t fs, const double2 *z, int64_t zs, const MergePair *pairs,
               int npairs, const double2 *wts, const double2 *zscal, int64_t zss, int bl_scal,
               bool real, bool accumulate, int nb, cudaStream_t st) {
  const int64_t total = (int64_t)nb * L * L;
  if (total <= 0) return;
  KTimer kt(KC_MERGE, st, 0.0, 0.0);
  k_merge<<<ceil_div(total, 256), 256, 0, st>>>(flm, L, fs, z, zs, pairs, npairs, wts, zscal, zss,
                                               bl_scal, real, accumulate, nb);
  S2G_LAUNCHED();
}

namespace {
int conv_grid(int64_t total) {
  static const int nsm = [] {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
  }();
  const int64_t want = ceil_div(total, 256);
  return (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)nsm * 8));
}
}  // namespace

void widen_rows(const float *src, int64_t ss, double *dst, int64_t ds, int64_t n, int rows, cudaStream_t st) {
  if (n <= 0 || rows <= 0) return;
  KTimer kt(KC_OTHER, st, 0.0, 12.0 * (double)n * rows);
  k_widen_rows<<<conv_grid(n * rows), 256, 0, st>>>(src, ss, dst, ds, n, rows);
  S2G_LAUNCHED();
}
void narrow_rows(const double *src, int64_t ss, float *dst, int64_t ds, int64_t n, int rows, cudaStream_t st) {
  if (n <= 0 || rows <= 0) return;
  KTimer kt(KC_OTHER, st, 0.0, 12.0 * (double)n * rows);
  k_narrow_rows<<<conv_grid(n * rows), 256, 0, st>>>(src, ss, dst, ds, n, rows);
  S2G_LAUNCHED();
}

void symmetrize_flm(double2 *flm, int L, int64_t fs, int nb, cudaStream_t st) {
  const int64_t total = (int64_t)nb * L * L;
  if (total <= 0) return;
  KTimer kt(KC_MERGE, st, 0.0, 0.0);
  k_symmetrize<<<ceil_div(total, 256), 256, 0, st>>>(flm, L, fs, nb);
  S2G_LAUNCHED();
}

void scale_copy(const double *x, double *y, int64_t n, double s, cudaStream_t st) {
  if (n <= 0) return;
  k_scale_copy<<<ceil_div(n, 256), 256, 0, st>>>(x, y, n, s);
  S2G_LAUNCHED();
}

void axpby(const double *x, int64_t xs, double *y, int64_t ys, int64_t n, int nb, double a, double c,
           cudaStream_t st) {
  if (n <= 0 || nb <= 0) return;
  k_axpby<<<ceil_div(n * nb, 256), 256, 0, st>>>(x, xs, y, ys, n, nb, a, c);
  S2G_LAUNCHED();
}

}  // namespace s2g

// ===========================================================================
// Wigner-layout tiling multiplies, axisymmetric multiplies, thresholding
// ===========================================================================

namespace s2g {

namespace {

__device__ __forceinline__ int64_t sumsq(int64_t k) { return k < 0 ? 0 : k * (k + 1) * (2 * k + 1) / 6; }

// SO3 compact storage index (src of the layout: so3_sampling_elmn2ind for
// SO3_STORAGE_COMPACT / SO3_N_ORDER_NEGATIVE_FIRST)
__device__ __forceinline__ int64_t so3_index(int l, int m, int n, int L, int N, bool real) {
  const int64_t L2 = (int64_t)L * L;
  if (real) return (int64_t)n * L2 - sumsq(n - 1) + (int64_t)l * l - (int64_t)n * n + l + m;
  const int64_t drop = (n <= 0) ? sumsq(N - 1) - sumsq(-n) : sumsq(N - 1) + sumsq(n - 1);
  return (int64_t)(n + N - 1) * L2 - drop + (int64_t)l * l - (int64_t)n * n + l + m;
}

__device__ __forceinline__ void lm_of(int i, int &l, int &m) {
  int q = (int)sqrt((double)i);
  while (q * q > i) --q;
  while ((q + 1) * (q + 1) <= i) ++q;
  l = q;
  m = i - q * q - q;
}

__global__ void k_lmn_split(double2 *flmn, double2 *fscal, const double2 *__restrict__ flm,
                            const double2 *__restrict__ psi, const double *__restrict__ phi,
                            const LmnScale *__restrict__ scales, int nscale, int L, int bl_scal, int spin,
                            int real, int mode) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L * L) return;
  int l, m;
  lm_of(i, l, m);
  const int k = blockIdx.y, zi = blockIdx.z;
  if (k == nscale) {  // scaling part
    if (zi != 0 || l >= bl_scal || l < (real ? 0 : (spin < 0 ? -spin : spin))) return;
    fscal[i] = scl2(flm[i], sqrt(4.0 * kPi / (2 * l + 1)) * phi[l]);
    return;
  }
  const LmnScale sc = scales[k];
  if (l >= sc.bl) return;
  const int n = real ? (1 - sc.Nj % 2) + 2 * zi : -sc.Nj + 1 + 2 * zi;
  if (n >= sc.Nj) return;
  const int an = n < 0 ? -n : n, as = spin < 0 ? -spin : spin;
  const int lmin = real ? n : (as > an ? as : an);
  if (l < lmin) return;
  double2 w = conj2(psi[(int64_t)sc.j * L * L + (int64_t)l * l + l + n]);
  if (mode == 0) w = scl2(w, 8.0 * kPi * kPi / (2 * l + 1));
  flmn[sc.loff + so3_index(l, m, n, sc.bl, sc.Nj, real)] = cmul(flm[i], w);
}

__global__ void k_lmn_merge(double2 *flm, const double2 *__restrict__ flmn, const double2 *__restrict__ fscal,
                            const double2 *__restrict__ psi, const double *__restrict__ phi,
                            const LmnScale *__restrict__ scales, int nscale, int L, int bl_scal, int spin,
                            int real, int mode) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L * L) return;
  int l, m;
  lm_of(i, l, m);
  const int as = spin < 0 ? -spin : spin;
  double2 acc = make_double2(0.0, 0.0);
  const double sc8 = (mode == 1) ? 8.0 * kPi * kPi / (2 * l + 1) : 1.0;
  for (int k = 0; k < nscale; ++k) {
    const LmnScale sc = scales[k];
    if (l >= sc.bl) continue;
    const int n0 = real ? 1 - sc.Nj % 2 : -sc.Nj + 1;
    for (int n = n0; n < sc.Nj; n += 2) {
      const int an = n < 0 ? -n : n;
      const int lmin = real ? n : (as > an ? as : an);
      if (l < lmin) continue;
      const double2 *ps = psi + (int64_t)sc.j * L * L + (int64_t)l * l + l;
      acc = add2(acc, cmul(flmn[sc.loff + so3_index(l, m, n, sc.bl, sc.Nj, real)], scl2(ps[n], sc8)));
      if (real && n) {
        double2 v = cmul(conj2(flmn[sc.loff + so3_index(l, -m, n, sc.bl, sc.Nj, real)]), scl2(ps[-n], sc8));
        if ((m + n) & 1) v = scl2(v, -1.0);
        acc = add2(acc, v);
      }
    }
  }
  if (l < bl_scal && l >= (real ? 0 : as)) acc = add2(acc, scl2(fscal[i], sqrt(4.0 * kPi / (2 * l + 1)) * phi[l]));
  flm[i] = acc;
}

__global__ void k_axi_lm(double2 *flm, double2 *fwav, double2 *fscal, const double *__restrict__ wav_lm,
                         const double *__restrict__ scal_lm, const int *__restrict__ bl,
                         const int64_t *__restrict__ off, int J_min, int nscale, int L, int bl_scal, int synth) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= L * L) return;
  int l, m;
  lm_of(i, l, m);
  const double nl = sqrt((4.0 * kPi) / (2.0 * l + 1.0));
  if (!synth) {
    for (int k = 0; k < nscale; ++k)
      if (l < bl[k]) fwav[off[k] + i] = scl2(flm[i], nl * wav_lm[(int64_t)(J_min + k) * L + l]);
    if (l < bl_scal) fscal[i] = scl2(flm[i], nl * scal_lm[l]);
  } else {
    double2 acc = flm[i];
    for (int k = 0; k < nscale; ++k)
      if (l < bl[k]) acc = add2(acc, scl2(fwav[off[k] + i], nl * wav_lm[(int64_t)(J_min + k) * L + l]));
    if (l < bl_scal) acc = add2(acc, scl2(fscal[i], nl * scal_lm[l]));
    flm[i] = acc;
  }
}

__global__ void k_threshold(double *g, const double *__restrict__ thr, const int64_t *__restrict__ off,
                            int nscale, int64_t total) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  int k = 0;
  while (k + 1 < nscale && off[k + 1] <= i) ++k;
  const double v = g[i];
  // the reference compares abs() of an int-converted double (truncation toward zero)
  const long long t = (fabs(v) < 9.2e18) ? (long long)v : 0x7fffffffffffffffLL;
  const long long a = t < 0 ? -t : t;
  if ((double)a < thr[k]) g[i] = 0.0;
}

}  // namespace

void lmn_split(double2 *flmn, double2 *fscal, const double2 *flm, const double2 *psi, const double *phi,
               const LmnScale *scales, int nscale, int Nmax, int L, int bl_scal, int spin, bool real,
               int mode, cudaStream_t st) {
  dim3 grid(ceil_div((int64_t)L * L, 128), nscale + 1, Nmax > 0 ? Nmax : 1);
  k_lmn_split<<<grid, 128, 0, st>>>(flmn, fscal, flm, psi, phi, scales, nscale, L, bl_scal, spin, real, mode);
  S2G_LAUNCHED();
}

void lmn_merge(double2 *flm, const double2 *flmn, const double2 *fscal, const double2 *psi,
               const double *phi, const LmnScale *scales, int nscale, int L, int bl_scal, int spin,
               bool real, int mode, cudaStream_t st) {
  k_lmn_merge<<<ceil_div((int64_t)L * L, 128), 128, 0, st>>>(flm, flmn, fscal, psi, phi, scales, nscale, L,
                                                              bl_scal, spin, real, mode);
  S2G_LAUNCHED();
}

void axisym_lm(double2 *flm, double2 *fwav, double2 *fscal, const double *wav_lm, const double *scal_lm,
               const int *bl, const int64_t *off, int J_min, int nscale, int L, int bl_scal, int synth,
               cudaStream_t st) {
  k_axi_lm<<<ceil_div((int64_t)L * L, 128), 128, 0, st>>>(flm, fwav, fscal, wav_lm, scal_lm, bl, off, J_min,
                                                           nscale, L, bl_scal, synth);
  S2G_LAUNCHED();
}

void hard_threshold(double *g, const double *thr, const int64_t *off, int nscale, int64_t total,
                    cudaStream_t st) {
  if (total <= 0) return;
  k_threshold<<<ceil_div(total, 256), 256, 0, st>>>(g, thr, off, nscale, total);
  S2G_LAUNCHED();
}

}  // namespace s2g
