// Conversions between FP64 and double-float (hi + lo, two floats) built from
// the IEEE-754 bit fields with integer arithmetic.
//
// GB300 executes FP64 instructions (including FP64 <-> FP32 conversions and
// ldexp) at a small fraction of the FP32 rate, so in the FP32-pipe kernels of
// the split-precision path these conversions, not the arithmetic, set the
// speed.  Everything here is integer work except one FP64 add per value
// converted back to FP64 and one int -> float conversion per value split.
//
// Scaling: a block of values is rescaled by a power of two 2^-e chosen from
// the largest exponent field, so that every scaled magnitude is below 1; values
// that the scaling puts below the float normal range (2^-126 of the block
// maximum) become zero, which is below the double-float resolution of the block.
#pragma once

#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define S2G_HD __host__ __device__ __forceinline__
#else
#define S2G_HD inline
#endif

namespace s2g {

S2G_HD uint64_t bits_of(double v) {
  uint64_t u;
  memcpy(&u, &v, 8);
  return u;
}
S2G_HD double double_of(uint64_t u) {
  double v;
  memcpy(&v, &u, 8);
  return v;
}
S2G_HD uint32_t bits_of(float v) {
  uint32_t u;
  memcpy(&u, &v, 4);
  return u;
}
S2G_HD float float_of(uint32_t u) {
  float v;
  memcpy(&v, &u, 4);
  return v;
}

// biased exponent field of v (0 for zero and subnormals)
S2G_HD int exp_field(double v) { return (int)((bits_of(v) >> 52) & 0x7FF); }

// scale exponent for a block whose largest exponent field is emax:
// |v| 2^-e < 1 for every v of the block
S2G_HD int block_scale(int emax) { return emax > 0 ? emax - 1022 : 0; }

// x * 2^k for a float x, exact while the result is a normal float; results
// below the normal range flush to zero
S2G_HD float scale_pow2(float x, int k) {
  const uint32_t b = bits_of(x);
  const int E = (int)((b >> 23) & 0xFF);
  if (E == 0) return 0.0f;
  const int ne = E + k;
  if (ne <= 0) return 0.0f;
  return float_of((b & 0x807FFFFFu) | ((uint32_t)ne << 23));
}

// v * 2^-e as (hi, lo): hi = the top 24 significant bits, lo = the next 29
// rounded to 24, then renormalised so that |lo| <= ulp(hi) / 2.  Error:
// |hi + lo - v 2^-e| <= max(2^-47 |v 2^-e|, 2^-126) (lo flushes once it would
// leave the float normal range).
S2G_HD void split_scaled(double v, int e, float &hi, float &lo) {
  const uint64_t u = bits_of(v);
  const int E = (int)((u >> 52) & 0x7FF);
  const int ex = E - 1023 - e;  // unbiased exponent of v 2^-e
  if (E == 0 || ex + 127 <= 0) {
    hi = lo = 0.0f;
    return;
  }
  const uint32_t sign = (uint32_t)(u >> 63) << 31;
  const uint64_t M = (u & 0xFFFFFFFFFFFFFull) | (1ull << 52);  // 53-bit significand
  const float h = float_of(sign | ((uint32_t)(ex + 127) << 23) | (uint32_t)((M >> 29) & 0x7FFFFFu));
  float l = scale_pow2((float)(uint32_t)(M & 0x1FFFFFFFu), ex - 52);
  if (sign) l = -l;
  // fast two-sum (|h| >= |l|)
  const float s = h + l;
  hi = s;
  lo = l - (s - h);
}

// exact float -> double with a power-of-two scale 2^k (x normal or zero)
S2G_HD double widen_scaled(float x, int k) {
  const uint32_t b = bits_of(x);
  const int E = (int)((b >> 23) & 0xFF);
  if (E == 0) return 0.0;
  const int de = E - 127 + 1023 + k;
  if (de <= 0) return 0.0;
  if (de >= 2047) return double_of(((uint64_t)(b >> 31) << 63) | (0x7FFull << 52));  // +-inf
  return double_of(((uint64_t)(b >> 31) << 63) | ((uint64_t)de << 52) | ((uint64_t)(b & 0x7FFFFFu) << 29));
}

// (hi + lo) 2^k as a double: one FP64 add
S2G_HD double join_scaled(float hi, float lo, int k) { return widen_scaled(hi, k) + widen_scaled(lo, k); }

// FP32 operations rounded to nearest: explicit intrinsics on the device (no
// contraction), IEEE single precision on the host (built with
// -ffp-contract=off)
#ifdef __CUDA_ARCH__
#define S2G_FADD(a, b) __fadd_rn((a), (b))
#define S2G_FSUB(a, b) __fsub_rn((a), (b))
#define S2G_FMUL(a, b) __fmul_rn((a), (b))
#else
#define S2G_FADD(a, b) ((a) + (b))
#define S2G_FSUB(a, b) ((a) - (b))
#define S2G_FMUL(a, b) ((a) * (b))
#endif

// Balanced base-128 digits of v 2^-e (|v| < 2^e) by FP32 arithmetic:
// v 2^-e ~ sum_{j<nd} d_j 2^(-6-7j) with integer |d_j| <= 64.  x = v 2^-e as a
// double-float (split_scaled), then per digit d = x rounded to an integer
// (adding and subtracting 1.5 * 2^23 rounds any |x| < 2^22) and x = (x - d)
// 128, kept exact in double-float (fast two-sum: the difference is either 0
// or at least the low word).  The remainder after nd = 7 digits is below
// 2^-49.  Each d is an integer-valued float of at most 7 significant bits, so
// its bf16 bit pattern is the float's top half, returned in the low 16 bits
// of out[j].
template <int nd>
S2G_HD void split_digits_fp32(double v, int e, uint32_t *out) {
  const float kRound = 12582912.0f;  // 1.5 * 2^23
  float h, l;
  split_scaled(v, e, h, l);
  h = S2G_FMUL(h, 64.0f);
  l = S2G_FMUL(l, 64.0f);
  for (int j = 0; j < nd; ++j) {
    const float r = S2G_FSUB(S2G_FADD(h, kRound), kRound);
    out[j] = bits_of(r) >> 16;
    const float sd = S2G_FSUB(h, r);  // exact
    const float t = S2G_FADD(sd, l);
    l = S2G_FSUB(l, S2G_FSUB(t, sd));
    h = S2G_FMUL(t, 128.0f);
    l = S2G_FMUL(l, 128.0f);
  }
}

}  // namespace s2g
