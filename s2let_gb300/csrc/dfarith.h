// Double-float arithmetic on the FP32 pipe (device code): unevaluated sums
// hi + lo of two floats, error-free transformations of Dekker / Knuth (two-sum,
// two-product by FMA) with explicit round-to-nearest intrinsics so that no
// multiply-add is contracted.  Sums and products are left unnormalised (no
// fast-two-sum after the error term is added): hi + lo still carries the value,
// |lo| grows by at most ulp(hi)/2 plus the inputs' lo per operation, and the
// widening to FP64 (dfconv.h) accepts any split.  Complex values are float4
// (re.hi, re.lo, im.hi, im.lo).
#pragma once

#include <cuda_runtime.h>

#include "dfconv.h"

namespace s2g {
namespace {

__device__ __forceinline__ float2 df_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float v = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, v)), __fsub_rn(b, v));
  return make_float2(s, e);
}
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
  float2 s = df_two_sum(a.x, b.x);
  s.y = __fadd_rn(s.y, __fadd_rn(a.y, b.y));
  return s;
}
__device__ __forceinline__ float2 df_neg(float2 a) { return make_float2(-a.x, -a.y); }
// a + b renormalised (fast two-sum of the result: |lo| <= ulp(hi) / 2), for
// accumulators summing many terms, where the unnormalised lo would grow
__device__ __forceinline__ float2 df_add_norm(float2 a, float2 b) {
  const float2 s = df_add(a, b);
  const float h = __fadd_rn(s.x, s.y);
  return make_float2(h, __fsub_rn(s.y, __fsub_rn(h, s.x)));
}
// a*b + c*d (double-float in, double-float out)
__device__ __forceinline__ float2 df_dot2(float2 a, float2 b, float2 c, float2 d) {
  const float p1 = __fmul_rn(a.x, b.x);
  const float e1 = __fmaf_rn(a.x, b.x, -p1);
  const float p2 = __fmul_rn(c.x, d.x);
  const float e2 = __fmaf_rn(c.x, d.x, -p2);
  const float2 s = df_two_sum(p1, p2);
  float e = __fadd_rn(s.y, __fadd_rn(e1, e2));
  e = __fmaf_rn(a.x, b.y, e);
  e = __fmaf_rn(a.y, b.x, e);
  e = __fmaf_rn(c.x, d.y, e);
  e = __fmaf_rn(c.y, d.x, e);
  return make_float2(s.x, e);
}
// complex double-float as float4 (re.hi, re.lo, im.hi, im.lo)
__device__ __forceinline__ float2 dre(float4 z) { return make_float2(z.x, z.y); }
__device__ __forceinline__ float2 dim_(float4 z) { return make_float2(z.z, z.w); }
__device__ __forceinline__ float4 dmk(float2 re, float2 im) { return make_float4(re.x, re.y, im.x, im.y); }
__device__ __forceinline__ float4 dc_mul(float4 a, float4 b) {
  return dmk(df_dot2(dre(a), dre(b), df_neg(dim_(a)), dim_(b)), df_dot2(dre(a), dim_(b), dim_(a), dre(b)));
}
__device__ __forceinline__ float4 dc_mulc(float4 a, float4 b) {  // a * conj(b)
  return dmk(df_dot2(dre(a), dre(b), dim_(a), dim_(b)), df_dot2(dim_(a), dre(b), df_neg(dre(a)), dim_(b)));
}
__device__ __forceinline__ float4 dc_add(float4 a, float4 b) {
  return dmk(df_add(dre(a), dre(b)), df_add(dim_(a), dim_(b)));
}
__device__ __forceinline__ float4 dc_sub(float4 a, float4 b) {
  return dmk(df_add(dre(a), df_neg(dre(b))), df_add(dim_(a), df_neg(dim_(b))));
}
__device__ __forceinline__ float4 dc_conj(float4 a) { return make_float4(a.x, a.y, -a.z, -a.w); }
// FP64 <-> double-float with a power-of-two block scale, by bit construction
// (dfconv.h): no FP64 instructions but one add per value joined
__device__ __forceinline__ float2 df_split(double v, int e) {
  float h, l;
  split_scaled(v, e, h, l);
  return make_float2(h, l);
}
__device__ __forceinline__ float4 dc_split(double2 v, int e) { return dmk(df_split(v.x, e), df_split(v.y, e)); }
__device__ __forceinline__ double2 dc_to(float4 z, int e) {
  return make_double2(join_scaled(z.x, z.y, e), join_scaled(z.z, z.w, e));
}
// a*b (double-float in and out)
__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  float e = __fmaf_rn(a.x, b.x, -p);
  e = __fmaf_rn(a.x, b.y, e);
  e = __fmaf_rn(a.y, b.x, e);
  return make_float2(p, e);
}

// s += v x (double-float real times complex), the accumulator renormalised
// after each add (for sums of many terms)
__device__ __forceinline__ void df_mac(float4 &s, float2 v, float4 x) {
  s = dmk(df_add_norm(dre(s), df_mul(v, dre(x))), df_add_norm(dim_(s), df_mul(v, dim_(x))));
}

}  // namespace
}  // namespace s2g
