// Double-float ("df") arithmetic: a value is an unevaluated sum hi + lo of two
// floats with |lo| <= ulp(hi)/2, giving about 48 significant bits with FP32
// instructions only.  The mixed-precision engine keeps the propagation state
// and the linear-step factors in this form because GB300's FP64 rate is a
// small fraction of its FP32 rate.
//
// The error-free transformations are the standard ones (Knuth's two-sum,
// Dekker's fast two-sum, and the FMA two-product), e.g. as collected in
// Muller et al., "Handbook of Floating-Point Arithmetic", 2nd ed., ch. 4.
#pragma once
#include <cuda_runtime.h>

namespace gnlse {

struct dff {
  float hi, lo;
};

// complex double-float, stored as float4 {re.hi, im.hi, re.lo, im.lo} so the
// first 8 bytes are the complex64 approximation
struct dfc {
  dff re, im;
};

__device__ __forceinline__ dff two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
__device__ __forceinline__ dff fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = a + b;
  return {s, b - (s - a)};
}
__device__ __forceinline__ dff two_prod(float a, float b) {
  const float p = a * b;
  return {p, fmaf(a, b, -p)};
}
__device__ __forceinline__ dff df_add(dff a, dff b) {
  dff s = two_sum(a.hi, b.hi);
  s.lo += a.lo + b.lo;
  return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ dff df_add_f(dff a, float b) {
  dff s = two_sum(a.hi, b);
  s.lo += a.lo;
  return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ dff df_neg(dff a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ dff df_mul(dff a, dff b) {
  dff p = two_prod(a.hi, b.hi);
  p.lo = fmaf(a.hi, b.lo, p.lo);
  p.lo = fmaf(a.lo, b.hi, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ dff df_mul_f(dff a, float b) {
  dff p = two_prod(a.hi, b);
  p.lo = fmaf(a.lo, b, p.lo);
  return fast_two_sum(p.hi, p.lo);
}
__device__ __forceinline__ dff df_from_double(double x) {
  const float hi = (float)x;
  return {hi, (float)(x - (double)hi)};
}
__device__ __forceinline__ double df_to_double(dff a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ dfc dfc_load(const float4* p, long long a) {
  const float4 v = p[a];
  return {{v.x, v.z}, {v.y, v.w}};
}
__device__ __forceinline__ void dfc_store(float4* p, long long a, dfc v) {
  p[a] = make_float4(v.re.hi, v.im.hi, v.re.lo, v.im.lo);
}
__device__ __forceinline__ float2 dfc_hi(dfc v) { return make_float2(v.re.hi, v.im.hi); }
__device__ __forceinline__ float2 ld_hi(const float4* p, long long a) {
  return *reinterpret_cast<const float2*>(p + a);
}
__device__ __forceinline__ dfc dfc_mul(dfc a, dfc b) {
  return {df_add(df_mul(a.re, b.re), df_neg(df_mul(a.im, b.im))),
          df_add(df_mul(a.re, b.im), df_mul(a.im, b.re))};
}
__device__ __forceinline__ dfc dfc_scale(dfc a, dff s) { return {df_mul(a.re, s), df_mul(a.im, s)}; }
__device__ __forceinline__ dfc dfc_add(dfc a, dfc b) { return {df_add(a.re, b.re), df_add(a.im, b.im)}; }
__device__ __forceinline__ dfc dfc_add_f(dfc a, float2 b) { return {df_add_f(a.re, b.x), df_add_f(a.im, b.y)}; }
__device__ __forceinline__ dfc dfc_sub(dfc a, dfc b) {
  return {df_add(a.re, df_neg(b.re)), df_add(a.im, df_neg(b.im))};
}

}  // namespace gnlse
