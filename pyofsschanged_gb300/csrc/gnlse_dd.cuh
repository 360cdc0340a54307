// Double-float scalar and complex types with arithmetic operators ("df" plans).
//
// A ddf is the unevaluated sum hi + lo of two floats (|lo| <= ulp(hi)/2), about
// 48 significant bits carried on FP32 instructions.  With the operators below the
// engine's generic transform, nonlinear and stage code (written for float2 /
// double2) runs unchanged on ddc values: every transform, the nonlinear term and
// the RK stage algebra keep ~1e-14 relative precision, close to FP64, at a cost
// set by GB300's FP32 rate instead of its much lower FP64 rate.
//
// Error-free transformations: Knuth's two-sum and the FMA two-product (Muller
// et al., "Handbook of Floating-Point Arithmetic", 2nd ed., ch. 4); addition is
// the "sloppy" double-word sum (error bounded by a few units of 2^-48 of the
// operands' magnitudes, which is what a norm-wise stable FFT needs) and
// multiplication the FMA double-word product.  Products use __fmul_rn, which the
// compiler never contracts into an FMA, so each error term is exact.
#pragma once
#include <cuda_runtime.h>
#include <math.h>

namespace gnlse {

// the double-float overloads below join, not hide, the FP32/FP64 math functions
using ::exp;
using ::fma;
using ::isfinite;

struct ddf {
  float hi, lo;
  ddf() = default;
  __host__ __device__ constexpr ddf(double d) : hi((float)d), lo((float)(d - (double)(float)d)) {}
  __host__ __device__ constexpr ddf(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ explicit operator double() const { return (double)hi + (double)lo; }
};

// complex double-float: memory layout {re.hi, re.lo, im.hi, im.lo}
struct __align__(16) ddc {
  ddf x, y;
};

__device__ __forceinline__ ddf dd_renorm(float s, float e) {  // fast two-sum, |s| >= |e|
  const float h = __fadd_rn(s, e);
  return ddf(h, __fsub_rn(e, __fsub_rn(h, s)));
}

__device__ __forceinline__ ddf operator+(ddf a, ddf b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  return dd_renorm(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ ddf operator-(ddf a) { return ddf(-a.hi, -a.lo); }
__device__ __forceinline__ ddf operator-(ddf a, ddf b) { return a + (-b); }
__device__ __forceinline__ ddf operator*(ddf a, ddf b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, e);
  e = fmaf(a.lo, b.hi, e);
  return dd_renorm(p, e);
}
__device__ __forceinline__ ddf& operator+=(ddf& a, ddf b) { return a = a + b; }
__device__ __forceinline__ ddf& operator-=(ddf& a, ddf b) { return a = a - b; }
__device__ __forceinline__ ddf& operator*=(ddf& a, ddf b) { return a = a * b; }

__device__ __forceinline__ bool isfinite(ddf a) { return ::isfinite(a.hi) && ::isfinite(a.lo); }
__device__ __forceinline__ ddf fma(ddf a, ddf b, ddf c) { return a * b + c; }
// the gain paths' exponential, in FP64 (once per element and linear-operator call)
__device__ __forceinline__ ddf exp(ddf a) { return ddf(::exp((double)a)); }

// a b + c d with one two-sum: the two leading products' exact rounding errors and the
// cross terms go into the low word
__device__ __forceinline__ ddf dd_dot2(ddf a, ddf b, ddf c, ddf d) {
  const float p = __fmul_rn(a.hi, b.hi);
  const float q = __fmul_rn(c.hi, d.hi);
  const float ep = fmaf(a.hi, b.hi, -p);  // exact rounding errors of p and q
  const float eq = fmaf(c.hi, d.hi, -q);
  const float s = __fadd_rn(p, q);        // two-sum of the leading products
  const float bb = __fsub_rn(s, p);
  const float t = __fadd_rn(__fsub_rn(p, __fsub_rn(s, bb)), __fsub_rn(q, bb));
  float lo = __fadd_rn(__fadd_rn(t, ep), eq);
  lo = fmaf(a.hi, b.lo, lo);
  lo = fmaf(a.lo, b.hi, lo);
  lo = fmaf(c.hi, d.lo, lo);
  lo = fmaf(c.lo, d.hi, lo);
  return dd_renorm(s, lo);
}

__device__ __forceinline__ ddc cmul(ddc a, ddc b) {
  return ddc{dd_dot2(a.x, b.x, -a.y, b.y), dd_dot2(a.x, b.y, a.y, b.x)};
}
__device__ __forceinline__ ddc cmulc(ddc a, ddc b) {  // a * conj(b)
  return ddc{dd_dot2(a.x, b.x, a.y, b.y), dd_dot2(a.y, b.x, -a.x, b.y)};
}

// GNLSE_DF_LAZY: 2 (default) transforms without renormalisation, 1 renormalised butterfly
// outputs, 0 renormalisation after every operation.  Measured on the ensemble's df classes
// (GB300): 1 is 3-5% and 2 a further 9-10% less SM time per attempt than 0, with the same
// results to the tests' 1e-9 and identical step sequences.
#ifndef GNLSE_DF_LAZY
#define GNLSE_DF_LAZY 2
#endif
#if GNLSE_DF_LAZY
// Lazy variants for the transforms' butterflies and twiddles: the same error-free
// transformations without the final renormalisation, so the low word may exceed half an
// ulp of the high word.  A two-sum of the high words stays exact for any inputs and the
// low words only accumulate, so a transform's few lazy operations per value keep the
// double-word accuracy norm-wise; the next non-lazy operation (the stage algebra, the
// nonlinear term) renormalises.
__device__ __forceinline__ ddf dd_add_lazy(ddf a, ddf b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  return ddf(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ ddf dd_dot2_lazy(ddf a, ddf b, ddf c, ddf d) {  // a b + c d
  const float p = __fmul_rn(a.hi, b.hi);
  const float q = __fmul_rn(c.hi, d.hi);
  const float ep = fmaf(a.hi, b.hi, -p);
  const float eq = fmaf(c.hi, d.hi, -q);
  const float s = __fadd_rn(p, q);
  const float bb = __fsub_rn(s, p);
  const float t = __fadd_rn(__fsub_rn(p, __fsub_rn(s, bb)), __fsub_rn(q, bb));
  float lo = __fadd_rn(__fadd_rn(t, ep), eq);
  lo = fmaf(a.hi, b.lo, lo);
  lo = fmaf(a.lo, b.hi, lo);
  lo = fmaf(c.hi, d.lo, lo);
  lo = fmaf(c.lo, d.hi, lo);
  return ddf(s, lo);
}
__device__ __forceinline__ ddc cadd_lazy(ddc a, ddc b) { return ddc{dd_add_lazy(a.x, b.x), dd_add_lazy(a.y, b.y)}; }
__device__ __forceinline__ ddc csub_lazy(ddc a, ddc b) { return ddc{dd_add_lazy(a.x, -b.x), dd_add_lazy(a.y, -b.y)}; }
__device__ __forceinline__ ddc cmul_lazy(ddc a, ddc b) {
  return ddc{dd_dot2_lazy(a.x, b.x, -a.y, b.y), dd_dot2_lazy(a.x, b.y, a.y, b.x)};
}
__device__ __forceinline__ ddc cmulc_lazy(ddc a, ddc b) {
  return ddc{dd_dot2_lazy(a.x, b.x, a.y, b.y), dd_dot2_lazy(a.y, b.x, -a.x, b.y)};
}
// renormalisation after lazy operations: a full two-sum, since cancellation of the high
// words may leave the low word the larger
__device__ __forceinline__ ddf dd_norm(ddf a) {
  const float s = __fadd_rn(a.hi, a.lo);
  const float bb = __fsub_rn(s, a.hi);
  return ddf(s, __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(a.lo, bb)));
}
#if GNLSE_DF_LAZY == 2
__device__ __forceinline__ ddc cnorm(ddc a) { return a; }
#else
__device__ __forceinline__ ddc cnorm(ddc a) { return ddc{dd_norm(a.x), dd_norm(a.y)}; }
#endif
#endif

}  // namespace gnlse
