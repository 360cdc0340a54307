// Double-float scalar and complex types with arithmetic operators ("df" plans).
//
// A ddf is the unevaluated sum hi + lo of two floats (|lo| <= ulp(hi)/2), about
// 48 significant bits carried on FP32 instructions.  With the operators below the
// engine's generic transform, nonlinear and stage code (written for float2 /
// double2, reading components through re / im / mk) runs on ddc values: every
// transform, the nonlinear term and the RK stage algebra keep ~1e-14 relative
// precision, close to FP64, at a cost set by GB300's FP32 rate instead of its much
// lower FP64 rate.  The complex operations run the real and imaginary components'
// sequences as paired FP32x2 instructions (see ddc below).
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

// GNLSE_DF_LAZY: 2 (default) transforms without renormalisation, 1 renormalised butterfly
// outputs, 0 renormalisation after every operation.  Measured on the ensemble's df classes
// (GB300): 1 is 3-5% and 2 a further 9-10% less SM time per attempt than 0, with the same
// results to the tests' 1e-9 and identical step sequences.
#ifndef GNLSE_DF_LAZY
#define GNLSE_DF_LAZY 2
#endif

// ---- complex double-float ----------------------------------------------------------
// Layout {re.hi, im.hi, re.lo, im.lo}: the high words of the two components form one
// float2 and the low words another, so the components' identical operation sequences run
// as Blackwell's paired FP32 instructions (__fadd2_rn / __fmul2_rn / __ffma2_rn, sm_100
// and later), one instruction per pair and each component rounded as the scalar
// operation rounds it.  GNLSE_DF_F32X2 = 0 issues the same sequences as scalar FP32
// instructions (identical results).  Measured on GB300 (ensemble df classes, SM time per
// ARK4IP attempt): the paired build takes 7-12% less than the scalar one (2^14 points
// on 8 CTAs: 2879 against 3241 us; 2^13 on 4: 1269 against 1444), despite the register
// pairs' extra spills.
#ifndef GNLSE_DF_F32X2
#define GNLSE_DF_F32X2 1
#endif

struct __align__(16) ddc {
  float2 hi, lo;
};
__host__ __device__ inline ddf re(const ddc& a) { return ddf(a.hi.x, a.lo.x); }
__host__ __device__ inline ddf im(const ddc& a) { return ddf(a.hi.y, a.lo.y); }
__host__ __device__ inline ddc mkdc(ddf r, ddf i) {
  return ddc{make_float2(r.hi, i.hi), make_float2(r.lo, i.lo)};
}

__device__ __forceinline__ float2 f2neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 f2add(float2 a, float2 b) {
#if GNLSE_DF_F32X2
  return __fadd2_rn(a, b);
#else
  return make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y));
#endif
}
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) {
#if GNLSE_DF_F32X2
  return __fadd2_rn(a, f2neg(b));
#else
  return make_float2(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y));
#endif
}
__device__ __forceinline__ float2 f2mul(float2 a, float2 b) {
#if GNLSE_DF_F32X2
  return __fmul2_rn(a, b);
#else
  return make_float2(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y));
#endif
}
__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) {
#if GNLSE_DF_F32X2
  return __ffma2_rn(a, b, c);
#else
  return make_float2(fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y));
#endif
}

// fast two-sum of both components (|s| >= |e|)
__device__ __forceinline__ ddc crenorm(float2 s, float2 e) {
  const float2 h = f2add(s, e);
  return ddc{h, f2sub(e, f2sub(h, s))};
}
// a + b and a - b per component (the sloppy double-word sum of operator+), low words
// not renormalised (cadd_u, csub_u) or renormalised (cadd, csub)
__device__ __forceinline__ ddc cadd_u(ddc a, ddc b) {
  const float2 s = f2add(a.hi, b.hi);
  const float2 bb = f2sub(s, a.hi);
  const float2 e = f2add(f2sub(a.hi, f2sub(s, bb)), f2sub(b.hi, bb));
  return ddc{s, f2add(e, f2add(a.lo, b.lo))};
}
__device__ __forceinline__ ddc csub_u(ddc a, ddc b) {
  const float2 s = f2sub(a.hi, b.hi);
  const float2 bb = f2sub(s, a.hi);
  const float2 e = f2sub(f2sub(a.hi, f2sub(s, bb)), f2add(b.hi, bb));
  return ddc{s, f2add(e, f2sub(a.lo, b.lo))};
}
__device__ __forceinline__ ddc cadd(ddc a, ddc b) {
  const ddc l = cadd_u(a, b);
  return crenorm(l.hi, l.lo);
}
__device__ __forceinline__ ddc csub(ddc a, ddc b) {
  const ddc l = csub_u(a, b);
  return crenorm(l.hi, l.lo);
}
// a b (CONJ: a conj(b)) as two double-word dot products, component 0 = a.x b.x -+ a.y b.y
// and component 1 = a.y b.x +- a.x b.y: the products of a with bx = (b.x, b.x) and of the
// swapped a = (a.y, a.x) (negated for CONJ) with ny = (-b.y, b.y), their exact rounding
// errors (FMA) and the cross terms in the low word; low word not renormalised.
template <bool CONJ>
__device__ __forceinline__ ddc cmul_bc(ddc a, float2 bxh, float2 nyh, float2 bxl, float2 nyl) {
  const float2 sh = CONJ ? make_float2(-a.hi.y, -a.hi.x) : make_float2(a.hi.y, a.hi.x);
  const float2 sl = CONJ ? make_float2(-a.lo.y, -a.lo.x) : make_float2(a.lo.y, a.lo.x);
  const float2 p = f2mul(a.hi, bxh);
  const float2 q = f2mul(sh, nyh);
  const float2 ep = f2fma(a.hi, bxh, f2neg(p));
  const float2 eq = f2fma(sh, nyh, f2neg(q));
  const float2 s = f2add(p, q);
  const float2 bb = f2sub(s, p);
  const float2 t = f2add(f2sub(p, f2sub(s, bb)), f2sub(q, bb));
  float2 lo = f2add(f2add(t, ep), eq);
  lo = f2fma(a.hi, bxl, lo);
  lo = f2fma(a.lo, bxh, lo);
  lo = f2fma(sh, nyl, lo);
  lo = f2fma(sl, nyh, lo);
  return ddc{s, lo};
}
template <bool CONJ>
__device__ __forceinline__ ddc cmul_pair(ddc a, ddc b) {
  return cmul_bc<CONJ>(a, make_float2(b.hi.x, b.hi.x), make_float2(-b.hi.y, b.hi.y),
                       make_float2(b.lo.x, b.lo.x), make_float2(-b.lo.y, b.lo.y));
}
__device__ __forceinline__ ddc cmul(ddc a, ddc b) {
  const ddc l = cmul_pair<false>(a, b);
  return crenorm(l.hi, l.lo);
}
__device__ __forceinline__ ddc cmulc(ddc a, ddc b) {
  const ddc l = cmul_pair<true>(a, b);
  return crenorm(l.hi, l.lo);
}
// the transforms' butterflies and twiddles: without renormalisation unless GNLSE_DF_LAZY
// is 0 (a two-sum of the high words stays exact for unnormalised inputs and the low words
// only accumulate over a transform's few operations per value; the next non-lazy
// operation renormalises)
__device__ __forceinline__ ddc cadd_lazy(ddc a, ddc b) { return GNLSE_DF_LAZY ? cadd_u(a, b) : cadd(a, b); }
__device__ __forceinline__ ddc csub_lazy(ddc a, ddc b) { return GNLSE_DF_LAZY ? csub_u(a, b) : csub(a, b); }
__device__ __forceinline__ ddc cmul_lazy(ddc a, ddc b) { return GNLSE_DF_LAZY ? cmul_pair<false>(a, b) : cmul(a, b); }
__device__ __forceinline__ ddc cmulc_lazy(ddc a, ddc b) { return GNLSE_DF_LAZY ? cmul_pair<true>(a, b) : cmulc(a, b); }
// a s for a double-float real s (operator* per component)
__device__ __forceinline__ ddc cscale(ddc a, ddf s) {
  const float2 sh = make_float2(s.hi, s.hi);
  const float2 p = f2mul(a.hi, sh);
  float2 e = f2fma(a.hi, sh, f2neg(p));
  e = f2fma(a.hi, make_float2(s.lo, s.lo), e);
  e = f2fma(a.lo, sh, e);
  return crenorm(p, e);
}
// |a|^2 = a.x a.x + a.y a.y: both squares paired, then one double-word sum
__device__ __forceinline__ ddf cabs2(ddc a) {
  const float2 p = f2mul(a.hi, a.hi);
  float2 e = f2fma(a.hi, a.hi, f2neg(p));
  e = f2fma(a.hi, a.lo, e);
  e = f2fma(a.lo, a.hi, e);
  const ddc q = crenorm(p, e);
  return re(q) + im(q);
}
__device__ __forceinline__ ddc cconj(ddc a) {
  return ddc{make_float2(a.hi.x, -a.hi.y), make_float2(a.lo.x, -a.lo.y)};
}
// SIGN i a
template <int SIGN>
__device__ __forceinline__ ddc cmul_i(ddc a) {
  return SIGN > 0 ? ddc{make_float2(-a.hi.y, a.hi.x), make_float2(-a.lo.y, a.lo.x)}
                  : ddc{make_float2(a.hi.y, -a.hi.x), make_float2(a.lo.y, -a.lo.x)};
}
// renormalisation after lazy operations (a full two-sum of each component: cancellation
// of the high words may leave the low word the larger); identity when the transforms
// run unnormalised (GNLSE_DF_LAZY 2)
__device__ __forceinline__ ddc cnorm(ddc a) {
#if GNLSE_DF_LAZY == 2
  return a;
#else
  const float2 s = f2add(a.hi, a.lo);
  const float2 bb = f2sub(s, a.hi);
  return ddc{s, f2add(f2sub(a.hi, f2sub(s, bb)), f2sub(a.lo, bb))};
#endif
}

}  // namespace gnlse
