// pc_ff.cuh — double-float ("float-float") arithmetic on the FP32 pipe, for
// the mixed-precision form: a value is the unevaluated sum hi + lo of two
// floats with |lo| <= ulp(hi)/2, about 48 significant bits.
//
// Built from error-free transformations: Knuth's TwoSum (The Art of Computer
// Programming vol. 2, 4.2.2), Dekker's FastTwoSum (Numer. Math. 18, 1971),
// and TwoProduct by one fused multiply-add (the exact product error
// fmaf(a, b, -a*b)); the add, multiply and divide below are the "sloppy"
// double-float forms of Dekker's paper (relative error a few units of
// 2^-48).  Every operation is an explicit round-to-nearest intrinsic
// (__fadd_rn, __fsub_rn, __fmul_rn, fmaf), which the compiler never fuses
// into a multiply-add, so the transformations stay error-free in a
// translation unit compiled with contraction on.
#pragma once

#include <cuda_runtime.h>

namespace pcg {

struct ff {
  float hi, lo;
};

// s + e = a + b exactly (any a, b).
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// s + e = a + b exactly when |a| >= |b| (or a == 0).
__device__ __forceinline__ ff fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ ff ff_of(float a) { return {a, 0.f}; }
// The double x as hi + lo (exact to about 2^-48 of x).
__device__ __forceinline__ ff ff_of(double x) {
  const float h = __double2float_rn(x);
  return {h, __double2float_rn(x - (double)h)};
}
__device__ __forceinline__ double ff_to_double(ff a) { return (double)a.hi + (double)a.lo; }
__device__ __forceinline__ float ff_to_float(ff a) { return __fadd_rn(a.hi, a.lo); }

__device__ __forceinline__ ff ff_add(ff a, ff b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  return fast_two_sum(s, e);
}
__device__ __forceinline__ ff ff_add(ff a, float b) {
  float s, e;
  two_sum(a.hi, b, s, e);
  e = __fadd_rn(e, a.lo);
  return fast_two_sum(s, e);
}
// a + b for two floats, exactly.
__device__ __forceinline__ ff ff_sum(float a, float b) {
  float s, e;
  two_sum(a, b, s, e);
  return {s, e};
}
__device__ __forceinline__ ff ff_neg(ff a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  return fast_two_sum(p, e);
}
__device__ __forceinline__ ff ff_mul(ff a, float b) {
  const float p = __fmul_rn(a.hi, b);
  float e = fmaf(a.hi, b, -p);
  e = fmaf(a.lo, b, e);
  return fast_two_sum(p, e);
}
// a * b + c
__device__ __forceinline__ ff ff_fma(ff a, ff b, ff c) { return ff_add(ff_mul(a, b), c); }

// a / b: a first quotient, then one correction from the remainder a - q b.
__device__ __forceinline__ ff ff_div(ff a, ff b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  const ff r = ff_sub(a, ff_mul(b, q1));
  const float q2 = __fdiv_rn(r.hi, b.hi);
  return fast_two_sum(q1, q2);
}

}  // namespace pcg
