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
// The double x as hi + lo (exact to about 2^-48 of x): hi = x rounded to
// float, lo = the exact remainder x - hi rounded to float.  ff_of_conv by
// the conversions and a double subtraction, which run on GB300's FP64 pipe
// at 1/64 of the FP32 rate; ff_of_fast the same bits on the integer pipe,
// without a branch, for x with 2^-72 <= |x| < 2^116 or x = 0 (ff_fast_ok):
// hi is x's 52-bit mantissa rounded to 23 bits (nearest, ties to even, a
// carry running into the exponent); the 29 bits below, less 2^29 where hi
// rounded up, are the remainder in units of 2^(e - 52), |r| <= 2^28, and
// lo = float(r) 2^(e - 52) (one integer-to-float rounding, then exact
// scalings by powers of two: lo is a normal float or zero in this range).
__device__ __forceinline__ ff ff_of_conv(double x) {
  const float h = __double2float_rn(x);
  return {h, __double2float_rn(x - (double)h)};
}
__device__ __forceinline__ bool ff_fast_ok(double x) {
  const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
  return ((hw >> 20) & 0x7ffu) - 951u <= 1138u - 951u || ((hw & 0x7fffffffu) | lw) == 0;
}
__device__ __forceinline__ ff ff_of_fast(double x) {
  const unsigned hw = (unsigned)__double2hiint(x), lw = (unsigned)__double2loint(x);
  const unsigned sign = hw & 0x80000000u, e11 = (hw >> 20) & 0x7ffu;
  const unsigned m = ((hw & 0xfffffu) << 3) | (lw >> 29);
  const unsigned r = lw & 0x1fffffffu;
  const unsigned up = (r > 0x10000000u || (r == 0x10000000u && (m & 1u))) ? 1u : 0u;
  const int ri = up ? (int)r - 0x20000000 : (int)r;
  // 2^(e11 - 1075) as 2^-64 2^(e11 - 1011)
  const float l = __fmul_rn(__fmul_rn(__int2float_rn(sign ? -ri : ri), 0x1p-64f), __uint_as_float((e11 - 884u) << 23));
  const bool zero = ((hw & 0x7fffffffu) | lw) == 0;
  return {__uint_as_float(zero ? sign : sign | (((e11 - 896u) << 23) + m + up)), zero ? 0.f : l};
}
// Either way bit for bit the same (the fast form where it applies).
__device__ __forceinline__ ff ff_of(double x) { return ff_fast_ok(x) ? ff_of_fast(x) : ff_of_conv(x); }
// f as a double, exactly: f2d_fast moves the exponent and mantissa fields
// into place on the integer pipe, without a branch, for a normal f or zero
// (f2d_fast_ok); the conversion otherwise.
__device__ __forceinline__ bool f2d_fast_ok(float f) {
  const unsigned u = __float_as_uint(f);
  return ((u >> 23) & 0xffu) - 1u < 254u || (u & 0x7fffffffu) == 0;
}
__device__ __forceinline__ double f2d_fast(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e8 = (u >> 23) & 0xffu;
  const bool zero = (u & 0x7fffffffu) == 0;
  const unsigned hw = zero ? (u & 0x80000000u) : (u & 0x80000000u) | ((e8 + 896u) << 20) | ((u & 0x7fffffu) >> 3);
  return __hiloint2double((int)hw, zero ? 0 : (int)(u << 29));
}
__device__ __forceinline__ double f2d_exact(float f) { return f2d_fast_ok(f) ? f2d_fast(f) : (double)f; }
// hi + lo rounded to double (one FP64 addition)
__device__ __forceinline__ double ff_to_double(ff a) { return f2d_exact(a.hi) + f2d_exact(a.lo); }
__device__ __forceinline__ double ff_to_double_fast(ff a) { return f2d_fast(a.hi) + f2d_fast(a.lo); }
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
