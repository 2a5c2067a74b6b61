// pc_exp.h — exp and log for the FP64 transport coefficients, one
// implementation compiled for the GPU kernels and for the CPU restatement
// used to check them, so that both evaluate the same IEEE operations and the
// FP64 right-hand side agrees bit for bit wherever the transport enters.
//
// exp: table-driven, after P. T. P. Tang, "Table-driven implementation of the
// exponential function in IEEE floating-point arithmetic", ACM TOMS 15(2),
// 1989: x = (64 m + j) ln2/64 + r, |r| <= ln2/128, e^x = 2^m 2^(j/64) e^r,
// with 2^(j/64) a double-double from a 64-entry table and e^r - 1 its
// degree-6 Taylor polynomial (truncation below 5e-20 relative).  12 FP64
// operations against about 15 for the CUDA library exp on this GPU.
//
// log: table-driven in the manner of Tang, "Table-driven implementation of the
// logarithm function in IEEE floating-point arithmetic", ACM TOMS 16(4), 1990:
// x = 2^m f, F = 1 + j/128 nearest to f, log x = m ln2 + log F + log1p(u),
// u = (f - F)/F (|u| <= 1/256), log1p by its degree-7 series, with ln2 and
// log F split so that m ln2_hi + log(F)_hi is exact.
//
// Both are within one ulp of the correctly rounded result (tests compare them
// with 60-digit decimal arithmetic).  Arguments outside their fast ranges
// (|x| >= 700 for exp; zero, negative, subnormal, infinite or NaN for log)
// go to the C library function.  The tables are generated by
// gen_exp_tables.py.
#pragma once

#include <math.h>
#include <stdint.h>
#include <string.h>

#include "pc_exp_tables.h"

#if defined(__CUDACC__)
#define PC_MATH_HD __host__ __device__ __forceinline__
#else
#define PC_MATH_HD inline
#endif

namespace pc_math {

#if defined(__CUDACC__)
static __device__ const double d_exp_hi[64] = PC_EXP_TABLE_HI;
static __device__ const double d_exp_lo[64] = PC_EXP_TABLE_LO;
static __device__ const double d_log_inv[129] = PC_LOG_TABLE_INV;
static __device__ const double d_log_hi[129] = PC_LOG_TABLE_HI;
static __device__ const double d_log_lo[129] = PC_LOG_TABLE_LO;
#endif
static const double h_exp_hi[64] = PC_EXP_TABLE_HI;
static const double h_exp_lo[64] = PC_EXP_TABLE_LO;
static const double h_log_inv[129] = PC_LOG_TABLE_INV;
static const double h_log_hi[129] = PC_LOG_TABLE_HI;
static const double h_log_lo[129] = PC_LOG_TABLE_LO;

PC_MATH_HD int64_t bits_of(double x) {
#if defined(__CUDA_ARCH__)
  return __double_as_longlong(x);
#else
  int64_t b;
  memcpy(&b, &x, sizeof b);
  return b;
#endif
}

PC_MATH_HD double double_of(int64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(b);
#else
  double x;
  memcpy(&x, &b, sizeof x);
  return x;
#endif
}

// Table entry: from global memory through the read-only cache on the GPU.
#if defined(__CUDA_ARCH__)
#define PC_MATH_TAB(name, j) __ldg(::pc_math::d_##name + (j))
#else
#define PC_MATH_TAB(name, j) (::pc_math::h_##name[(j)])
#endif

PC_MATH_HD double exp(double x) {
  if (!((bits_of(x) & INT64_C(0x7fffffffffffffff)) < bits_of(700.0))) return ::exp(x);  // |x| < 700 (NaN: no)
  const double shifter = 0x1.8p52;  // adding it rounds |x 64/ln2| < 2^51 to an integer
  const double t = fma(x, PC_EXP_64_LN2, shifter);
  const int k = (int)(int32_t)(uint32_t)(uint64_t)bits_of(t);  // that integer, from the low word
  const double kd = t - shifter;
  double r = fma(-kd, PC_EXP_LN2_64_HI, x);  // exact: kd ln2_hi has at most 48 bits
  r = fma(-kd, PC_EXP_LN2_64_LO, r);
  const double r2 = r * r;
  double q = fma(r, 1.0 / 720.0, 1.0 / 120.0);
  q = fma(q, r, 1.0 / 24.0);
  q = fma(q, r, 1.0 / 6.0);
  q = fma(q, r, 0.5);
  const double p = fma(r2, q, r);  // e^r - 1
  const int j = k & 63;
  const int m = (k - j) / 64;
  const double th = PC_MATH_TAB(exp_hi, j);
  const double s = th + fma(th, p, PC_MATH_TAB(exp_lo, j));  // 2^(j/64) e^r, in [0.99, 2.02)
  return double_of(bits_of(s) + (int64_t)m * ((int64_t)1 << 52));  // times 2^m: stays normal for |x| < 700
}

PC_MATH_HD double log(double x) {
  const int64_t b = bits_of(x);
  if (!(b >= INT64_C(0x0010000000000000) && b <= INT64_C(0x7fefffffffffffff))) return ::log(x);  // positive normal x
  const int m = (int)(b >> 52) - 1023;
  const int64_t mant = b & (((int64_t)1 << 52) - 1);
  const double f = double_of(mant | ((int64_t)1023 << 52));            // in [1, 2)
  const int j = (int)((mant + ((int64_t)1 << 44)) >> 45);              // nearest j/128 to f - 1, 0..128
  const double F = double_of((INT64_C(1023) << 52) + ((int64_t)j << 45));  // 1 + j/128, exactly
  const double d = f - F;                                                // exact
  const double iF = PC_MATH_TAB(log_inv, j);
  const double u = d * iF;
  const double ul = fma(-u, F, d) * iF;                                  // u + ul = d / F to ~2^-106
  double q = fma(u, 1.0 / 7.0, -1.0 / 6.0);
  q = fma(q, u, 1.0 / 5.0);
  q = fma(q, u, -0.25);
  q = fma(q, u, 1.0 / 3.0);
  q = fma(q, u, -0.5);
  const double lo = fma((double)m, PC_LOG_LN2_LO, PC_MATH_TAB(log_lo, j)) + (ul + (u * u) * q);
  const double hi = fma((double)m, PC_LOG_LN2_HI, PC_MATH_TAB(log_hi, j));  // exact: both on the 2^-42 grid
  const double s = hi + u;  // hi + u = s + e exactly (Knuth's TwoSum)
  const double bv = s - hi;
  const double e = (hi - (s - bv)) + (u - bv);
  return s + (e + lo);
}

}  // namespace pc_math
