// pc_dual.cuh — dual numbers (value, tangent) for the forward-mode tangent
// of the RHS: the forward device code is templated on its scalar type, and
// instantiated with Dual it carries d(quantity)/d(direction) alongside every
// value.  The value part of each operation is the same IEEE operation the
// FP64 forward performs (this header is used in translation units compiled
// without multiply-add contraction), so a Dual evaluation takes exactly the
// forward's branches and reproduces its values bit for bit.
#pragma once

#include <cuda_runtime.h>

#include "pc_exp.h"

namespace pcg {

// The double overloads stay visible next to the Dual ones.
using ::copysign;
using ::exp;
using ::fabs;
using ::fma;
using ::fmax;
using ::fmin;
using ::log;
using ::sqrt;

struct Dual {
  double v, d;
  __host__ __device__ Dual() : v(0.0), d(0.0) {}
  __host__ __device__ Dual(double x) : v(x), d(0.0) {}  // constants
  __host__ __device__ Dual(double x, double dx) : v(x), d(dx) {}
};

__device__ __forceinline__ double val(double x) { return x; }
__device__ __forceinline__ double val(const Dual& x) { return x.v; }

__device__ __forceinline__ Dual operator-(const Dual& a) { return Dual(-a.v, -a.d); }
__device__ __forceinline__ Dual operator+(const Dual& a, const Dual& b) { return Dual(a.v + b.v, a.d + b.d); }
__device__ __forceinline__ Dual operator-(const Dual& a, const Dual& b) { return Dual(a.v - b.v, a.d - b.d); }
__device__ __forceinline__ Dual operator*(const Dual& a, const Dual& b) { return Dual(a.v * b.v, a.v * b.d + a.d * b.v); }
__device__ __forceinline__ Dual operator/(const Dual& a, const Dual& b) {
  const double q = a.v / b.v;
  return Dual(q, (a.d - q * b.d) / b.v);
}
__device__ __forceinline__ Dual operator+(const Dual& a, double b) { return Dual(a.v + b, a.d); }
__device__ __forceinline__ Dual operator+(double a, const Dual& b) { return Dual(a + b.v, b.d); }
__device__ __forceinline__ Dual operator-(const Dual& a, double b) { return Dual(a.v - b, a.d); }
__device__ __forceinline__ Dual operator-(double a, const Dual& b) { return Dual(a - b.v, -b.d); }
__device__ __forceinline__ Dual operator*(const Dual& a, double b) { return Dual(a.v * b, a.d * b); }
__device__ __forceinline__ Dual operator*(double a, const Dual& b) { return Dual(a * b.v, a * b.d); }
__device__ __forceinline__ Dual operator/(const Dual& a, double b) { return Dual(a.v / b, a.d / b); }
__device__ __forceinline__ Dual operator/(double a, const Dual& b) {
  const double q = a / b.v;
  return Dual(q, -q * b.d / b.v);
}
__device__ __forceinline__ Dual& operator+=(Dual& a, const Dual& b) { return a = a + b; }
__device__ __forceinline__ Dual& operator-=(Dual& a, const Dual& b) { return a = a - b; }
__device__ __forceinline__ Dual& operator*=(Dual& a, const Dual& b) { return a = a * b; }

#define PCG_DUAL_CMP(op)                                                                                      \
  __device__ __forceinline__ bool operator op(const Dual& a, const Dual& b) { return a.v op b.v; }          \
  __device__ __forceinline__ bool operator op(const Dual& a, double b) { return a.v op b; }                 \
  __device__ __forceinline__ bool operator op(double a, const Dual& b) { return a op b.v; }
PCG_DUAL_CMP(<)
PCG_DUAL_CMP(>)
PCG_DUAL_CMP(<=)
PCG_DUAL_CMP(>=)
PCG_DUAL_CMP(==)
PCG_DUAL_CMP(!=)
#undef PCG_DUAL_CMP

__device__ __forceinline__ Dual fma(const Dual& a, const Dual& b, const Dual& c) {
  return Dual(::fma(a.v, b.v, c.v), a.v * b.d + a.d * b.v + c.d);
}
__device__ __forceinline__ Dual fma(double a, const Dual& b, const Dual& c) {
  return Dual(::fma(a, b.v, c.v), a * b.d + c.d);
}
__device__ __forceinline__ Dual fma(const Dual& a, double b, const Dual& c) {
  return Dual(::fma(a.v, b, c.v), a.d * b + c.d);
}
__device__ __forceinline__ Dual fma(const Dual& a, const Dual& b, double c) {
  return Dual(::fma(a.v, b.v, c), a.v * b.d + a.d * b.v);
}
__device__ __forceinline__ Dual fma(double a, double b, const Dual& c) { return Dual(::fma(a, b, c.v), c.d); }
__device__ __forceinline__ Dual fma(const Dual& a, double b, double c) { return Dual(::fma(a.v, b, c), a.d * b); }
__device__ __forceinline__ Dual fma(double a, const Dual& b, double c) { return Dual(::fma(a, b.v, c), a * b.d); }

// min/max/|x|: the derivative of the argument the value selects.
__device__ __forceinline__ Dual fmax(const Dual& a, const Dual& b) { return (::fmax(a.v, b.v) == a.v) ? a : b; }
__device__ __forceinline__ Dual fmin(const Dual& a, const Dual& b) { return (::fmin(a.v, b.v) == a.v) ? a : b; }
__device__ __forceinline__ Dual fmax(double a, const Dual& b) {
  const double m = ::fmax(a, b.v);
  return (m == b.v && !(a > b.v)) ? b : Dual(m);
}
__device__ __forceinline__ Dual fmax(const Dual& a, double b) { return fmax(b, a); }
__device__ __forceinline__ Dual fmin(double a, const Dual& b) {
  const double m = ::fmin(a, b.v);
  return (m == b.v && !(a < b.v)) ? b : Dual(m);
}
__device__ __forceinline__ Dual fmin(const Dual& a, double b) { return fmin(b, a); }
__device__ __forceinline__ Dual fabs(const Dual& a) { return (a.v < 0.0) ? -a : a; }
__device__ __forceinline__ double copysign(double a, const Dual& b) { return ::copysign(a, b.v); }

__device__ __forceinline__ Dual sqrt(const Dual& a) {
  const double s = ::sqrt(a.v);
  return Dual(s, (s > 0.0) ? a.d / (2.0 * s) : 0.0);
}
// The transport's exp and log (pc_exp.h) on dual numbers.
__device__ __forceinline__ Dual pc_exp(const Dual& a) {
  const double e = ::pc_math::exp(a.v);
  return Dual(e, e * a.d);
}
__device__ __forceinline__ Dual pc_log(const Dual& a) { return Dual(::pc_math::log(a.v), a.d / a.v); }

}  // namespace pcg
