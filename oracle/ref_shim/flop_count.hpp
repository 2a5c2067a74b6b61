// flop_count.hpp — ORACLE test infrastructure (oracle/ref_build.py, the
// counting build only): a double that tallies its arithmetic.  With
// -DPC_COUNT_FLOPS, amrex::Real is pcc::CReal, so the reference's own
// hot-path sources and the oracle's equation of state and transport (templated
// on their scalar type) run the same IEEE double operations as the plain
// build, each counted once by class: add (+ and -), mul, div, fma, sqrt, exp,
// log, pow, and cmp (comparisons, min, max; not floating-point work).
// Negation, fabs and copysign are sign operations and are not counted.
// Operations evaluated at compile time (constant folding of constexpr
// constants) are not counted.  One counting run at a time (the tallies are
// process-wide).
#pragma once

#include <cmath>
#include <limits>

namespace pcc {

struct Tally {
  unsigned long long add = 0, mul = 0, div = 0, fma = 0, sqrt = 0, exp = 0, log = 0, pow = 0, cmp = 0;
};
inline Tally& tally() {
  static Tally t;
  return t;
}

#define PCC_COUNT(field)                                   \
  do {                                                     \
    if (!__builtin_is_constant_evaluated()) ++::pcc::tally().field; \
  } while (0)

struct CReal {
  double v;
  CReal() = default;
  constexpr CReal(double x) : v(x) {}
  explicit constexpr operator double() const { return v; }
  constexpr CReal& operator+=(CReal o) {
    PCC_COUNT(add);
    v += o.v;
    return *this;
  }
  constexpr CReal& operator-=(CReal o) {
    PCC_COUNT(add);
    v -= o.v;
    return *this;
  }
  constexpr CReal& operator*=(CReal o) {
    PCC_COUNT(mul);
    v *= o.v;
    return *this;
  }
  constexpr CReal& operator/=(CReal o) {
    PCC_COUNT(div);
    v /= o.v;
    return *this;
  }
};

constexpr CReal operator+(CReal a, CReal b) {
  PCC_COUNT(add);
  return CReal(a.v + b.v);
}
constexpr CReal operator-(CReal a, CReal b) {
  PCC_COUNT(add);
  return CReal(a.v - b.v);
}
constexpr CReal operator*(CReal a, CReal b) {
  PCC_COUNT(mul);
  return CReal(a.v * b.v);
}
constexpr CReal operator/(CReal a, CReal b) {
  PCC_COUNT(div);
  return CReal(a.v / b.v);
}
constexpr CReal operator-(CReal a) { return CReal(-a.v); }
constexpr CReal operator+(CReal a) { return a; }
constexpr bool operator<(CReal a, CReal b) {
  PCC_COUNT(cmp);
  return a.v < b.v;
}
constexpr bool operator>(CReal a, CReal b) {
  PCC_COUNT(cmp);
  return a.v > b.v;
}
constexpr bool operator<=(CReal a, CReal b) {
  PCC_COUNT(cmp);
  return a.v <= b.v;
}
constexpr bool operator>=(CReal a, CReal b) {
  PCC_COUNT(cmp);
  return a.v >= b.v;
}
constexpr bool operator==(CReal a, CReal b) {
  PCC_COUNT(cmp);
  return a.v == b.v;
}
constexpr bool operator!=(CReal a, CReal b) {
  PCC_COUNT(cmp);
  return a.v != b.v;
}

}  // namespace pcc

// The <cmath> functions the counted code calls, for CReal arguments.
namespace std {
inline pcc::CReal sqrt(pcc::CReal a) {
  PCC_COUNT(sqrt);
  return pcc::CReal(std::sqrt(a.v));
}
inline pcc::CReal exp(pcc::CReal a) {
  PCC_COUNT(exp);
  return pcc::CReal(std::exp(a.v));
}
inline pcc::CReal log(pcc::CReal a) {
  PCC_COUNT(log);
  return pcc::CReal(std::log(a.v));
}
inline pcc::CReal pow(pcc::CReal a, pcc::CReal b) {
  PCC_COUNT(pow);
  return pcc::CReal(std::pow(a.v, b.v));
}
inline pcc::CReal fma(pcc::CReal a, pcc::CReal b, pcc::CReal c) {
  PCC_COUNT(fma);
  return pcc::CReal(std::fma(a.v, b.v, c.v));
}
inline pcc::CReal abs(pcc::CReal a) { return pcc::CReal(std::fabs(a.v)); }
inline pcc::CReal fabs(pcc::CReal a) { return pcc::CReal(std::fabs(a.v)); }
inline pcc::CReal copysign(pcc::CReal a, pcc::CReal b) { return pcc::CReal(std::copysign(a.v, b.v)); }
inline bool isfinite(pcc::CReal a) { return std::isfinite(a.v); }
inline bool isnan(pcc::CReal a) { return std::isnan(a.v); }
inline pcc::CReal max(pcc::CReal a, double b) { return (a < b) ? pcc::CReal(b) : a; }
inline pcc::CReal max(double a, pcc::CReal b) { return (pcc::CReal(a) < b) ? b : pcc::CReal(a); }
inline pcc::CReal min(pcc::CReal a, double b) { return (pcc::CReal(b) < a) ? pcc::CReal(b) : a; }
inline pcc::CReal min(double a, pcc::CReal b) { return (b < pcc::CReal(a)) ? b : pcc::CReal(a); }

template <>
struct numeric_limits<pcc::CReal> : numeric_limits<double> {
  static constexpr pcc::CReal epsilon() noexcept { return pcc::CReal(numeric_limits<double>::epsilon()); }
  static constexpr pcc::CReal max() noexcept { return pcc::CReal(numeric_limits<double>::max()); }
  static constexpr pcc::CReal min() noexcept { return pcc::CReal(numeric_limits<double>::min()); }
  static constexpr pcc::CReal lowest() noexcept { return pcc::CReal(numeric_limits<double>::lowest()); }
  static constexpr pcc::CReal infinity() noexcept { return pcc::CReal(numeric_limits<double>::infinity()); }
  static constexpr pcc::CReal quiet_NaN() noexcept { return pcc::CReal(numeric_limits<double>::quiet_NaN()); }
};
}  // namespace std
