// pc_device.cuh — device-side physics of the MOL right-hand side (sm_103a).
//
// Pointwise pieces of PeleC's getMOLSrcTerm path, restructured for a GPU
// whose FP64 pipe is the binding resource (GB300: ~1.2 TFLOP/s FP64 against
// ~74 TFLOP/s FP32): species sums are contracted into mixture polynomial
// coefficients once per state, reciprocals replace repeated divisions, and
// dead EOS evaluations of the reference are skipped.  Each function names the
// reference code whose result it reproduces.
#pragma once

#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include <type_traits>

#include "pc_exp.h"

// A translation unit may compile this code a second time with quotients by a
// shared divisor taken as products with its reciprocal (PCG_RECIPROCAL_QUOTIENTS,
// see div_by); it then names its namespace differently (PCG_NAMESPACE), so
// that the two compilations of the same templates never meet at link time.
#ifndef PCG_NAMESPACE
#define PCG_NAMESPACE pcg
#endif

namespace PCG_NAMESPACE {

constexpr double RU = 8.31446261815324e7;  // erg/(mol K)

// Conserved and primitive indices, Source/IndexDefines.H:6-23.
enum { URHO = 0, UMX = 1, UMY = 2, UMZ = 3, UEDEN = 4, UEINT = 5, UTEMP = 6, UFS = 7 };

// Source/Constants.H:10-24.
constexpr double kSmallU = 1.0e-12;
constexpr double kSmallNum = 1.0e-8;
#define PCG_VERY_SMALL_NUM (2.220446049250313e-16 * 1e-100)

// Device copy of the species data in the form the kernels evaluate.
// NASA-7 coefficients are folded with R/W_k: cpc[r][n][k] = (R/W_k) a_{n,k}
// for n = 0..5, r = 0 below tmid and 1 above.
template <int NS>
struct DevMech {
  double rW[NS];     // R / W_k
  double irW[NS];    // rcp_q(R / W_k): the shared divisor's reciprocal of W_k / Wbar
  double gamma, gm1; // GammaLaw
  double cpk[NS];    // GammaLaw cp_k = gamma/(gamma-1) R/W_k
  double tmid;
  double cpc[2][6][NS];
  double visc[NS][4], cond[NS][4], bulk[NS];
  double diff[(NS * (NS - 1)) / 2 + 1][4];  // pairs k<j in row order
  double inv_pref;                          // 1 / diff_pref
  double const_mu, const_xi, const_lam, const_rhoD;
};

// Operator flags (static PeleC parameters read by getMOLSrcTerm).
struct DevFlags {
  int do_hydro, diffuse_vel, diffuse_temp, diffuse_spec, diffuse_enth;
  int slopes;  // plm_iorder != 1
  int laxf, harmonic, check_output, newton_maxit;
};

// The FP64 arithmetic below is a fixed sequence of IEEE operations: explicit
// fma() where a fused multiply-add is meant, and otherwise separate, correctly
// rounded multiplies, adds, divisions and square roots (this translation unit
// is compiled without multiply-add contraction).  The CPU restatement used
// to check the kernels evaluates the same sequence.

// Runs f() on the lanes where need holds, inside a branch that a warp takes
// only if one of its lanes needs it, so that rare paths cost nothing in warps
// where no lane needs them.  The empty volatile asm keeps the compiler from
// evaluating the path's FP64 operations speculatively on every lane (code
// without side effects may otherwise be executed ahead of its branch).
template <class F>
__device__ __forceinline__ void rare_for_warp(bool need, F&& f) {
  if (__any_sync(__activemask(), need)) {
    if (need) {
      asm volatile("");
      f();
    }
  }
}

// The reciprocal y of a shared divisor b that div_fast and div_by expect:
// 1/b rounded toward zero (in the PC_PRECISION_FP64_RCP compilation, 1/b
// rounded to nearest, whose product with a is the quotient of that form).
__device__ __forceinline__ double rcp_q(double b) {
#ifdef PCG_RECIPROCAL_QUOTIENTS
  return 1.0 / b;
#else
  return __drcp_rz(b);
#endif
}

// rcp_q(b) from r = 1.0 / b (rounded to nearest) where that is at hand: r
// stepped one ulp toward zero (its bit pattern decremented) where r b > 1,
// decided by one fused multiply-add.  Operands that make r infinite, zero or
// NaN are the ones div_fast sends to a real division anyway.
__device__ __forceinline__ double rcp_q_from_rn(double b, double r) {
#ifdef PCG_RECIPROCAL_QUOTIENTS
  (void)b;
  return r;
#else
  const long long e = __double_as_longlong(fma(r, b, -1.0));
  return (e > 0) ? __longlong_as_double(__double_as_longlong(r) - 1) : r;
#endif
}

// a / b, correctly rounded, for a divisor b shared by several quotients, given
// y = rcp_q(b) (1/b rounded toward zero), without a branch: the result for
// the common operands, with slow set for the rare ones that need a real
// division (the caller then evaluates again with exact_quotient, see Quot).
//
// q0 = a y rounded toward zero is at most the quotient in magnitude and
// within four ulps of it (y and the product each lose less than an ulp), so
// the correctly rounded quotient is q0 + s ulp(q0) for some s in [0, 4].
// s is decided exactly in integer arithmetic on the significands, off the
// FP64 pipe (the binding resource on GB300, which runs integer instructions
// at 32-64 times its FP64 rate): with a = A 2^(ea-1075), b = B 2^(eb-1075)
// and q0 = M 2^(eq-1075) (A, B, M the 53-bit significands),
//   R = A 2^k - B M,   k = ea - eb - eq + 1075 (51 <= k <= 55),
// equals (|a/b| - |q0|) / ulp(q0) times B, 0 <= R < 4B < 2^55, so it is exact
// modulo 2^64; and as k >= 32, A 2^k mod 2^64 depends only on A's low word.
// s counts the half-integers 1/2 .. 7/2 that R/B exceeds (a quotient of two
// doubles is never exactly halfway between two doubles, so there are no
// ties), and s ulp is added to q0's bit pattern.  One FP64 multiply instead
// of a division.  Rounding toward zero keeps the quotient on q0's side of
// any power of two below it; above it (q0 within 4 ulp of the next power of
// two P = q0 + d ulp and s > d) the doubles are 2 ulp apart, and the
// quotient, less than 3 ulp above P, rounds to P or to P + 2 ulp.  A zero
// numerator gives a*y, the correctly signed zero.
// Slow: a nonzero numerator that is subnormal, infinite or NaN; b zero,
// subnormal, infinite, NaN or above 2^1022 (1/b not a normal number); q0
// outside [2^-1021, 2^1022) (the quotient or its neighbours not normal); or
// R < 0 (y not rounded toward zero).  For a zero numerator only b zero or
// subnormal (1/b infinite).
__device__ __forceinline__ double div_fast(double a, double b, double y, bool& slow) {
#ifdef PCG_RECIPROCAL_QUOTIENTS
  // The PC_PRECISION_FP64_RCP compilation: a y = a/b (1 + e) with
  // |e| <= 2^-52 + 2^-106, within one ulp of the correctly rounded quotient.
  (void)b;
  (void)slow;
  return a * y;
#else
  const double q0 = __dmul_rz(a, y);
  const unsigned ah = (unsigned)__double2hiint(a), al = (unsigned)__double2loint(a);
  const unsigned bh = (unsigned)__double2hiint(b), bl = (unsigned)__double2loint(b);
  const unsigned qh = (unsigned)__double2hiint(q0), ql = (unsigned)__double2loint(q0);
  const unsigned ea = (ah >> 20) & 0x7ffu, eb = (bh >> 20) & 0x7ffu, eq = (qh >> 20) & 0x7ffu;
  const unsigned sh = (ea - eb - eq + 1043u) & 31u;  // k - 32
  const unsigned Bh = (bh & 0xfffffu) | 0x100000u, Mh = (qh & 0xfffffu) | 0x100000u;
  const unsigned long long p = (unsigned long long)bl * ql;  // B M mod 2^64 = p + (bl Mh + Bh ql) 2^32
  const unsigned phi = (unsigned)(p >> 32) + bl * Mh + Bh * ql;
  const long long R = (long long)(((unsigned long long)(al << sh) << 32) - (((unsigned long long)phi << 32) | (unsigned)p));
  const long long Bs = (long long)(((unsigned long long)Bh << 32) | bl), R2 = 2 * R;
  int st = (int)(R2 > Bs) + (int)(R2 > 3 * Bs) + (int)(R2 > 5 * Bs) + (int)(R2 > 7 * Bs);
  // q0 = P - d ulp below a power of two P (d = 1..4) and s > d: P, or P + 2 ulp
  // (the next double up) if the quotient is an ulp or more above P.
  const int d = (int)(0xffffffffu - ql) + 1;
  if ((qh & 0xfffffu) == 0xfffffu && ql >= 0xfffffffcu && st > d) st = d + (int)(R >= (long long)(d + 1) * Bs);
  const bool zero = ((ah << 1) | al) == 0u;
  slow |= zero ? (eb == 0u) : (ea - 1u > 2045u || eb - 1u > 2043u || eq - 2u > 2043u || R < 0);
  const unsigned long long iq = ((unsigned long long)qh << 32) | ql;
  return zero ? q0 : __longlong_as_double((long long)(iq + (unsigned long long)(long long)st));
#endif
}

// a / b by IEEE division (a y in the PC_PRECISION_FP64_RCP compilation).
__device__ __forceinline__ double exact_quotient(double a, double b, double y) {
#ifdef PCG_RECIPROCAL_QUOTIENTS
  (void)b;
  return a * y;
#else
  (void)y;
  return a / b;
#endif
}

// a / b, correctly rounded, for a divisor b shared by several quotients, given
// y = rcp_q(b): div_fast, with the rare operands divided in a branch that only
// warps containing one take.
__device__ __forceinline__ double div_by(double a, double b, double y) {
  bool slow = false;
  double q = div_fast(a, b, y, slow);
  rare_for_warp(slow, [&] { q = exact_quotient(a, b, y); });
  return q;
}

// Quotient policies.  Quot<false> divides with div_fast and records in
// .slow whether any operand needed a real division; a pass evaluated that
// way counts such lanes, and an exact twin of the pass (Quot<true>: IEEE
// division), launched after it, evaluates everything again when the count is
// not zero.  The fast pass thus has no branch per quotient, and the compiler
// can interleave the integer work of neighbouring quotients.  QuotSelf
// (div_by: rare operands divided in a per-warp branch) serves passes without
// an exact twin.  The dual numbers of the tangent have their own div_fast,
// exact_quotient and div_by (pc_tangent.cuh), found by argument lookup.
template <bool kExact>
struct Quot;
template <>
struct Quot<false> {
  bool slow = false;
  template <class R>
  __device__ __forceinline__ R operator()(const R& a, const R& b, const R& y) {
    return div_fast(a, b, y, slow);
  }
  __device__ __forceinline__ double operator()(double a, double b, double y) { return div_fast(a, b, y, slow); }
};
template <>
struct Quot<true> {
  bool slow = false;
  template <class R>
  __device__ __forceinline__ R operator()(const R& a, const R& b, const R& y) {
    return exact_quotient(a, b, y);
  }
  __device__ __forceinline__ double operator()(double a, double b, double y) { return exact_quotient(a, b, y); }
};
struct QuotSelf {
  bool slow = false;
  template <class R>
  __device__ __forceinline__ R operator()(const R& a, const R& b, const R& y) {
    return div_by(a, b, y);
  }
};

// Exact binary scalings on the bit patterns (integer pipe).  Multiplying by
// 0.5 or 2 is exact except where the result leaves the normal range, and
// those cases are rounded here as IEEE multiplication rounds them, so the
// results equal 0.5 * x and 2 * |x| bit for bit.
__device__ __forceinline__ unsigned long long dbits(double x) { return (unsigned long long)__double_as_longlong(x); }
__device__ __forceinline__ double dfrom(unsigned long long b) { return __longlong_as_double((long long)b); }

// 0.5 * x (R = double: integer form; other scalar types multiply).
template <class R>
__device__ __forceinline__ R halve(R x) {
  return 0.5 * x;
}
template <>
__device__ __forceinline__ double halve<double>(double x) {
  const unsigned long long b = dbits(x), sgn = b & 0x8000000000000000ULL, mag = b ^ sgn;
  const unsigned e = (unsigned)(mag >> 52);
  unsigned long long r;
  if (e >= 2u)
    r = (e == 0x7ffu) ? mag : mag - (1ULL << 52);  // normal result (infinities and NaNs unchanged)
  else
    r = (mag >> 1) + (mag & (mag >> 1) & 1ULL);  // subnormal result: halve the integer significand, ties to even
  return dfrom(r | sgn);
}

// 2 * m for the bit pattern m of a non-negative double.
__device__ __forceinline__ unsigned long long twice_mag(unsigned long long m) {
  const unsigned e = (unsigned)(m >> 52);
  if (e == 0u) return m << 1;                                 // zero or subnormal: exact (may become normal)
  if (e >= 0x7feu) return e == 0x7ffu ? m : 0x7ff0000000000000ULL;  // inf/NaN unchanged; overflow to inf
  return m + (1ULL << 52);
}

// max(c, x) for a constant c >= 0, as std::max(c, x) = (c < x) ? x : c
// evaluates it (R = double: on the bit patterns; a negative, -0 or NaN x
// gives c).
template <class R>
__device__ __forceinline__ R fmax_pos(R x, double c) {
  return fmax(x, c);
}
template <>
__device__ __forceinline__ double fmax_pos<double>(double x, double c) {
  const long long ix = __double_as_longlong(x), ic = __double_as_longlong(c);
  return (ix > ic && ix <= 0x7ff0000000000000LL) ? x : c;
}

// 0 where -c < x < c (c > 0), else x (R = double: |x| < c compared on the
// bit patterns, false for a NaN like the floating-point comparison).
template <class R>
__device__ __forceinline__ R zero_below(R x, double c) {
  return (-c < x && x < c) ? R(0.0) : x;
}
template <>
__device__ __forceinline__ double zero_below<double>(double x, double c) {
  return (dbits(x) & 0x7fffffffffffffffULL) < dbits(c) ? 0.0 : x;
}

// copysign(1, s) * x (R = double: x with its sign bit flipped where s is
// negative, which is what the multiplication by +-1 gives).
template <class R>
__device__ __forceinline__ R signed_by(R x, R s) {
  return copysign(1.0, s) * x;
}
template <>
__device__ __forceinline__ double signed_by<double>(double x, double s) {
  return dfrom(dbits(x) ^ (dbits(s) & 0x8000000000000000ULL));
}

// exp and log of the transport fits: pc_exp.h's table-driven functions, the
// ones the CPU restatement evaluates too (the Dual overloads are in
// pc_dual.cuh).
__device__ __forceinline__ double pc_exp(double x) { return pc_math::exp(x); }
__device__ __forceinline__ double pc_log(double x) { return pc_math::log(x); }

// The functions below are templates on the scalar type R: double for the
// RHS, Dual (pc_dual.cuh) for its forward-mode tangent.
template <class R>
__device__ __forceinline__ R horner4(const double c[4], R L) {
  return fma(L, fma(L, fma(L, c[3], c[2]), c[1]), c[0]);
}

// R/Wbar = sum_k Y_k R/W_k.
template <int NS, class R>
__device__ __forceinline__ R mix_rw(const DevMech<NS>& m, const R* Y) {
  R s = 0.0;
#pragma unroll
  for (int k = 0; k < NS; ++k) s = fma(Y[k], m.rW[k], s);
  return s;
}

// Y2X: X_k = Y_k (R/W_k) / (R/Wbar).
template <int NS, class R, class Q>
__device__ __forceinline__ void y2x(const DevMech<NS>& m, const R* Y, R rw, R* X, Q& q) {
  const R irw = rcp_q(rw);
#pragma unroll
  for (int k = 0; k < NS; ++k) X[k] = q(Y[k] * m.rW[k], rw, irw);  // = Y_k (R/W_k) / rw
}
template <int NS, class R>
__device__ __forceinline__ void y2x(const DevMech<NS>& m, const R* Y, R rw, R* X) {
  QuotSelf q;
  y2x(m, Y, rw, X, q);
}

// ---------------------------------------------------------------------------
// GammaLaw EOS (calorically perfect gas).
// ---------------------------------------------------------------------------
template <int NS>
struct GammaLawEos {
  static constexpr bool kIdealMix = false;
  // REY2T: T = e (gamma-1) / (R/Wbar).
  template <class R>
  __device__ static R rey2t(const DevMech<NS>& m, const R* /*Y*/, R rw, R e, double /*Tguess*/, int /*maxit*/,
                            bool& ok) {
    ok = true;
    return e * m.gm1 / rw;
  }
  // RPY2Cs / RTY2Cs: c = sqrt(gamma p / rho).
  template <class R>
  __device__ static R cs_rp(const DevMech<NS>& m, const R*, R, R rho, R p) {
    return sqrt(m.gamma * p / rho);
  }
  template <class R>
  __device__ static R cs_T(const DevMech<NS>& m, const R*, R, R rho, R /*T*/, R p) {
    return sqrt(m.gamma * p / rho);
  }
  // RYP2E: e = p / ((gamma-1) rho).
  template <class R>
  __device__ static R e_rp(const DevMech<NS>& m, const R*, R, R rho, R p) {
    return p / (m.gm1 * rho);
  }
  // T2Hi: h_k = cp_k T.
  template <class R>
  __device__ static void hi(const DevMech<NS>& m, R T, R* h) {
#pragma unroll
    for (int k = 0; k < NS; ++k) h[k] = m.cpk[k] * T;
  }
};

// ---------------------------------------------------------------------------
// Ideal-gas mixture with NASA-7 species thermodynamics, one range split tmid.
// Mixture coefficients C_n = sum_k Y_k (R/W_k) a_{n,k}; then
//   cv(T) = (C0 - rw) + T (C1 + T (C2 + T (C3 + T C4)))
//   e(T)  = C5 + T ((C0 - rw) + T (C1/2 + T (C2/3 + T (C3/4 + T C4/5)))).
// ---------------------------------------------------------------------------
template <int NS>
struct IdealMixEos {
  static constexpr bool kIdealMix = true;
  template <class R>
  __device__ static int range(const DevMech<NS>& m, R T) {
    return (T < m.tmid) ? 0 : 1;
  }
  template <int NC = 6, class R>
  __device__ static void coefs(const DevMech<NS>& m, const R* Y, int r, R C[6]) {
#pragma unroll
    for (int n = 0; n < NC; ++n) {
      R s = 0.0;
#pragma unroll
      for (int k = 0; k < NS; ++k) s = fma(Y[k], m.cpc[r][n][k], s);
      C[n] = s;
    }
  }
  template <class R>
  __device__ static R cv_of(const R C[6], R rw, R T) {
    return (C[0] - rw) + T * fma(T, fma(T, fma(T, C[4], C[3]), C[2]), C[1]);
  }
  template <class R>
  __device__ static R e_of(const R C[6], R rw, R T) {
    const R p = fma(T, fma(T, fma(T, fma(T, C[4] * 0.2, C[3] * 0.25), C[2] * (1.0 / 3.0)), C[1] * 0.5), C[0] - rw);
    return fma(T, p, C[5]);
  }
  // REY2T: Newton's method on e(T) = e from the guess U(UTEMP)
  // (Utilities.H:285).  Steps clamped to +-1000 K, T >= 10 K, stop once
  // |T_new - T| <= 1e-12 T_new; ok=false after maxit iterations.
  __device__ static double rey2t(const DevMech<NS>& m, const double* Y, double rw, double ein, double Tguess,
                                 int maxit, bool& ok) {
    double t = Tguess;
    if (!(t > 0.0) || !isfinite(t)) t = 1000.0;
    int r = range(m, t);
    double C[6];
    coefs(m, Y, r, C);
    ok = false;
    for (int it = 0; it < maxit; ++it) {
      const int rn = range(m, t);
      if (rn != r) {
        r = rn;
        coefs(m, Y, r, C);
      }
      const double e = e_of(C, rw, t);
      const double cv = cv_of(C, rw, t);
      double dt = (ein - e) / cv;
      if (dt > 1000.0) dt = 1000.0;
      if (dt < -1000.0) dt = -1000.0;
      double tn = t + dt;
      if (tn < 10.0) tn = 10.0;
      const bool conv = fabs(tn - t) <= 1e-12 * tn;
      t = tn;
      if (conv) {
        ok = true;
        break;
      }
    }
    return t;
  }
  // c^2 = (cp/cv) p / rho, cp = cv + R/Wbar, at temperature T.
  template <class R>
  __device__ static R cs_T(const DevMech<NS>& m, const R* Y, R rw, R rho, R T, R p) {
    R C[6];
    coefs<5>(m, Y, range(m, T), C);
    const R cv = cv_of(C, rw, T);
    return sqrt((cv + rw) * p / (cv * rho));
  }
  // RPY2Cs: T = p / (rho R/Wbar).
  template <class R>
  __device__ static R cs_rp(const DevMech<NS>& m, const R* Y, R rw, R rho, R p) {
    return cs_T(m, Y, rw, rho, p / (rho * rw), p);
  }
  // RYP2E.
  template <class R>
  __device__ static R e_rp(const DevMech<NS>& m, const R* Y, R rw, R rho, R p) {
    const R T = p / (rho * rw);
    R C[6];
    coefs(m, Y, range(m, T), C);
    return e_of(C, rw, T);
  }
  // T2Hi: h_k = c5 + T (c0 + T (c1/2 + T (c2/3 + T (c3/4 + T c4/5)))), c = (R/W_k) a.
  template <class R>
  __device__ static void hi(const DevMech<NS>& m, R T, R* h) {
    const int r = range(m, T);
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const R p = fma(T, fma(T, fma(T, fma(T, m.cpc[r][4][k] * 0.2, m.cpc[r][3][k] * 0.25),
                                           m.cpc[r][2][k] * (1.0 / 3.0)),
                                  m.cpc[r][1][k] * 0.5),
                           m.cpc[r][0][k]);
      h[k] = fma(T, p, m.cpc[r][5][k]);
    }
  }
};

// ---------------------------------------------------------------------------
// Transport (pc_transcoeff, Source/TransCoeff.H:7-37).
// out layout: rhoD[NS], mu, xi, lambda (dComp_* of IndexDefines.H:39-42).
// ---------------------------------------------------------------------------
template <int NS>
struct ConstantTransport {
  template <class R, class Q = QuotSelf>
  __device__ static void eval(const DevMech<NS>& m, R, R, R, const R*, const R*, R* out, Q&& = Q()) {
#pragma unroll
    for (int k = 0; k < NS; ++k) out[k] = m.const_rhoD;
    out[NS] = m.const_mu;
    out[NS + 1] = m.const_xi;
    out[NS + 2] = m.const_lam;
  }
};

// Mixture-averaged transport (Docs/sphinx/Algorithms.rst:540-566):
// mu = (sum X mu_k^6)^(1/6), lambda = (sum X lambda_k^(1/4))^4,
// xi = sum X bulk_k mu_k, rhoD_k = rho (W_k/Wbar) (1-Y_k) /
// sum_{j!=k} max(X_j,1e-15) / D_kj(T,p) (Hirschfelder-Curtiss mass flux
// rhoD_k grad X_k), 1/D_kj(T,p) = exp(-fit_kj(ln T)) p / p_ref.
template <int NS>
struct SimpleTransport {
  template <class R, class Q = QuotSelf>
  __device__ static void eval(const DevMech<NS>& m, R T, R rho, R p, const R* Y, const R* X, R* out,
                              Q&& q = Q()) {
    const R L = pc_log(T);
    R smu = 0.0, slam = 0.0, sxi = 0.0;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const R mk = pc_exp(horner4(m.visc[k], L));
      const R m2 = mk * mk;
      smu = fma(X[k], m2 * m2 * m2, smu);
      slam = fma(X[k], pc_exp(0.25 * horner4(m.cond[k], L)), slam);
      sxi = fma(X[k], m.bulk[k] * mk, sxi);
    }
    R s[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) s[k] = 0.0;
    const R pr = p * m.inv_pref;
    int pq = 0;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
#pragma unroll
      for (int j = k + 1; j < NS; ++j, ++pq) {
        const R invD = pc_exp(-horner4(m.diff[pq], L)) * pr;
        s[k] = fma(fmax_pos(X[j], 1e-15), invD, s[k]);
        s[j] = fma(fmax_pos(X[k], 1e-15), invD, s[j]);
      }
    }
    const R rw = mix_rw<NS>(m, Y);
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const R wrat = q(rw, R(m.rW[k]), R(m.irW[k]));  // W_k / Wbar, correctly rounded
      out[k] = (s[k] > 0.0) ? rho * (1.0 - Y[k]) * wrat / s[k] : 0.0;
    }
    out[NS] = pc_exp(pc_log(smu) * (1.0 / 6.0));
    out[NS + 1] = sxi;
    const R l2 = slam * slam;
    out[NS + 2] = l2 * l2;
  }
};

// pc_move_transcoefs_to_ec, Source/Utilities.H:322-342.
template <class R>
__device__ __forceinline__ R twice_pos(R x) {
  return 2.0 * x;
}
template <>
__device__ __forceinline__ double twice_pos<double>(double x) {  // 2 x for x > 0, on the bit pattern
  return dfrom(twice_mag(dbits(x)));
}
template <class R>
__device__ __forceinline__ R face_coef(R a, R b, bool harmonic) {
  if (harmonic) {
    const R ab = a * b;
    return (ab > 0.0) ? twice_pos(ab) / (a + b) : R(0.0);
  }
  return halve(a + b);
}

// MC-type limiter of mol_slope, Source/MOL.H:104-112.
template <class R>
__device__ __forceinline__ R mc_limit(R dl, R dr) {
  const R dcen = 0.5 * (dl + dr);
  const R dlim = (dl * dr >= 0.0) ? 2.0 * fmin(fabs(dl), fabs(dr)) : R(0.0);
  return copysign(1.0, dcen) * fmin(dlim, fabs(dcen));
}

// The same limiter for double, with every step that is exact in binary done
// on the bit patterns by the integer pipe: the halving of dl + dr (halve),
// min(|dl|, |dr|) and min(dlim, |dcen|) (non-negative doubles order like
// their bit patterns; a NaN never wins, like fmin), the doubling (twice_mag)
// and the sign of dcen (copysign(1, dcen) * r = r with dcen's sign bit for
// r >= 0).  Only dl + dr and the sign test dl * dr >= 0 stay on the FP64
// pipe: 3 FP64 operations instead of 8, bit for bit the same result.
__device__ __forceinline__ double mc_limit(double dl, double dr) {
  constexpr unsigned long long kSign = 0x8000000000000000ULL;
  const unsigned long long bc = dbits(halve(dl + dr));
  const unsigned long long sgn = bc & kSign, acen = bc ^ sgn;
  const unsigned long long al = dbits(dl) & ~kSign, ar = dbits(dr) & ~kSign;
  const unsigned long long dlim = (dl * dr >= 0.0) ? twice_mag(al < ar ? al : ar) : 0ULL;
  return dfrom((dlim < acen ? dlim : acen) | sgn);
}

// ---------------------------------------------------------------------------
// Species counts with compiled kernels.  NUM_SPECIES is a compile-time
// constant of the reference's mechanism (Source/IndexDefines.H:4); the
// library instantiates its passes for these counts: 1 (GammaLaw EOS with
// constant transport) and 9 and 21 (ideal mixture with mixture-averaged
// transport; H2/air-sized and DRM19-sized mechanisms).
// ---------------------------------------------------------------------------
template <int NS>
struct Physics {  // ideal-gas mixture, mixture-averaged transport
  using EOS = IdealMixEos<NS>;
  using TR = SimpleTransport<NS>;
  static constexpr bool MIX = true;
};
template <>
struct Physics<1> {  // one species: GammaLaw, constant transport
  using EOS = GammaLawEos<1>;
  using TR = ConstantTransport<1>;
  static constexpr bool MIX = false;
};

// The device species tables of every compiled count (only the handle's
// count is filled).
struct MechSet {
  DevMech<1> m1;
  DevMech<9> m9;
  DevMech<21> m21;
  template <int NS>
  const DevMech<NS>& get() const {
    if constexpr (NS == 1)
      return m1;
    else if constexpr (NS == 9)
      return m9;
    else
      return m21;
  }
  template <int NS>
  DevMech<NS>& get() {
    if constexpr (NS == 1)
      return m1;
    else if constexpr (NS == 9)
      return m9;
    else
      return m21;
  }
};

template <int NS>
using SpeciesCount = std::integral_constant<int, NS>;

// f(SpeciesCount<NS>{}) for the species count of a handle (1, 9 or 21).
template <class F>
inline auto with_species(int nspec, F&& f) {
  if (nspec == 1) return f(SpeciesCount<1>{});
  if (nspec == 21) return f(SpeciesCount<21>{});
  return f(SpeciesCount<9>{});
}

}  // namespace PCG_NAMESPACE
