// pc_mixed.cuh — mixed-precision form of the MOL right-hand side.
//
// Same two passes as the FP64 form (pc_kernels.cuh) with the precision split
// of PC_PRECISION_MIXED:
//   FP64 accuracy, in double-float arithmetic (pc_ff.cuh, ~48 bits on the
//         FP32 pipe; FP64 itself for the GammaLaw cell pass): conserved ->
//         primitive conversion including the cell mass fractions
//         Y_k = rho Y_k / rho, the EOS temperature Newton solve,
//         p = rho (R/Wbar) T, mole fractions, the Godunov-state internal
//         energy and energy fluxes, and the flux-divergence accumulation (the
//         difference of two FP32 face fluxes taken exactly, then scaled and
//         summed in double-float and rounded to FP64 once, so the telescoping
//         sum conserves mass, momentum and energy far below the form's error).
//   FP32: sound speed, transport coefficients, MOL slopes and face states
//         (including the face mass-fraction renormalisation), the Riemann
//         solver and its EOS calls, and the diffusion fluxes.
// FP32 pressure is carried as p - p_ref (p_ref from the configuration): the
// slopes, the Riemann star pressure and the pressure gradients only use
// differences, the EOS calls add p_ref back, and the normal-momentum flux
// drops the constant p_ref, whose divergence is zero on a uniform grid.
// Records are FP32 (16-byte groups, MRec) except the mole fractions and the
// temperature, kept at FP64 accuracy after the FP32 groups (MPair): diffusion
// is driven by their cell-to-cell
// differences, which in the far field are ~1e-6 of X itself and would be lost
// in FP32, and whose second differences (the conduction term of the energy
// RHS) are ~1e-3 of T.  Those FP64 values are stored as double-float pairs
// (pc_ff.cuh: hi + lo, about 48 bits), so the flux pass forms their
// differences on the FP32 pipe, to full FP32 accuracy of the difference.  The
// internal energy of the Godunov state, whose formation-energy terms cancel
// to ~1e-2 of their size, is evaluated in double-float arithmetic at a
// double-float density and composition: the upwind cell's values plus FP32
// increments (hydro_face_f).  The cell's part of the mixture sums (R/Wbar and
// the NASA-7 coefficients of both ranges) is formed once per cell in the cell
// pass; a face adds the FP32 sums over its composition increments.  The
// energy fluxes formed from it reach the divergence as double-float pairs.
#pragma once

#include "pc_ff.cuh"
#include "pc_kernels.cuh"

namespace pcg {

template <int NS>
struct MechF {
  float rW[NS];
  float cpc[2][6][NS];
  float tmid;
  float visc[NS][4], cond[NS][4], bulk[NS];
  float diff[(NS * (NS - 1)) / 2 + 1][4];
  float inv_pref;
  float gamma, gm1, cpk[NS];
  float const_mu, const_xi, const_lam, const_rhoD;
  float p_ref;
  // double-float copies for the Godunov-state energy (e_rp_ff)
  ff rWf[NS];
  ff cpcf[2][6][NS];
  ff gm1f, third, fifth;
};

// hi + lo of a double on the host (the pair ff_of gives on the device).
inline ff ff_host(double x) {
  const float h = (float)x;
  return {h, (float)(x - (double)h)};
}

template <int NS>
__host__ MechF<NS> to_float(const DevMech<NS>& m, double p_ref) {
  MechF<NS> f{};
  for (int k = 0; k < NS; ++k) {
    f.rWf[k] = ff_host(m.rW[k]);
    for (int r = 0; r < 2; ++r)
      for (int n = 0; n < 6; ++n) f.cpcf[r][n][k] = ff_host(m.cpc[r][n][k]);
  }
  f.gm1f = ff_host(m.gm1);
  f.third = ff_host(1.0 / 3.0);
  f.fifth = ff_host(0.2);
  for (int k = 0; k < NS; ++k) {
    f.rW[k] = (float)m.rW[k];
    f.cpk[k] = (float)m.cpk[k];
    f.bulk[k] = (float)m.bulk[k];
    for (int n = 0; n < 4; ++n) {
      f.visc[k][n] = (float)m.visc[k][n];
      f.cond[k][n] = (float)m.cond[k][n];
    }
    for (int r = 0; r < 2; ++r)
      for (int n = 0; n < 6; ++n) f.cpc[r][n][k] = (float)m.cpc[r][n][k];
  }
  for (int q = 0; q < (NS * (NS - 1)) / 2 + 1; ++q)
    for (int n = 0; n < 4; ++n) f.diff[q][n] = (float)m.diff[q][n];
  f.tmid = (float)m.tmid;
  f.inv_pref = (float)m.inv_pref;
  f.gamma = (float)m.gamma;
  f.gm1 = (float)m.gm1;
  f.const_mu = (float)m.const_mu;
  f.const_xi = (float)m.const_xi;
  f.const_lam = (float)m.const_lam;
  f.const_rhoD = (float)m.const_rhoD;
  f.p_ref = (float)p_ref;
  return f;
}

// FP64-accuracy fields stored after the FP32 fields of a mixed record, for
// the cells whose faces the pass evaluates (the valid cells and one layer
// around them), each a double-float pair (hi, lo), two pairs to a 16-byte
// group (hi, lo, hi, lo), group g of cell c at [g N + c] (MPair): the mole
// fractions X_k and the temperature (X_0 X_1 | X_2 X_3 | ... | T last), then
// (rho, R/Wbar) (R/Wbar with the ideal-mixture EOS only) and, with the
// ideal-mixture EOS, the mixture NASA-7 coefficients C_n = sum_k Y_k (R/W_k)
// a_{n,k} of both temperature ranges, three groups a range.  X and T enter
// the diffusion fluxes only through differences between neighbouring cells,
// which FP32 values would resolve to no better than 1e-4 K / 1e-7 (the
// flame's second differences of T are a few K per cell).  rho, R/Wbar and C are the cell's part of the Godunov
// state's density and mixture sums (energy fluxes, hydro_face_f), to which a
// face adds only FP32 increments.  The fields start after the FP32 groups
// (MRec) of every cell; a mixed record stays within the FP64 record's size.
//
// The FP32 fields of a mixed record are 16-byte groups (float4), group g of
// cell c at [g N + c], so that a face reads four fields of a neighbour with
// one load: G0 = (rho, u', v', w') (velocity offsets from the box's
// reference velocity), G1 = (p', c, T, 0) (p' = p - p_ref); then the mass
// fractions Y_k four to a group, the species enthalpies h_k four to a group,
// and D_k, mu, xi, lambda (the transport coefficients, in that order) four to
// a group, the last group of each padded with 0.  h_k and the transport
// coefficients are written for the valid cells and one layer around them (the
// cells whose faces carry diffusion fluxes) only.  The record arena of a box
// starts on a 256-byte boundary.
template <int NS>
struct MRec {
  static constexpr int Q = (NS + 3) / 4, QD = (NS + 6) / 4;  // groups of Y / h, of the transport coefficients
  static constexpr int G0 = 0, G1 = 1, Y = 2, H = 2 + Q, D = 2 + 2 * Q;
  static constexpr int G = 2 + 2 * Q + QD;  // groups in all
};
template <int NS>
struct MPair {
  static constexpr int XT = 0, QX = (NS + 2) / 2;  // groups of X_k and T; T in group NS / 2, slot NS % 2
  static constexpr int RHO = QX;           // (rho, R/Wbar)
  static constexpr int COEF = QX + 1;      // C[r][n] in group COEF + 3 r + n / 2, slot n % 2
  template <bool MIX>
  static constexpr int G = MIX ? QX + 7 : QX + 1;  // groups in all
};
template <int NS>
__device__ __forceinline__ float4* mixed_x(const DevBox& b) {
  return reinterpret_cast<float4*>(b.rec) + (long long)MRec<NS>::G * b.ncell;
}
// Loads / stores of the groups of a mixed record.
__device__ __forceinline__ float4 ld_group(const float4* rec, int g, long long N, long long c) {
  return __ldg(rec + (long long)g * N + c);
}
__device__ __forceinline__ float grp(const float4& v, int i) {  // component i (a constant after unrolling)
  return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}
// n values v[0..n) of cell c from the groups starting at g
template <int n>
__device__ __forceinline__ void ld_groups(const float4* rec, int g, long long N, long long c, float* v) {
#pragma unroll
  for (int q = 0; q < (n + 3) / 4; ++q) {
    const float4 t = ld_group(rec, g + q, N, c);
#pragma unroll
    for (int l = 0; l < 4; ++l)
      if (4 * q + l < n) v[4 * q + l] = grp(t, l);
  }
}
template <int n>
__device__ __forceinline__ void st_groups(float4* r, int g, long long N, const float* v) {
#pragma unroll
  for (int q = 0; q < (n + 3) / 4; ++q) {
    float t[4];
#pragma unroll
    for (int l = 0; l < 4; ++l) t[l] = 4 * q + l < n ? v[4 * q + l] : 0.f;
    r[(long long)(g + q) * N] = make_float4(t[0], t[1], t[2], t[3]);
  }
}
__device__ __forceinline__ ff pair_of(const float4& v, int slot) {  // slot 0 or 1 of a pair group
  return slot == 0 ? ff{v.x, v.y} : ff{v.z, v.w};
}
__device__ __forceinline__ float4 pair_group(ff a, ff b) { return make_float4(a.hi, a.lo, b.hi, b.lo); }
// x1 - x2 of two stored pairs, rounded to FP32 (the hi parts of nearby
// values subtract exactly; the lo parts carry the rest)
__device__ __forceinline__ float pair_diff(ff a, ff b) {
  return __fadd_rn(__fsub_rn(a.hi, b.hi), __fsub_rn(a.lo, b.lo));
}
// X_0..X_{NS-1} and T (NS + 1 pairs) into their groups at cell c
template <int NS>
__device__ __forceinline__ void st_xt(float4* xr, long long N, const ff* X, ff T) {
#pragma unroll
  for (int q = 0; q < MPair<NS>::QX; ++q) {
    ff v[2];
#pragma unroll
    for (int l = 0; l < 2; ++l) {
      const int n = 2 * q + l;
      v[l] = n < NS ? X[n] : (n == NS ? T : ff_of(0.f));
    }
    xr[(long long)(MPair<NS>::XT + q) * N] = pair_group(v[0], v[1]);
  }
}
template <int NS>
__device__ __forceinline__ void st_coefs(float4* xr, long long N, int range, const ff* C) {
#pragma unroll
  for (int q = 0; q < 3; ++q) xr[(long long)(MPair<NS>::COEF + 3 * range + q) * N] = pair_group(C[2 * q], C[2 * q + 1]);
}
template <int NS>
constexpr bool mixed_fits() {  // FP32 groups and pair groups against the FP64 record (in floats)
  return 4 * MRec<NS>::G + 4 * MPair<NS>::template G<Physics<NS>::MIX> <= 2 * Rec<NS>::N;
}
static_assert(mixed_fits<1>() && mixed_fits<9>() && mixed_fits<21>(), "mixed record exceeds the FP64 record");

// Reference velocity of a box: the velocity of its first valid cell (lo
// corner), in FP64 (0 where that is not finite).  The FP32 records hold the
// velocity minus it, so that FP32 resolves the velocity's variations within
// the box rather than its mean: a face flux u * (rho e) whose divergence is
// a small difference (rho e nearly uniform across a low-Mach flame) is then
// formed in FP64 as (U + u') rho e, with the FP32 rounding on u' only.  The
// Riemann solver is Galilean covariant in u (u* of shifted states is u* + U),
// so the face states and u* are computed on the offsets; its switches and
// wave speeds use U + u' in FP32.
__device__ __forceinline__ void box_uref(const DevBox& b, double U[3]) {
  const double* s = b.S + (b.lo[0] - b.sb[0]) + (long long)(b.lo[1] - b.sb[1]) * b.sj +
                    (long long)(b.lo[2] - b.sb[2]) * b.sk;
  const double ir = 1.0 / __ldg(s + URHO * b.sn);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const double u = __ldg(s + (UMX + a) * b.sn) * ir;
    U[a] = isfinite(u) ? u : 0.0;
  }
}

// Per-tile values of the face fluxes, formed once per tile by one thread:
// conversions from FP64 run on the FP64 pipe, at a small fraction of the
// FP32 rate, and would otherwise be repeated on every face.  The box's
// reference velocity in FP64, double-float and FP32; 1/dx and p_ref in FP32.
struct FaceConsts {
  double Ud[3];
  ff Uff[3];
  float U[3];
  float dxi[3];
  float pref;
};
__device__ __forceinline__ void face_consts(const DevBox& b, const Geo& g, FaceConsts& fc) {
  box_uref(b, fc.Ud);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    fc.Uff[a] = ff_of(fc.Ud[a]);
    fc.U[a] = (float)fc.Ud[a];
    fc.dxi[a] = (float)g.dxinv[a];
  }
  fc.pref = (float)g.p_ref;
}

template <int NS>
__device__ __forceinline__ float mix_rwf(const MechF<NS>& m, const float* Y) {
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < NS; ++k) s = fmaf(Y[k], m.rW[k], s);
  return s;
}

// FP32 equations of state; p is the absolute pressure.
template <int NS, bool MIX>
struct EosF;

template <int NS>
struct EosF<NS, false> {
  __device__ static float cs_T(const MechF<NS>& m, const float*, float, float rho, float, float p) {
    return sqrtf(m.gamma * p / rho);
  }
  __device__ static float cs_rp(const MechF<NS>& m, const float*, float, float rho, float p) {
    return sqrtf(m.gamma * p / rho);
  }
  __device__ static float e_rp(const MechF<NS>& m, const float*, float, float rho, float p) { return p / (m.gm1 * rho); }
  __device__ static void hi(const MechF<NS>& m, float T, float* h) {
#pragma unroll
    for (int k = 0; k < NS; ++k) h[k] = m.cpk[k] * T;
  }
};

template <int NS>
struct EosF<NS, true> {
  template <int NC>
  __device__ static void coefs(const MechF<NS>& m, const float* Y, int r, float* C) {
#pragma unroll
    for (int n = 0; n < NC; ++n) {
      float s = 0.f;
#pragma unroll
      for (int k = 0; k < NS; ++k) s = fmaf(Y[k], m.cpc[r][n][k], s);
      C[n] = s;
    }
  }
  // sound speed from the mixture coefficients C of T's range
  __device__ static float cs_C(const float C[5], float rw, float rho, float T, float p) {
    const float cv = (C[0] - rw) + T * fmaf(T, fmaf(T, fmaf(T, C[4], C[3]), C[2]), C[1]);
    return sqrtf((cv + rw) * p / (cv * rho));
  }
  __device__ static float cs_T(const MechF<NS>& m, const float* Y, float rw, float rho, float T, float p) {
    float C[5];
    coefs<5>(m, Y, T < m.tmid ? 0 : 1, C);
    return cs_C(C, rw, rho, T, p);
  }
  __device__ static float cs_rp(const MechF<NS>& m, const float* Y, float rw, float rho, float p) {
    return cs_T(m, Y, rw, rho, p / (rho * rw), p);
  }
  __device__ static float e_rp(const MechF<NS>& m, const float* Y, float rw, float rho, float p) {
    const float T = p / (rho * rw);
    float C[6];
    coefs<6>(m, Y, T < m.tmid ? 0 : 1, C);
    const float q = fmaf(T, fmaf(T, fmaf(T, fmaf(T, C[4] * 0.2f, C[3] * 0.25f), C[2] * (1.f / 3.f)), C[1] * 0.5f), C[0] - rw);
    return fmaf(T, q, C[5]);
  }
  __device__ static void hi(const MechF<NS>& m, float T, float* h) {
    const int r = T < m.tmid ? 0 : 1;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const float q = fmaf(T, fmaf(T, fmaf(T, fmaf(T, m.cpc[r][4][k] * 0.2f, m.cpc[r][3][k] * 0.25f),
                                           m.cpc[r][2][k] * (1.f / 3.f)),
                                  m.cpc[r][1][k] * 0.5f),
                           m.cpc[r][0][k]);
      h[k] = fmaf(T, q, m.cpc[r][5][k]);
    }
  }
};

__device__ __forceinline__ float horner4f(const float c[4], float L) { return fmaf(L, fmaf(L, fmaf(L, c[3], c[2]), c[1]), c[0]); }

// FP32 transport: the same formulas as SimpleTransport / ConstantTransport.
template <int NS, bool SIMPLE>
struct TransF {
  __device__ static void eval(const MechF<NS>& m, float T, float rho, float p, const float* Y, const float* X, float* out) {
    if constexpr (!SIMPLE) {
#pragma unroll
      for (int k = 0; k < NS; ++k) out[k] = m.const_rhoD;
      out[NS] = m.const_mu;
      out[NS + 1] = m.const_xi;
      out[NS + 2] = m.const_lam;
    } else {
      const float L = logf(T);
      float smu = 0.f, slam = 0.f, sxi = 0.f;
#pragma unroll
      for (int k = 0; k < NS; ++k) {
        const float mk = expf(horner4f(m.visc[k], L));
        const float m2 = mk * mk;
        smu = fmaf(X[k], m2 * m2 * m2, smu);
        slam = fmaf(X[k], expf(0.25f * horner4f(m.cond[k], L)), slam);
        sxi = fmaf(X[k], m.bulk[k] * mk, sxi);
      }
      float s[NS];
#pragma unroll
      for (int k = 0; k < NS; ++k) s[k] = 0.f;
      const float pr = p * m.inv_pref;
      int q = 0;
#pragma unroll
      for (int k = 0; k < NS; ++k) {
#pragma unroll
        for (int j = k + 1; j < NS; ++j, ++q) {
          const float invD = expf(-horner4f(m.diff[q], L)) * pr;
          s[k] = fmaf(fmaxf(X[j], 1e-15f), invD, s[k]);
          s[j] = fmaf(fmaxf(X[k], 1e-15f), invD, s[j]);
        }
      }
      const float rw = mix_rwf<NS>(m, Y);
#pragma unroll
      for (int k = 0; k < NS; ++k) out[k] = (s[k] > 0.f) ? rho * (1.f - Y[k]) * (rw / m.rW[k]) / s[k] : 0.f;
      out[NS] = expf(logf(smu) * (1.f / 6.f));
      out[NS + 1] = sxi;
      const float l2 = slam * slam;
      out[NS + 2] = l2 * l2;
    }
  }
};

__device__ __forceinline__ float mc_limitf(float dl, float dr) {
  const float dcen = 0.5f * (dl + dr);
  const float dlim = (dl * dr >= 0.f) ? 2.f * fminf(fabsf(dl), fabsf(dr)) : 0.f;
  return copysignf(1.f, dcen) * fminf(dlim, fabsf(dcen));
}

__device__ __forceinline__ float face_coeff(float a, float b, bool harmonic) {
  if (harmonic) {
    const float ab = a * b;
    return (ab > 0.f) ? 2.f * ab / (a + b) : 0.f;
  }
  return 0.5f * (a + b);
}

// Double-float counterparts of IdealMixEos's mixture sums and polynomials:
// R/Wbar = sum_k Y_k R/W_k, the mixture NASA-7 coefficients of range r,
// e(T) = C5 + T ((C0 - R/Wbar) + T (C1/2 + T (C2/3 + T (C3/4 + T C4/5))))
// and cv(T) = (C0 - R/Wbar) + T (C1 + T (C2 + T (C3 + T C4))).
// sum_k a_k b_k of double-float operands as a compensated dot product
// (Ogita, Rump and Oishi, "Accurate sum and dot product", SIAM J. Sci.
// Comput. 26, 2005, Dot2): the products of the hi parts split exactly by
// TwoProduct and summed by TwoSum, their errors, the cross terms and the
// sums' errors gathered in one float, added by one TwoSum at the end.  About
// 2^-48 of the terms' magnitude, like a chain of ff_fma, in fewer FP32
// operations.
template <int NS>
__device__ __forceinline__ ff dot_ff(const ff* a, const ff* b) {
  float s = __fmul_rn(a[0].hi, b[0].hi);
  float c = fmaf(a[0].hi, b[0].hi, -s);
  c = fmaf(a[0].hi, b[0].lo, fmaf(a[0].lo, b[0].hi, c));
#pragma unroll
  for (int k = 1; k < NS; ++k) {
    const float p = __fmul_rn(a[k].hi, b[k].hi);
    float e;
    float t;
    two_sum(s, p, t, e);
    s = t;
    c = __fadd_rn(c, __fadd_rn(e, fmaf(a[k].hi, b[k].lo, fmaf(a[k].lo, b[k].hi, fmaf(a[k].hi, b[k].hi, -p)))));
  }
  return ff_sum(s, c);  // TwoSum: exact even where the sum cancels below c
}
template <int NS>
__device__ __forceinline__ ff mix_rw_ff(const MechF<NS>& m, const ff* Y) {
  return dot_ff<NS>(Y, m.rWf);
}
template <int NS>
__device__ __forceinline__ void mix_coefs_ff(const MechF<NS>& m, const ff* Y, int r, ff C[6]) {
#pragma unroll
  for (int n = 0; n < 6; ++n) C[n] = dot_ff<NS>(Y, m.cpcf[r][n]);
}
template <int NS>
__device__ __forceinline__ ff e_of_ff(const MechF<NS>& m, const ff C[6], ff c0, ff T) {
  ff q = ff_fma(T, ff_mul(C[4], m.fifth), ff_mul(C[3], 0.25f));
  q = ff_fma(T, q, ff_mul(C[2], m.third));
  q = ff_fma(T, q, ff_mul(C[1], 0.5f));
  q = ff_fma(T, q, c0);
  return ff_fma(T, q, C[5]);
}
__device__ __forceinline__ ff cv_of_ff(const ff C[6], ff c0, ff T) {
  ff w = ff_fma(T, C[4], C[3]);
  w = ff_fma(T, w, C[2]);
  w = ff_fma(T, w, C[1]);
  return ff_fma(T, w, c0);
}

// REY2T in double-float arithmetic: IdealMixEos::rey2t's Newton iteration
// on e(T) = e from the guess (steps clamped to +-1000 K, T >= 10 K, stop
// once |T_new - T| <= 1e-12 T_new, ok = false after maxit iterations).
// rC, C: the temperature range of the last iteration and the mixture
// coefficients of that range (mix_coefs_ff), which the cell pass stores.
template <int NS>
__device__ ff rey2t_ff(const MechF<NS>& m, const ff* Y, ff rw, ff ein, double Tguess, int maxit, bool& ok, int& rC,
                       ff C[6]) {
  // Tguess > 0 and finite, tested on its bits (integer pipe)
  const long long tb = __double_as_longlong(Tguess);
  ff t = (tb > 0 && tb < 0x7ff0000000000000LL) ? ff_of(Tguess) : ff_of(1000.f);
  int r = t.hi < m.tmid ? 0 : 1;
  mix_coefs_ff<NS>(m, Y, r, C);
  ok = false;
  for (int it = 0; it < maxit; ++it) {
    const int rn = t.hi < m.tmid ? 0 : 1;
    if (rn != r) {
      r = rn;
      mix_coefs_ff<NS>(m, Y, r, C);
    }
    const ff c0 = ff_sub(C[0], rw);
    ff dt = ff_div(ff_sub(ein, e_of_ff<NS>(m, C, c0, t)), cv_of_ff(C, c0, t));
    if (dt.hi > 1000.f) dt = ff_of(1000.f);
    if (dt.hi < -1000.f) dt = ff_of(-1000.f);
    ff tn = ff_add(t, dt);
    if (tn.hi < 10.f) tn = ff_of(10.f);
    const bool conv = fabsf(ff_to_float(ff_sub(tn, t))) <= 1e-12f * tn.hi;
    t = tn;
    if (conv) {
      ok = true;
      break;
    }
  }
  rC = r;
  return t;
}

// One cell of the mixed cell pass with the ideal-mixture EOS, in
// double-float arithmetic (pc_ff.cuh): the FP64 state read as hi + lo pairs,
// then ctoprim (Y_k = rho Y_k / rho with the |Y| < 1e-4 eps zeroing of
// Utilities.H:288-294, e = (rho E - rho |u|^2 / 2) / rho), the temperature
// Newton solve, p = rho (R/Wbar) T and the mole fractions; the record's FP32
// fields are those values rounded, its FP64 fields (X, T, rho, Y) the pairs.
template <int NS, bool SIMPLE>
__device__ __forceinline__ void cell_mixed_ff(const DevBox& b, const MechF<NS>& mf, const DevFlags& f, long long c,
                                              const double* Us, bool& newton_fail, bool& nonpos) {
  using MR = MRec<NS>;
  const int nx = b.n2[0], ny = b.n2[1];
  const int i = b.g2lo[0] + (int)(c % nx);
  const int j = b.g2lo[1] + (int)((c / nx) % ny);
  const int k = b.g2lo[2] + (int)(c / ((long long)nx * ny));
  const double* s = b.S + (i - b.sb[0]) + (long long)(j - b.sb[1]) * b.sj + (long long)(k - b.sb[2]) * b.sk;
  const long long sn = b.sn;
  // the conserved state (rho, momenta, rho E, rho Y_k): every load first,
  // then one warp-uniform choice of the conversion to double-float (the
  // integer-pipe form unless a lane holds a value outside its range)
  constexpr int NU = 5 + NS;
  double u[NU];
  u[0] = __ldg(s + URHO * sn);
#pragma unroll
  for (int a = 0; a < 3; ++a) u[1 + a] = __ldg(s + (UMX + a) * sn);
  u[4] = __ldg(s + UEDEN * sn);
#pragma unroll
  for (int n = 0; n < NS; ++n) u[5 + n] = __ldg(s + (UFS + n) * sn);
  const double Tguess = __ldg(s + UTEMP * sn);
  bool fast = true;
#pragma unroll
  for (int n = 0; n < NU; ++n) fast &= ff_fast_ok(u[n]);
  ff Uc[NU];
  if (__all_sync(__activemask(), fast)) {
#pragma unroll
    for (int n = 0; n < NU; ++n) Uc[n] = ff_of_fast(u[n]);
  } else {
#pragma unroll
    for (int n = 0; n < NU; ++n) Uc[n] = ff_of_conv(u[n]);
  }
  const ff rho = Uc[0];
  const ff ir = ff_div(ff_of(1.f), rho);
  const ff vx = ff_mul(Uc[1], ir);
  const ff vy = ff_mul(Uc[2], ir);
  const ff vz = ff_mul(Uc[3], ir);
  const ff v2 = ff_fma(vz, vz, ff_fma(vy, vy, ff_mul(vx, vx)));
  const ff e = ff_mul(ff_sub(Uc[4], ff_mul(ff_mul(rho, v2), 0.5f)), ir);
  ff Y[NS];
  float Yf[NS];
#pragma unroll
  for (int n = 0; n < NS; ++n) {
    ff y = ff_mul(Uc[5 + n], ir);
    if (fabsf(y.hi) < 1e-4f * 2.220446049250313e-16f) y = ff_of(0.f);
    Y[n] = y;
    Yf[n] = ff_to_float(y);
  }
  const ff rw = mix_rw_ff<NS>(mf, Y);
  bool ok = true;
  int rC;
  ff C[6];
  const ff T = rey2t_ff<NS>(mf, Y, rw, e, Tguess, f.newton_maxit, ok, rC, C);
  const bool inner = i >= b.lo[0] - 1 && i <= b.hi[0] + 1 && j >= b.lo[1] - 1 && j <= b.hi[1] + 1 &&
                     k >= b.lo[2] - 1 && k <= b.hi[2] + 1;
  const long long N = b.ncell;
  if (inner) {  // the mixture coefficients of both ranges: the Newton solve's own, and the other's
    float4* xr = mixed_x<NS>(b) + c;
    st_coefs<NS>(xr, N, rC, C);
    mix_coefs_ff<NS>(mf, Y, 1 - rC, C);
    st_coefs<NS>(xr, N, 1 - rC, C);
  }
  const ff p = ff_mul(ff_mul(rho, rw), T);
  newton_fail = !ok;
  nonpos = !(rho.hi > 0.f) || !(p.hi > 0.f) || !(T.hi > 0.f);
  const float rhof = ff_to_float(rho), Tf = ff_to_float(T), pf = ff_to_float(p), rwf = ff_to_float(rw);
  const float cs = EosF<NS, true>::cs_T(mf, Yf, rwf, rhof, Tf, pf);
  float4* r = reinterpret_cast<float4*>(b.rec) + c;
  // velocity offsets from the box's reference velocity
  r[MR::G0 * N] = make_float4(rhof, ff_to_float(ff_sub(vx, ff_of(Us[0]))), ff_to_float(ff_sub(vy, ff_of(Us[1]))),
                              ff_to_float(ff_sub(vz, ff_of(Us[2]))));
  r[MR::G1 * N] = make_float4(ff_to_float(ff_sub(p, ff_of(mf.p_ref))), cs, Tf, 0.f);
  st_groups<NS>(r, MR::Y, N, Yf);
  if (inner) {
    float X[NS];
    float4* xr = mixed_x<NS>(b) + c;
    const ff irw = ff_div(ff_of(1.f), rw);
    ff Xp[NS];
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      Xp[n] = ff_mul(ff_mul(Y[n], mf.rWf[n]), irw);
      X[n] = ff_to_float(Xp[n]);
    }
    st_xt<NS>(xr, N, Xp, T);
    xr[MPair<NS>::RHO * N] = pair_group(rho, rw);
    float out[NS + 3];
    TransF<NS, SIMPLE>::eval(mf, Tf, rhof, pf, Yf, X, out);
    float h[NS];
    EosF<NS, true>::hi(mf, Tf, h);
    st_groups<NS>(r, MR::H, N, h);
    st_groups<NS + 3>(r, MR::D, N, out);
  }
}

// ---------------------------------------------------------------------------
// Pass 1, mixed precision.  Records: the FP32 groups of MRec<NS> (p - p_ref
// in place of p), then the double-float pairs (mixed_x).
// ---------------------------------------------------------------------------
template <int NS, class EOSD, bool MIX, bool SIMPLE, bool STRICT = false>
__global__ void __launch_bounds__(kCellThreads)
    cell_kernel_mixed(const DevBox* __restrict__ boxes, const int2* __restrict__ items,
                      const __grid_constant__ DevMech<NS> m, const __grid_constant__ MechF<NS> mf, const DevFlags f,
                      unsigned long long* __restrict__ counters) {
  using MR = MRec<NS>;
  const int2 it = items[blockIdx.x];
  const DevBox& b = boxes[it.x];
  const long long c = (long long)it.y + threadIdx.x;
  __shared__ double Us[3];  // the box's reference velocity
  if (threadIdx.x == 0) box_uref(b, Us);
  __syncthreads();
  bool newton_fail = false, nonpos = false;
  if constexpr (MIX && !STRICT) {
    if (c < b.ncell) cell_mixed_ff<NS, SIMPLE>(b, mf, f, c, Us, newton_fail, nonpos);
  } else if (c < b.ncell) {  // FP64 (GammaLaw, or PC_PRECISION_MIXED_FP64)
    const int nx = b.n2[0], ny = b.n2[1];
    const int i = b.g2lo[0] + (int)(c % nx);
    const int j = b.g2lo[1] + (int)((c / nx) % ny);
    const int k = b.g2lo[2] + (int)(c / ((long long)nx * ny));
    const double* s = b.S + (i - b.sb[0]) + (long long)(j - b.sb[1]) * b.sj + (long long)(k - b.sb[2]) * b.sk;
    const long long sn = b.sn;
    const double rho = __ldg(s + URHO * sn);
    const double rhoinv = 1.0 / rho;
    const double vx = __ldg(s + UMX * sn) * rhoinv;
    const double vy = __ldg(s + UMY * sn) * rhoinv;
    const double vz = __ldg(s + UMZ * sn) * rhoinv;
    const double e = (__ldg(s + UEDEN * sn) - 0.5 * rho * (vx * vx + vy * vy + vz * vz)) * rhoinv;
    double Y[NS];
    float Yf[NS];
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      double y = __ldg(s + (UFS + n) * sn) * rhoinv;
      if (-1e-4 * 2.220446049250313e-16 < y && y < 1e-4 * 2.220446049250313e-16) y = 0.0;
      Y[n] = y;
      Yf[n] = (float)y;
    }
    const double rw = mix_rw<NS>(m, Y);
    bool ok = true;
    const double T = EOSD::rey2t(m, Y, rw, e, __ldg(s + UTEMP * sn), f.newton_maxit, ok);
    const double p = rho * rw * T;
    newton_fail = !ok;
    nonpos = !(rho > 0.0) || !(p > 0.0) || !(T > 0.0);
    const float rhof = (float)rho, Tf = (float)T, pf = (float)p, rwf = (float)rw;
    const float cs = EosF<NS, MIX>::cs_T(mf, Yf, rwf, rhof, Tf, pf);
    float4* r = reinterpret_cast<float4*>(b.rec) + c;
    const long long N = b.ncell;
    // velocity offsets from the box's reference velocity
    r[MR::G0 * N] = make_float4(rhof, (float)(vx - Us[0]), (float)(vy - Us[1]), (float)(vz - Us[2]));
    r[MR::G1 * N] = make_float4((float)(p - (double)mf.p_ref), cs, Tf, 0.f);
    st_groups<NS>(r, MR::Y, N, Yf);
    const bool inner = i >= b.lo[0] - 1 && i <= b.hi[0] + 1 && j >= b.lo[1] - 1 && j <= b.hi[1] + 1 &&
                       k >= b.lo[2] - 1 && k <= b.hi[2] + 1;
    if (inner) {
      float X[NS];
      float4* xr = mixed_x<NS>(b) + c;
      const double irw = 1.0 / rw;
      ff Xp[NS];
#pragma unroll
      for (int n = 0; n < NS; ++n) {
        const double x = Y[n] * m.rW[n] * irw;
        Xp[n] = ff_of(x);
        X[n] = (float)x;
      }
      st_xt<NS>(xr, N, Xp, ff_of(T));
      // the cell's mixture sums for the Godunov energy, in double-float (ideal mixture)
      xr[MPair<NS>::RHO * N] = pair_group(ff_of(rho), MIX ? ff_of(rw) : ff_of(0.f));
      if constexpr (MIX) {
        ff Yp[NS];
#pragma unroll
        for (int n = 0; n < NS; ++n) Yp[n] = ff_of(Y[n]);
#pragma unroll
        for (int range = 0; range < 2; ++range) {
          ff C[6];
          mix_coefs_ff<NS>(mf, Yp, range, C);
          st_coefs<NS>(xr, N, range, C);
        }
      }
      float out[NS + 3];
      TransF<NS, SIMPLE>::eval(mf, Tf, rhof, pf, Yf, X, out);
      float h[NS];
      EosF<NS, MIX>::hi(mf, Tf, h);
      st_groups<NS>(r, MR::H, N, h);
      st_groups<NS + 3>(r, MR::D, N, out);
    }
  }
  warp_count(&counters[kCounterNewton], newton_fail);
  warp_count(&counters[kCounterNonpos], nonpos);
}

// FP32 hyperbolic face flux (not area-scaled); normal momentum without p_ref.
// Internal energy at (rho, Y, p) in double-float arithmetic: the operations
// of IdealMixEos::e_rp / GammaLawEos::e_rp (RYP2E), each a double-float one.
template <int NS, bool MIX>
__device__ __forceinline__ ff e_rp_ff(const MechF<NS>& m, const ff* Y, ff rho, ff p) {
  if constexpr (MIX) {
    const ff rw = mix_rw_ff<NS>(m, Y);
    const ff T = ff_div(p, ff_mul(rho, rw));
    ff C[6];
    mix_coefs_ff<NS>(m, Y, T.hi < m.tmid ? 0 : 1, C);
    return e_of_ff<NS>(m, C, ff_sub(C[0], rw), T);
  } else {
    return ff_div(p, ff_mul(m.gm1f, rho));
  }
}

// The same at species densities rho Y_k (FP32) and density rho.
template <int NS, bool MIX>
__device__ __forceinline__ ff e_rp_ff_rY(const MechF<NS>& m, const float* rY, float rho, ff p) {
  const ff ir = ff_div(ff_of(1.f), ff_of(rho));
  ff Y[NS];
#pragma unroll
  for (int n = 0; n < NS; ++n) Y[n] = ff_mul(ir, rY[n]);
  return e_rp_ff<NS, MIX>(m, Y, ff_of(rho), p);
}

// Internal energy of a Godunov state whose composition is that of the
// upwind cell (its R/Wbar rw_cell and, in the pair groups xr, the mixture
// coefficients of both ranges, from the cell pass) plus FP32 increments dY,
// at density rho and pressure p:
// the sums of e_rp_ff with the cell's part in double-float and the
// increments' part sum_k dY_k c_k in FP32 (its rounding falls on the
// increments only).
template <int NS>
__device__ __forceinline__ ff e_godunov_ff(const MechF<NS>& m, const float4* xr, long long N, const float* dY, ff rho,
                                           ff p, ff rw_cell) {
  float drw = 0.f;
#pragma unroll
  for (int k = 0; k < NS; ++k) drw = fmaf(dY[k], m.rW[k], drw);
  const ff rw = ff_add(rw_cell, drw);
  const ff T = ff_div(p, ff_mul(rho, rw));
  const int r = T.hi < m.tmid ? 0 : 1;
  ff C[6];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const float4 g = __ldg(xr + (long long)(MPair<NS>::COEF + 3 * r + q) * N);
#pragma unroll
    for (int l = 0; l < 2; ++l) {
      const int n = 2 * q + l;
      float dc = 0.f;
#pragma unroll
      for (int k = 0; k < NS; ++k) dc = fmaf(dY[k], m.cpc[r][n][k], dc);
      C[n] = ff_add(pair_of(g, l), dc);
    }
  }
  return e_of_ff<NS>(m, C, ff_sub(C[0], rw), T);
}

// FP64 internal energy from FP32 mass fractions Y (for Lax-Friedrichs sides).
template <int NS, bool MIX>
__device__ __forceinline__ double e_rpY_fp64(const DevMech<NS>& md, const float* Yf, float rho, double p) {
  double Y[NS];
#pragma unroll
  for (int n = 0; n < NS; ++n) Y[n] = (double)Yf[n];
  const double rw = mix_rw<NS>(md, Y);
  if constexpr (MIX)
    return IdealMixEos<NS>::e_rp(md, Y, rw, (double)rho, p);
  else
    return GammaLawEos<NS>::e_rp(md, Y, rw, (double)rho, p);
}

// (rho, normal velocity, first and second transverse velocity) of a G0
// group for faces of direction d: the transverse axes are t1 = (d == 0 ? 1
// : 0) and t2 = (d == 2 ? 1 : 2).
__device__ __forceinline__ float4 rot_g0(const float4& a, int d) {
  return make_float4(a.x, d == 0 ? a.y : (d == 1 ? a.z : a.w), d == 0 ? a.z : a.y, d == 2 ? a.z : a.w);
}

// The face code takes the direction d at run time, so that the pass holds
// one copy of it rather than one per direction (its instruction footprint,
// not its arithmetic, was what the warps waited on).  The momentum fluxes
// are returned in rotated order: F[UMX] normal, F[UMY] along t1, F[UMZ]
// along t2 (face_mixed stages them at their axes).  The total and internal
// energy fluxes (FE, FEI) are returned in double-float: their divergence is
// ~1e-3 of their size, below what an FP32 flux can resolve.
template <int NS, bool MIX>
__device__ __forceinline__ void hydro_face_f(const DevBox& b, const MechF<NS>& m, const DevMech<NS>& md,
                                             const DevFlags& f, int d, long long cR, long long st,
                                             const FaceConsts& fc, float* F, ff& FE, ff& FEI) {
  using MR = MRec<NS>;
  using E = EosF<NS, MIX>;
  const float4* rec = reinterpret_cast<const float4*>(b.rec);
  const long long N = b.ncell;
  const long long cL = cR - st, cLL = cL - st, cRR = cR + st;
  // reference velocity of the normal and the two transverse components (the
  // velocities below are offsets from them)
  const float Unf = fc.U[d], Ut1f = fc.U[(d == 0) ? 1 : 0], Ut2f = fc.U[(d == 2) ? 1 : 2];
  const float4 aLL = rot_g0(ld_group(rec, MR::G0, N, cLL), d), aL = rot_g0(ld_group(rec, MR::G0, N, cL), d);
  const float4 aR = rot_g0(ld_group(rec, MR::G0, N, cR), d), aRR = rot_g0(ld_group(rec, MR::G0, N, cRR), d);
  const float4 bL = ld_group(rec, MR::G1, N, cL), bR = ld_group(rec, MR::G1, N, cR);  // (p', c, T, 0)
  const float* g1 = reinterpret_cast<const float*>(rec + (long long)MR::G1 * N);
  const float rLL = aLL.x, rL = aL.x, rR = aR.x, rRR = aRR.x;
  const float pLL = __ldg(g1 + 4 * cLL), pL = bL.x, pR = bR.x, pRR = __ldg(g1 + 4 * cRR);
  const float uLL = aLL.y, uL = aL.y, uR = aR.y, uRR = aRR.y;
  const float cLc = bL.y, cRc = bR.y;
  const float t1L = aL.z, t1R = aR.z, t2L = aL.w, t2R = aR.w;
  const float icL = 1.f / cLc, icR = 1.f / cRc;
  float dqL[4] = {0.f, 0.f, 0.f, 0.f}, dqR[4] = {0.f, 0.f, 0.f, 0.f};
  const bool slopes = f.slopes != 0;
  const float dpl = pL - pLL, dpc = pR - pL, dpr = pRR - pR;
  if (slopes) {
    const float t1LL = aLL.z, t1RR = aRR.z, t2LL = aLL.w, t2RR = aRR.w;
    {
      const float a = 0.5f * dpl * icL, bb = 0.5f * rL * (uL - uLL);
      const float a2 = 0.5f * dpc * icL, b2 = 0.5f * rL * (uR - uL);
      dqL[0] = mc_limitf(a - bb, a2 - b2);
      dqL[1] = mc_limitf(a + bb, a2 + b2);
      dqL[2] = mc_limitf(t1L - t1LL, t1R - t1L);
      dqL[3] = mc_limitf(t2L - t2LL, t2R - t2L);
    }
    {
      const float a = 0.5f * dpc * icR, bb = 0.5f * rR * (uR - uL);
      const float a2 = 0.5f * dpr * icR, b2 = 0.5f * rR * (uRR - uR);
      dqR[0] = mc_limitf(a - bb, a2 - b2);
      dqR[1] = mc_limitf(a + bb, a2 + b2);
      dqR[2] = mc_limitf(t1R - t1L, t1RR - t1R);
      dqR[3] = mc_limitf(t2R - t2L, t2RR - t2R);
    }
  }
  const float unl = uL + 0.5f * (dqL[1] - dqL[0]) / rL;
  const float pl = pL + 0.5f * (dqL[0] + dqL[1]) * cLc;  // offset pressure
  const float ut1l = t1L + 0.5f * dqL[2];
  const float ut2l = t2L + 0.5f * dqL[3];
  const float unr = uR - 0.5f * (dqR[1] - dqR[0]) / rR;
  const float pr = pR - 0.5f * (dqR[0] + dqR[1]) * cRc;
  const float ut1r = t1R - 0.5f * dqR[2];
  const float ut2r = t2R - 0.5f * dqR[3];
  float spl[NS], spr[NS];
  // increments of the face species densities over the cell's: rho Y_k + h_k
  float hL[NS], hR[NS];
  float HL = 0.f, HR = 0.f;
  float rl = 0.f, rr = 0.f;
  {
    const float sL = (dqL[0] + dqL[1]) * icL, sR = (dqR[0] + dqR[1]) * icR;
    const float icL2 = icL * icL, icR2 = icR * icR;
#pragma unroll
    for (int q = 0; q < MR::Q; ++q) {  // four species a group
      const float4 gLL = ld_group(rec, MR::Y + q, N, cLL), gL = ld_group(rec, MR::Y + q, N, cL);
      const float4 gR = ld_group(rec, MR::Y + q, N, cR), gRR = ld_group(rec, MR::Y + q, N, cRR);
#pragma unroll
      for (int l = 0; l < 4; ++l) {
        const int n = 4 * q + l;
        if (n >= NS) break;
        const float yLL = grp(gLL, l), yL = grp(gL, l), yR = grp(gR, l), yRR = grp(gRR, l);
        float dsL = 0.f, dsR = 0.f;
        if (slopes) {
          const float ryL = rL * yL, ryR = rR * yR;
          dsL = mc_limitf(ryL - rLL * yLL - yL * dpl * icL2, ryR - ryL - yL * dpc * icL2);
          dsR = mc_limitf(ryR - ryL - yR * dpc * icR2, rRR * yRR - ryR - yR * dpr * icR2);
        }
        hL[n] = 0.5f * (dsL + yL * sL);
        hR[n] = -(0.5f * (dsR + yR * sR));
        HL += hL[n];
        HR += hR[n];
        spl[n] = yL * rL + hL[n];
        spr[n] = yR * rR + hR[n];
        rl += spl[n];
        rr += spr[n];
      }
    }
    const float irl = 1.f / rl, irr = 1.f / rr;
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      spl[n] *= irl;
      spr[n] *= irr;
    }
  }
  const float pref = m.p_ref;
  const float cavg = 0.5f * (cRc + cLc);
  const float rwl = mix_rwf<NS>(m, spl), rwr = mix_rwf<NS>(m, spr);
  // The mixture coefficients of the two face states are kept: the upwind
  // state of the solver has one of their compositions, and so has the star
  // state unless a species density is clamped.
  float CLc[5], CRc[5];
  int rgL = 0, rgR = 0;
  float cl, cr;
  if constexpr (MIX) {
    const float TLs = (pl + pref) / (rl * rwl), TRs = (pr + pref) / (rr * rwr);
    rgL = TLs < m.tmid ? 0 : 1;
    rgR = TRs < m.tmid ? 0 : 1;
    E::template coefs<5>(m, spl, rgL, CLc);
    E::template coefs<5>(m, spr, rgR, CRc);
    cl = E::cs_C(CLc, rwl, rl, TLs, pl + pref);
    cr = E::cs_C(CRc, rwr, rr, TRs, pr + pref);
  } else {
    cl = E::cs_rp(m, spl, rwl, rl, pl + pref);
    cr = E::cs_rp(m, spr, rwr, rr, pr + pref);
  }
  float fl_rho, fl_un, fl_ut1, fl_ut2;
  ff fl_E, fl_ei;
  float flY[NS];
  if (!f.laxf) {
    const float wsmall = 1.17549435e-38f;
    const float wl = fmaxf(wsmall, cl * rl);
    const float wr = fmaxf(wsmall, cr * rr);
    const float iw = 1.f / (wl + wr);
    const float pstar = fmaxf(wsmall - pref, ((wr * pl + wl * pr) + wl * wr * (unl - unr)) * iw);
    float ustar = ((wl * unl + wr * unr) + (pl - pr)) * iw;  // offset from Un
    bool mask = ustar + Unf > 0.f;
    float uo = mask ? unl : unr;
    float po = mask ? pl : pr;
    const float usa = ustar + Unf;
    const bool m0 = fabsf(usa) < 1e-12f * 0.5f * (fabsf(unl + Unf) + fabsf(unr + Unf)) || usa == 0.f;
    ustar = m0 ? -Unf : ustar;
    float rspo[NS];
    float ro = 0.f;
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      const float a = rl * spl[n], bq = rr * spr[n];
      rspo[n] = m0 ? 0.5f * (a + bq) : (mask ? a : bq);
      ro += rspo[n];
    }
    uo = m0 ? 0.5f * (unl + unr) : uo;
    po = m0 ? 0.5f * (pl + pr) : po;
    float Yt[NS];
    {
      const float y = 1.f / ro;
#pragma unroll
      for (int n = 0; n < NS; ++n) Yt[n] = rspo[n] * y;
    }
    // the upwind state is the upwind face state (u* != 0): its sound speed
    const float co = (MIX && !m0) ? (mask ? cl : cr) : E::cs_rp(m, Yt, mix_rwf<NS>(m, Yt), ro, po + pref);
    const float drho = (pstar - po) / (co * co);
    float rspstar[NS];
    float rstar = 0.f;
    bool clamped = false;
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      const float v = rspo[n] + drho * Yt[n];
      clamped |= !(v >= 0.f);
      rspstar[n] = fmaxf(0.f, v);
      rstar += rspstar[n];
    }
    float cstar = 0.f;
    bool star_done = false;
    if constexpr (MIX) {
      if (!m0 && !clamped) {  // the upwind face state's composition at (rstar, pstar)
        const float rwo = mask ? rwl : rwr;
        const float Ts = (pstar + pref) / (rstar * rwo);
        if ((Ts < m.tmid ? 0 : 1) == (mask ? rgL : rgR)) {
          float Co[5];
#pragma unroll
          for (int n = 0; n < 5; ++n) Co[n] = mask ? CLc[n] : CRc[n];
          cstar = E::cs_C(Co, rwo, rstar, Ts, pstar + pref);
          star_done = true;
        }
      }
    }
    if (!star_done) {
      const float y = 1.f / rstar;
#pragma unroll
      for (int n = 0; n < NS; ++n) Yt[n] = rspstar[n] * y;
      cstar = E::cs_rp(m, Yt, mix_rwf<NS>(m, Yt), rstar, pstar + pref);
    }
    const float sgnm = copysignf(1.f, m0 ? 0.f : ustar + Unf);
    float spout = co - sgnm * (uo + Unf);
    float spin = cstar - sgnm * (m0 ? 0.f : ustar + Unf);
    const float ushock = 0.5f * (spin + spout);
    mask = pstar < po;
    spout = mask ? spout : ushock;
    spin = mask ? spin : ushock;
    const float scr = (fabsf(spout - spin) < 1e-30f) ? 1e-8f * cavg : spout - spin;
    const float frac = fmaxf(0.f, fminf(1.f, (1.f + (spout + spin) / scr) * 0.5f));
    mask = !m0 && ustar + Unf > 0.f;
    float iv1 = mask ? ut1l : ut1r;
    float iv2 = mask ? ut2l : ut2r;
    iv1 = m0 ? 0.5f * (ut1l + ut1r) : iv1;
    iv2 = m0 ? 0.5f * (ut2l + ut2r) : iv2;
    const bool mout = spout < 0.f, min_ = spin >= 0.f;
    float iu = frac * ustar + (1.f - frac) * uo;
    float gdp = frac * pstar + (1.f - frac) * po;
    iu = mout ? uo : iu;
    gdp = mout ? po : gdp;
    iu = min_ ? ustar : iu;
    gdp = min_ ? pstar : gdp;
    float rgd = 0.f;
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      float g = frac * rspstar[n] + (1.f - frac) * rspo[n];
      g = mout ? rspo[n] : g;
      g = min_ ? rspstar[n] : g;
      flY[n] = g;
      rgd += g;
    }
    const ff gdpa = ff_sum(gdp, pref);  // absolute pressure, exact
    ff regd;
    if (!m0 && !clamped) {
      // The Godunov state has the upwind face's composition, and its density
      // is the upwind face's plus w drho (w: the star state's share).  Both
      // are formed in double-float arithmetic as the upwind cell's stored
      // values plus the FP32 increments (slopes, star jump), so the FP32
      // rounding falls on the increments only: rho e carries the formation
      // energies, which turn a 6e-8 rounding of Y_k or of rho into far more
      // than rho e varies by across the flame.
      const long long cu = mask ? cL : cR;
      const float4* xr = mixed_x<NS>(b) + cu;
      const float w = min_ ? 1.f : (mout ? 0.f : frac);
      const float H = mask ? HL : HR, irf = mask ? 1.f / rl : 1.f / rr;
      const float4 rr_cell = __ldg(xr + (long long)MPair<NS>::RHO * N);  // (rho, R/Wbar) of the upwind cell
      const ff rg = ff_add(pair_of(rr_cell, 0), H + w * drho);
      if constexpr (MIX) {
        // Y_k of the Godunov state = the cell's Y_k + d_k, d_k = (h_k - Y_k H) / rho
        // in FP32; its mixture sums are the cell's (pairs) + sum_k d_k c_k (FP32)
        float dY[NS];
        ld_groups<NS>(rec, MR::Y, N, cu, dY);  // the upwind cell's Y_k
#pragma unroll
        for (int n = 0; n < NS; ++n) {
          const float h = mask ? hL[n] : hR[n];
          dY[n] = (h - dY[n] * H) * irf;
        }
        regd = ff_mul(rg, e_godunov_ff<NS>(m, xr, N, dY, rg, gdpa, pair_of(rr_cell, 1)));
      } else {
        regd = ff_mul(rg, e_rp_ff<NS, false>(m, nullptr, rg, gdpa));
      }
    } else {
      regd = ff_mul(e_rp_ff_rY<NS, MIX>(m, flY, rgd, gdpa), rgd);
    }
    const float iua = iu + Unf, iv1a = iv1 + Ut1f, iv2a = iv2 + Ut2f;  // absolute velocities
    fl_rho = rgd * iua;
#pragma unroll
    for (int n = 0; n < NS; ++n) flY[n] *= iua;
    fl_un = fl_rho * iua + gdp;  // p_ref dropped: zero divergence
    fl_ut1 = fl_rho * iv1a;
    fl_ut2 = fl_rho * iv2a;
    const ff iud = ff_add(fc.Uff[d], iu);  // U + u' in double-float
    const ff tot = ff_add(ff_add(regd, 0.5f * rgd * (iua * iua + iv1a * iv1a + iv2a * iv2a)), gdpa);
    fl_E = ff_mul(iud, tot);
    fl_ei = ff_mul(iud, regd);
  } else {
    // Lax-Friedrichs on absolute velocities (U + u')
    const double Un = fc.Ud[d];
    const float unlA = unl + Unf, unrA = unr + Unf, ut1lA = ut1l + Ut1f, ut1rA = ut1r + Ut1f;
    const float ut2lA = ut2l + Ut2f, ut2rA = ut2r + Ut2f;
    const double pla = (double)pl + (double)pref, pra = (double)pr + (double)pref;
    const double el = e_rpY_fp64<NS, MIX>(md, spl, rl, pla);
    const double er = e_rpY_fp64<NS, MIX>(md, spr, rr, pra);
    const double r_elt = (double)rl * (el + (double)(0.5f * (unlA * unlA + ut1lA * ut1lA + ut2lA * ut2lA)));
    const double r_ert = (double)rr * (er + (double)(0.5f * (unrA * unrA + ut1rA * ut1rA + ut2rA * ut2rA)));
    const float wl = fmaxf(1.17549435e-38f, cl * rl);
    const float wr = fmaxf(1.17549435e-38f, cr * rr);
    float ustar = ((wl * unlA + wr * unrA) + (pl - pr)) / (wl + wr);
    const bool m0 = fabsf(ustar) < 1e-12f * 0.5f * (fabsf(unlA) + fabsf(unrA)) || ustar == 0.f;
    ustar = m0 ? 0.f : ustar;
    const float mw = fabsf(ustar) + 0.5f * (cr + cl);
    fl_rho = 0.f;
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      flY[n] = 0.5f * ((rl * unlA * spl[n] + rr * unrA * spr[n]) - mw * (rr * spr[n] - rl * spl[n]));
      fl_rho += flY[n];
    }
    fl_un = 0.5f * ((rl * unlA * unlA + pl + rr * unrA * unrA + pr) - mw * (rr * unrA - rl * unlA));
    fl_ut1 = 0.5f * ((rl * ut1lA * unlA + rr * ut1rA * unrA) - mw * (rr * ut1rA - rl * ut1lA));
    fl_ut2 = 0.5f * ((rl * ut2lA * unlA + rr * ut2rA * unrA) - mw * (rr * ut2rA - rl * ut2lA));
    const double mwd = (double)mw;
    fl_E = ff_of(0.5 * (((r_elt + pla) * (Un + (double)unl) + (r_ert + pra) * (Un + (double)unr)) -
                        mwd * (r_ert - r_elt)));
    fl_ei = ff_of(0.5 * (((double)rl * el * (Un + (double)unl) + (double)rr * er * (Un + (double)unr)) -
                         mwd * ((double)rr * er - (double)rl * el)));
  }
  F[URHO] = fl_rho;
  F[UMX] = fl_un;  // rotated order
  F[UMY] = fl_ut1;
  F[UMZ] = fl_ut2;
  F[UEDEN] = 0.f;  // energy fluxes travel in double-float (FE, FEI)
  F[UEINT] = 0.f;
  F[UTEMP] = 0.f;
  FE = fl_E;
  FEI = fl_ei;
#pragma unroll
  for (int n = 0; n < NS; ++n) F[UFS + n] = flY[n];
}

// FP32 diffusion flux (not area-scaled), added to F (momentum in the rotated
// order of hydro_face_f).  st: the cell stride of direction d; s1, s2: those
// of the transverse axes t1, t2.
template <int NS>
__device__ __forceinline__ void diffusion_face_f(const DevBox& b, const DevFlags& f, int d, long long cR,
                                                 long long st, long long s1, long long s2, const FaceConsts& fc,
                                                 float* F) {
  using MR = MRec<NS>;
  const float4* rec = reinterpret_cast<const float4*>(b.rec);
  const long long N = b.ncell;
  const float4* xrec = mixed_x<NS>(b);
  const long long cL = cR - st;
  const int t1 = (d == 0) ? 1 : 0, t2 = (d == 2) ? 1 : 2;
  const bool harm = f.harmonic != 0;
  // mu, xi, lambda follow D_k: the group holding mu (and the next one where
  // they straddle two)
  constexpr int gm = MR::D + NS / 4, lm = NS % 4;
  const float4 tR0 = ld_group(rec, gm, N, cR), tL0 = ld_group(rec, gm, N, cL);
  float4 tR1 = tR0, tL1 = tL0;
  if constexpr (lm >= 2) {
    tR1 = ld_group(rec, gm + 1, N, cR);
    tL1 = ld_group(rec, gm + 1, N, cL);
  }
  auto coef = [&](const float4& t0, const float4& t1, int i) {
    return lm + i < 4 ? grp(t0, lm + i) : grp(t1, lm + i - 4);
  };
  const float mu = face_coeff(coef(tR0, tR1, 0), coef(tL0, tL1, 0), harm);
  const float xi = face_coeff(coef(tR0, tR1, 1), coef(tL0, tL1, 1), harm);
  const float lam = face_coeff(coef(tR0, tR1, 2), coef(tL0, tL1, 2), harm);
  // velocity gradients in the rotated frame (0: normal, 1: t1, 2: t2),
  // grad[c][a] = d u_c / d x_a
  float grad[3][3];
  const float4 aR = rot_g0(ld_group(rec, MR::G0, N, cR), d), aL = rot_g0(ld_group(rec, MR::G0, N, cL), d);
  const float uR[3] = {aR.y, aR.z, aR.w};
  const float uL[3] = {aL.y, aL.z, aL.w};
  const float dxi = fc.dxi[d];
#pragma unroll
  for (int c = 0; c < 3; ++c) grad[c][0] = dxi * (uR[c] - uL[c]);
#pragma unroll
  for (int a = 1; a < 3; ++a) {
    const long long sa = a == 1 ? s1 : s2;
    const float q4 = 0.25f * fc.dxi[a == 1 ? t1 : t2];
    const float4 vRp = ld_group(rec, MR::G0, N, cR + sa), vLp = ld_group(rec, MR::G0, N, cL + sa);
    const float4 vRm = ld_group(rec, MR::G0, N, cR - sa), vLm = ld_group(rec, MR::G0, N, cL - sa);
    // components of G0 = (rho, u, v, w) along axis a and along the normal
    const int ia = 1 + (a == 1 ? t1 : t2), in = 1 + d;
    grad[a][a] = (grp(vRp, ia) + grp(vLp, ia) - grp(vRm, ia) - grp(vLm, ia)) * q4;
    grad[0][a] = (grp(vRp, in) + grp(vLp, in) - grp(vRm, in) - grp(vLm, in)) * q4;
  }
  const float divu = grad[0][0] + grad[1][1] + grad[2][2];
  float tau[3];
  tau[0] = mu * (2.f * grad[0][0] - (2.f / 3.f) * divu) + xi * divu;
#pragma unroll
  for (int a = 1; a < 3; ++a) tau[a] = mu * (grad[0][a] + grad[a][0]);
  constexpr int gT = MPair<NS>::XT + NS / 2;  // the pair group holding T
  const float4 xtR = __ldg(xrec + gT * N + cR), xtL = __ldg(xrec + gT * N + cL);
  const float dT = pair_diff(pair_of(xtR, NS % 2), pair_of(xtL, NS % 2));
  // the work term needs absolute velocities: the offsets plus the box's reference
  const float Uf[3] = {fc.U[d], fc.U[t1], fc.U[t2]};
  float fE = 0.5f * (-tau[0] * (uR[0] + uL[0] + 2.f * Uf[0]) - tau[1] * (uR[1] + uL[1] + 2.f * Uf[1]) -
                     tau[2] * (uR[2] + uL[2] + 2.f * Uf[2])) -
             lam * dxi * dT;
  const bool spec = f.diffuse_spec != 0;
  const bool ener = (f.diffuse_temp != 0) || (f.diffuse_enth != 0);
  {
    const float pR = __ldg(reinterpret_cast<const float*>(rec + (long long)MR::G1 * N + cR));
    const float pL = __ldg(reinterpret_cast<const float*>(rec + (long long)MR::G1 * N + cL));
    // d ln p / dx from the offset pressure: p = p_ref + p'.
    const float dlnp = dxi * (pR - pL) / (0.5f * (pR + pL) + fc.pref);
    float Vd[NS], Yf[NS], hf[NS];
    float Vc = 0.f;
#pragma unroll
    for (int q = 0; q < MR::Q; ++q) {  // four species a group
      const float4 yR = ld_group(rec, MR::Y + q, N, cR), yL = ld_group(rec, MR::Y + q, N, cL);
      const float4 hR = ld_group(rec, MR::H + q, N, cR), hL = ld_group(rec, MR::H + q, N, cL);
      const float4 dR = (MR::D + q == gm) ? tR0 : ld_group(rec, MR::D + q, N, cR);
      const float4 dL = (MR::D + q == gm) ? tL0 : ld_group(rec, MR::D + q, N, cL);
      // the pair groups of X_{4q} .. X_{4q+3}
      float4 xR[2], xL[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int gx = MPair<NS>::XT + 2 * q + h;
        if (2 * (2 * q + h) >= NS) break;
        xR[h] = gx == gT ? xtR : __ldg(xrec + gx * N + cR);
        xL[h] = gx == gT ? xtL : __ldg(xrec + gx * N + cL);
      }
#pragma unroll
      for (int l = 0; l < 4; ++l) {
        const int n = 4 * q + l;
        if (n >= NS) break;
        const ff x1 = pair_of(xR[l / 2], l % 2), x2 = pair_of(xL[l / 2], l % 2);
        const float dX = pair_diff(x1, x2);
        const float Xface = 0.5f * ((x1.hi + x2.hi) + (x1.lo + x2.lo));
        Yf[n] = 0.5f * (grp(yR, l) + grp(yL, l));
        hf[n] = 0.5f * (grp(hR, l) + grp(hL, l));
        const float D = face_coeff(grp(dR, l), grp(dL, l), harm);
        Vd[n] = -D * (dxi * dX + (Xface - Yf[n]) * dlnp);
        Vc += Vd[n];
        fE += Vd[n] * hf[n];
      }
    }
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      fE -= Yf[n] * hf[n] * Vc;
      if (spec) F[UFS + n] += Vd[n] - Yf[n] * Vc;
    }
  }
  if (f.diffuse_vel) {
#pragma unroll
    for (int a = 0; a < 3; ++a) F[UMX + a] -= tau[a];
  }
  if (ener) F[UEDEN] += fE;
}

// Dynamic shared memory of the mixed-precision flux pass: the
// face fluxes of all three directions of a tile at once, FP32 except the
// total and internal energy fluxes (double-float pairs); the temperature
// component, whose flux is zero, is not staged.
template <int NS, class TL>
constexpr size_t mixed_flux_smem_bytes() {
  return (size_t)(TL::F0 + TL::F1 + TL::F2) * (2 * sizeof(double) + sizeof(float) * (4 + NS));
}

// Shared-memory staging of the face fluxes of a tile, all three directions
// at once: the total and internal energy fluxes first, as double-float
// pairs, then the other components in FP32.  Direction d's faces start at
// face slot base(d).
template <int NS, class TL>
struct FaceStage {
  static constexpr int TOT = TL::F0 + TL::F1 + TL::F2;
  float2* e;  // [2][TOT]: UEDEN, UEINT
  float* v;   // [4 + NS][TOT]: rho, the momenta, the species (row()); UTEMP's flux is zero
  __device__ static constexpr int base(int d) { return d == 0 ? 0 : d == 1 ? TL::F0 : TL::F0 + TL::F1; }
  // the row of v holding component n (not UEDEN, UEINT, UTEMP)
  __device__ static constexpr int row(int n) { return n < UEDEN ? n : n - 3; }
  // F(slot, n) - F(slot2, n) for component n, exactly for the FP32
  // components (TwoSum), to double-float accuracy for the energy fluxes
  __device__ ff diff(int n, int slot, int slot2) const {
    if (n == UEDEN || n == UEINT) {
      const float2 a = e[(n == UEINT) * TOT + slot], c = e[(n == UEINT) * TOT + slot2];
      return ff_sub(ff{a.x, a.y}, ff{c.x, c.y});
    }
    if (n == UTEMP) return ff_of(0.f);
    return ff_sum(v[row(n) * TOT + slot], -v[row(n) * TOT + slot2]);
  }
  // the staged flux of component n as a double (the FP32 ones widened
  // exactly, on the integer pipe where they are normal or zero)
  __device__ double get(int n, int slot) const {
    if (n == UEDEN || n == UEINT) {
      const float2 a = e[(n == UEINT) * TOT + slot];
      return ff_to_double(ff{a.x, a.y});
    }
    if (n == UTEMP) return 0.0;
    return f2d_exact(v[row(n) * TOT + slot]);
  }
};

// One face of direction d (index fi in the tile's face block of that
// direction, nf0 x nf1 x nf2): hydrodynamic and diffusion fluxes, staged
// (the rotated momentum components at their axes).
template <int NS, bool MIX, class TL, bool EXPORT>
__device__ __forceinline__ void face_mixed(const DevBox& b, const MechF<NS>& m, const DevMech<NS>& md,
                                           const DevFlags& f, const int o[3], const long long stv[3], int d, int fi,
                                           int nf0, int nf1, bool diff, const FaceConsts& fc,
                                           const FaceStage<NS, TL>& fs, const FluxBox* fxb, const Geo& g) {
  constexpr int NVAR = 7 + NS;
  const int fx = fi % nf0, fy = (fi / nf0) % nf1, fz = fi / (nf0 * nf1);
  const int i = o[0] + fx, j = o[1] + fy, k = o[2] + fz;
  const long long cR = (i - b.g2lo[0]) + (j - b.g2lo[1]) * stv[1] + (k - b.g2lo[2]) * stv[2];
  // strides of the normal and the two transverse axes
  const long long st = d == 0 ? stv[0] : (d == 1 ? stv[1] : stv[2]);
  const long long s1 = d == 0 ? stv[1] : stv[0], s2 = d == 2 ? stv[1] : stv[2];
  float F[NVAR];
  ff FE = ff_of(0.f), FEI = ff_of(0.f);
  if (f.do_hydro) {
    hydro_face_f<NS, MIX>(b, m, md, f, d, cR, st, fc, F, FE, FEI);
  } else {
#pragma unroll
    for (int n = 0; n < NVAR; ++n) F[n] = 0.f;
  }
  if (diff) diffusion_face_f<NS>(b, f, d, cR, st, s1, s2, fc, F);
  const int slot = FaceStage<NS, TL>::base(d) + fi;
  constexpr int TOT = FaceStage<NS, TL>::TOT;
  const int rowt1 = d == 0 ? UMY : UMX, rowt2 = d == 2 ? UMY : UMZ;  // rows of the transverse momenta
#pragma unroll
  for (int n = 0; n < NVAR; ++n) {
    if (n == UEDEN || n == UEINT || n == UTEMP) continue;  // UTEMP's flux is zero
    const int comp = n == UMX ? UMX + d : (n == UMY ? rowt1 : (n == UMZ ? rowt2 : n));
    fs.v[FaceStage<NS, TL>::row(comp) * TOT + slot] = F[n];
  }
  const ff fe = ff_add(FE, F[UEDEN]);
  fs.e[slot] = make_float2(fe.hi, fe.lo);
  fs.e[TOT + slot] = make_float2(FEI.hi, FEI.lo);
  // Export (refluxing), times the face area, in FP64; the normal-momentum
  // flux gets back the p_ref the FP32 form leaves out.  A face shared by two
  // tiles is written twice, with the same values.  A separate instantiation
  // (EXPORT), so that the plain pass carries none of it.
  if constexpr (EXPORT) {
    const double A = d == 0 ? g.area[0] : (d == 1 ? g.area[1] : g.area[2]);
    double* q = fxb->p[d] + (i - fxb->b[d][0]) + (long long)(j - fxb->b[d][1]) * fxb->js[d] +
                (long long)(k - fxb->b[d][2]) * fxb->ks[d];
    const long long ns = fxb->ns[d];
#pragma unroll
    for (int n = 0; n < NVAR; ++n) {
      if (n == UEDEN || n == UEINT || n == UTEMP) continue;
      const int comp = n == UMX ? UMX + d : (n == UMY ? rowt1 : (n == UMZ ? rowt2 : n));
      q[comp * ns] = (n == UMX ? f2d_exact(F[n]) + g.p_ref : f2d_exact(F[n])) * A;
    }
    q[UEDEN * ns] = ff_to_double(fe) * A;
    q[UEINT * ns] = ff_to_double(FEI) * A;
    q[UTEMP * ns] = 0.0;
  }
}

// Pass 2 over the tile list; CTA b takes tiles b, b + gridDim.x, ... (one
// each with one CTA per tile; a persistent launch strides over the list).
// All faces of a tile, the three directions together, are evaluated before
// one barrier (per-direction barriers would leave most warps idle while the
// last faces of a direction finish: 288 faces of 8x8x4 cells on 256 threads
// take two rounds): each thread the low x, y and z faces of its own cell,
// then the tile's high boundary faces.  Then each cell sums its six faces,
// each difference F_lo - F_hi of two staged FP32 fluxes taken exactly and
// scaled by 1/dx in double-float arithmetic on the FP32 pipe (on cubic
// cells the three differences summed first and scaled once), rounded to
// FP64 once at the end: about 48 significant bits, so the telescoping sum
// conserves to far below the form's error.
template <int NS, bool MIX, class TL = TileDefault, bool STRICT = false, bool EXPORT = false>
__global__ void __launch_bounds__(TL::NT, TL::MINB)
    flux_kernel_mixed(const DevBox* __restrict__ boxes, const int4* __restrict__ tiles, int ntiles,
                      const __grid_constant__ MechF<NS> m, const __grid_constant__ DevMech<NS> md, const DevFlags f,
                      const Geo g, unsigned long long* __restrict__ counters, const FluxBox* __restrict__ fluxes) {
  constexpr int NVAR = 7 + NS;
  extern __shared__ double flux_dyn_smem[];
  FaceStage<NS, TL> fs;
  fs.e = reinterpret_cast<float2*>(flux_dyn_smem);
  fs.v = reinterpret_cast<float*>(flux_dyn_smem + 2 * FaceStage<NS, TL>::TOT);
  const bool diff = f.diffuse_vel || f.diffuse_temp || f.diffuse_spec || f.diffuse_enth;
  const int tx = threadIdx.x % TL::TX, ty = (threadIdx.x / TL::TX) % TL::TY, tz = threadIdx.x / (TL::TX * TL::TY);
  const ff dxi[3] = {ff_of(g.dxinv[0]), ff_of(g.dxinv[1]), ff_of(g.dxinv[2])};
  const bool iso = g.dxinv[0] == g.dxinv[1] && g.dxinv[1] == g.dxinv[2];  // cubic cells
  for (int tb = blockIdx.x; tb < ntiles; tb += gridDim.x) {
    const int4 t = tiles[tb];
    const DevBox& b = boxes[t.x];
    const int o[3] = {t.y, t.z, t.w};
    const int ext[3] = {min(TL::TX, b.hi[0] - o[0] + 1), min(TL::TY, b.hi[1] - o[1] + 1),
                        min(TL::TZ, b.hi[2] - o[2] + 1)};
    const bool mine = tx < ext[0] && ty < ext[1] && tz < ext[2];
    const long long stv[3] = {1, b.n2[0], (long long)b.n2[0] * b.n2[1]};
    const FluxBox* fxb = EXPORT ? fluxes + t.x : nullptr;
    __shared__ FaceConsts fc;  // the box's reference velocity, 1/dx, p_ref
    if (threadIdx.x == 0) face_consts(b, g, fc);
    __syncthreads();
    // Cell-major face order: the faces of direction d form a block of
    // (ext + e_d) faces.  In rounds 0-2 each thread evaluates the low x, y
    // and z faces of its own cell (a warp revisits the same cells' records
    // three times in a row); the later rounds spread the tile's high
    // boundary faces (x = ext[0], y = ext[1], z = ext[2]) over all threads.
    // One call site: the face code is inlined once.
    {
      const int nb0 = ext[1] * ext[2], nb1 = ext[0] * ext[2], nb2 = ext[0] * ext[1];
      const int nrounds = 3 + (nb0 + nb1 + nb2 + TL::NT - 1) / TL::NT;
#pragma unroll 1
      for (int k = 0; k < nrounds; ++k) {
        int d, c0, c1, c2;
        bool act;
        if (k < 3) {
          d = k;
          act = mine;
          c0 = tx;
          c1 = ty;
          c2 = tz;
        } else {
          const int q = (k - 3) * TL::NT + threadIdx.x;
          act = q < nb0 + nb1 + nb2;
          d = q < nb0 ? 0 : (q < nb0 + nb1 ? 1 : 2);
          const int r = q - (d == 0 ? 0 : (d == 1 ? nb0 : nb0 + nb1));
          const int e1 = d == 0 ? ext[1] : ext[0];  // extent of the first of the other two axes
          c0 = d == 0 ? ext[0] : r % e1;
          c1 = d == 1 ? ext[1] : (d == 0 ? r % e1 : r / e1);
          c2 = d == 2 ? ext[2] : r / e1;
        }
        if (act) {
          const int nf0 = ext[0] + (d == 0), nf1 = ext[1] + (d == 1);
          face_mixed<NS, MIX, TL, EXPORT>(b, m, md, f, o, stv, d, c0 + nf0 * (c1 + nf1 * c2), nf0, nf1, diff, fc,
                                          fs, fxb, g);
        }
      }
    }
    __syncthreads();
    bool bad = false;
    if (mine) {
      const int i = o[0] + tx, j = o[1] + ty, k = o[2] + tz;
      double* r = b.R + (i - b.rb[0]) + (long long)(j - b.rb[1]) * b.rj + (long long)(k - b.rb[2]) * b.rk;
      if constexpr (STRICT) {  // PC_PRECISION_MIXED_FP64: each flux widened to FP64, summed in FP64
        double acc[NVAR];
#pragma unroll
        for (int n = 0; n < NVAR; ++n) acc[n] = 0.0;
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const int nf0 = ext[0] + (d == 0), nf1 = ext[1] + (d == 1);
          const int flo = FaceStage<NS, TL>::base(d) + tx + nf0 * (ty + nf1 * tz);
          const int fhi = flo + ((d == 0) ? 1 : (d == 1) ? nf0 : nf0 * nf1);
#pragma unroll
          for (int n = 0; n < NVAR; ++n) acc[n] = fma(fs.get(n, flo) - fs.get(n, fhi), g.dxinv[d], acc[n]);
        }
#pragma unroll
        for (int n = 0; n < NVAR; ++n) {
          bad |= !isfinite(acc[n]);
          r[n * b.rn] = acc[n];
        }
      } else {
        ff acc[NVAR];
#pragma unroll
        for (int n = 0; n < NVAR; ++n) acc[n] = ff_of(0.f);
        int flo[3], fhi[3];
#pragma unroll
        for (int d = 0; d < 3; ++d) {
          const int nf0 = ext[0] + (d == 0), nf1 = ext[1] + (d == 1);
          flo[d] = FaceStage<NS, TL>::base(d) + tx + nf0 * (ty + nf1 * tz);
          fhi[d] = flo[d] + ((d == 0) ? 1 : (d == 1) ? nf0 : nf0 * nf1);
        }
        if (iso) {  // one 1/dx: the three exact differences summed, then scaled once
#pragma unroll
          for (int n = 0; n < NVAR; ++n)
            acc[n] = ff_mul(ff_add(ff_add(fs.diff(n, flo[0], fhi[0]), fs.diff(n, flo[1], fhi[1])),
                                   fs.diff(n, flo[2], fhi[2])),
                            dxi[0]);
        } else {
#pragma unroll
          for (int d = 0; d < 3; ++d)
#pragma unroll
            for (int n = 0; n < NVAR; ++n) acc[n] = ff_add(ff_mul(fs.diff(n, flo[d], fhi[d]), dxi[d]), acc[n]);
        }
        // to FP64: on the integer pipe (and one FP64 addition) unless a lane
        // of the warp holds a subnormal, infinite or NaN part
        bool fast = true;
#pragma unroll
        for (int n = 0; n < NVAR; ++n) fast &= f2d_fast_ok(acc[n].hi) && f2d_fast_ok(acc[n].lo);
        double v[NVAR];
        if (__all_sync(__activemask(), fast)) {
#pragma unroll
          for (int n = 0; n < NVAR; ++n) v[n] = ff_to_double_fast(acc[n]);
        } else {
#pragma unroll
          for (int n = 0; n < NVAR; ++n) v[n] = ff_to_double(acc[n]);
        }
#pragma unroll
        for (int n = 0; n < NVAR; ++n) {
          bad |= !isfinite(v[n]);
          r[n * b.rn] = v[n];
        }
      }
    }
    if (f.check_output) warp_count(&counters[kCounterNonfinite], bad);
    if (threadIdx.x == 0) atomicAdd(&counters[kCounterCells], (unsigned long long)(ext[0] * ext[1] * ext[2]));
    __syncthreads();  // the next tile's faces overwrite the staging
  }
}

// Host: launch the mixed flux pass at tile shape TL, one CTA per tile or
// (persistent) as many CTAs as are resident on the device at once; with
// fluxes, the instantiation that also exports the face fluxes.
template <int NS, bool MIX, class TL, bool STRICT, bool EXPORT>
inline cudaError_t launch_flux_mixed_kernel(const DevBox* boxes, const int4* tiles, int ntiles, const MechF<NS>& mf,
                                            const DevMech<NS>& md, const DevFlags& f, const Geo& g,
                                            unsigned long long* counters, cudaStream_t s, bool persistent,
                                            const FluxBox* fluxes) {
  static std::atomic<unsigned long long> opted{0};  // bit per device
  static std::atomic<int> resident[64];             // persistent grid per device (0: not known yet)
  constexpr size_t smem = mixed_flux_smem_bytes<NS, TL>();
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = (dev >= 0 && dev < 64) ? (1ull << dev) : 0ull;
  if (!bit || !(opted.load() & bit)) {
    e = cudaFuncSetAttribute(flux_kernel_mixed<NS, MIX, TL, STRICT, EXPORT>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    opted.fetch_or(bit);
  }
  int grid = ntiles;
  if (persistent) {
    int r = bit ? resident[dev].load() : 0;
    if (r <= 0) {
      r = resident_ctas(flux_kernel_mixed<NS, MIX, TL, STRICT, EXPORT>, TL::NT, smem);
      if (bit && r > 0) resident[dev].store(r);
    }
    if (r > 0 && r < grid) grid = r;
  }
  flux_kernel_mixed<NS, MIX, TL, STRICT, EXPORT><<<grid, TL::NT, smem, s>>>(boxes, tiles, ntiles, mf, md, f, g,
                                                                              counters, fluxes);
  return cudaGetLastError();
}
template <int NS, bool MIX, class TL, bool STRICT = false>
inline cudaError_t launch_flux_mixed_at(const DevBox* boxes, const int4* tiles, int ntiles, const MechF<NS>& mf,
                                        const DevMech<NS>& md, const DevFlags& f, const Geo& g,
                                        unsigned long long* counters, cudaStream_t s, bool persistent,
                                        const FluxBox* fluxes = nullptr) {
  if (ntiles <= 0) return cudaSuccess;
  return fluxes ? launch_flux_mixed_kernel<NS, MIX, TL, STRICT, true>(boxes, tiles, ntiles, mf, md, f, g, counters, s,
                                                                      persistent, fluxes)
                : launch_flux_mixed_kernel<NS, MIX, TL, STRICT, false>(boxes, tiles, ntiles, mf, md, f, g, counters,
                                                                       s, persistent, nullptr);
}

}  // namespace pcg
