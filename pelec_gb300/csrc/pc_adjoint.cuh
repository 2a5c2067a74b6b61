// pc_adjoint.cuh — hand-written reverse mode (vector-Jacobian product) of the
// FP64 MOL right-hand side of pc_kernels.cuh.
//
// Given the RHS cotangent rbar (valid cells), computes
//   Ubar = (dRHS/dU)^T rbar   on grow(valid, 2)
// in three passes that mirror the forward ones:
//   1. cell_kernel (the forward pass 1, unchanged): the per-cell records.
//   2. face_adjoint_kernel: one thread per face.  The face cotangent is
//      Fbar = (rbar_R - rbar_L) / V (the divergence transposed); the thread
//      re-evaluates the face flux with the forward's exact operation sequence
//      — so every limiter min/max, Riemann upwind / sonic / shock-rarefaction
//      switch and clipping branch takes the forward's decision — and then
//      runs the derivative of that branch path backwards, accumulating the
//      cotangents of the record fields of every stencil cell (LL, L, R, RR;
//      the transverse neighbours of the viscous stress) with FP64 atomics
//      into a record-shaped buffer.
//   3. cell_adjoint_kernel: one thread per cell.  Re-evaluates pass 1 and
//      pulls the record cotangents back to the conserved state: the EOS
//      temperature solve is differentiated by the implicit-function theorem
//      (e(T, Y) = e, so dT = (de - sum_k e_k dY_k) / cv), the transport fits
//      and mixture rules by their closed-form derivatives.
// The RHS does not read UEINT, and UTEMP only as the Newton initial guess
// (the converged T does not depend on it), so their cotangents are zero.
// Derivatives at the kinks of min/max/|x| take the side the forward chose.
#pragma once

#include "pc_kernels.cuh"

namespace pcg {

// ---------------------------------------------------------------------------
// Scalar helpers.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double horner4_d(const double c[4], double L) {
  // d/dL of c0 + L c1 + L^2 c2 + L^3 c3
  return fma(L, fma(L, 3.0 * c[3], 2.0 * c[2]), c[1]);
}

// Ties (equal arguments of a min/max, |x| at x = 0) take the same side as
// the Dual tangent of pc_dual.cuh: fmin/fmax keep their first argument, the
// clamps pass the derivative on their boundary, |x|' = +1 at x = +-0.  The
// synthetic states hit such ties exactly (first-order-extrapolated ghost
// layers, species that are exactly zero), so the convention matters.
__device__ __forceinline__ double abs_sign(double x) { return (x < 0.0) ? -1.0 : 1.0; }

// mc_limit reverse: ob is the cotangent of mc_limit(dl, dr); adds to dlb, drb.
__device__ __forceinline__ void mc_limit_rev(double dl, double dr, double ob, double& dlb, double& drb) {
  const double dcen = 0.5 * (dl + dr);
  const double adl = fabs(dl), adr = fabs(dr);
  const double dlim = (dl * dr >= 0.0) ? 2.0 * fmin(adl, adr) : 0.0;
  const double s = copysign(1.0, dcen);
  if (dlim <= fabs(dcen)) {
    if (dl * dr >= 0.0) {
      if (adl <= adr)
        dlb += ob * s * 2.0 * abs_sign(dl);
      else
        drb += ob * s * 2.0 * abs_sign(dr);
    }
  } else {
    const double q = 0.5 * ob * s * abs_sign(dcen);  // s |dcen|
    dlb += q;
    drb += q;
  }
}

// face_coef reverse.
__device__ __forceinline__ void face_coef_rev(double a, double b, bool harmonic, double ob, double& ab_, double& bb_) {
  if (harmonic) {
    const double ab = a * b;
    if (ab > 0.0) {
      const double s = a + b, is2 = 1.0 / (s * s);
      ab_ += ob * 2.0 * b * b * is2;
      bb_ += ob * 2.0 * a * a * is2;
    }
  } else {
    ab_ += 0.5 * ob;
    bb_ += 0.5 * ob;
  }
}

// ---------------------------------------------------------------------------
// EOS derivatives.  Mixture quantities enter through Y (mixture polynomial
// coefficients C_n = sum_k Y_k cpc[n][k]) and rw = R/Wbar = sum_k Y_k rW_k;
// the caller folds rwb into Yb.
// ---------------------------------------------------------------------------
template <int NS, class EOS>
struct EosAdj;

template <int NS>
struct EosAdj<NS, GammaLawEos<NS>> {
  // c = sqrt(gamma p / rho)
  __device__ static void cs_rp(const DevMech<NS>& m, const double*, double, double rho, double p, double cb, double*,
                               double&, double& rhob, double& pb) {
    const double c = sqrt(m.gamma * p / rho);
    if (!(c > 0.0)) return;
    const double gb = cb / (2.0 * c);
    pb += gb * m.gamma / rho;
    rhob -= gb * m.gamma * p / (rho * rho);
  }
  __device__ static void cs_T(const DevMech<NS>& m, const double* Y, double rw, double rho, double, double p,
                              double cb, double* Yb, double& rwb, double& rhob, double&, double& pb) {
    cs_rp(m, Y, rw, rho, p, cb, Yb, rwb, rhob, pb);
  }
  // e = p / (gm1 rho)
  __device__ static void e_rp(const DevMech<NS>& m, const double*, double, double rho, double p, double eb, double*,
                              double&, double& rhob, double& pb) {
    pb += eb / (m.gm1 * rho);
    rhob -= eb * p / (m.gm1 * rho * rho);
  }
  // h_k = cp_k T
  __device__ static void hi_dT(const DevMech<NS>& m, double, double* dh) {
#pragma unroll
    for (int k = 0; k < NS; ++k) dh[k] = m.cpk[k];
  }
  // T = e gm1 / rw: adds the cotangents of e and rw.
  __device__ static void rey2t(const DevMech<NS>& m, const double*, double rw, double T, double Tb, double& eb,
                               double*, double& rwb) {
    eb += Tb * m.gm1 / rw;
    rwb -= Tb * T / rw;
  }
};

template <int NS>
struct EosAdj<NS, IdealMixEos<NS>> {
  using E = IdealMixEos<NS>;
  // Cotangents of C_0..C_{nc-1} to Y.
  __device__ static void coefs_rev(const DevMech<NS>& m, int r, const double* Cb, int nc, double* Yb) {
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      double s = 0.0;
      for (int n = 0; n < nc; ++n) s = fma(Cb[n], m.cpc[r][n][k], s);
      Yb[k] += s;
    }
  }
  // cv = (C0 - rw) + T (C1 + T (C2 + T (C3 + T C4))): dcv/dT.
  __device__ static double dcv_dT(const double C[6], double T) {
    return fma(T, fma(T, fma(T, 4.0 * C[4], 3.0 * C[3]), 2.0 * C[2]), C[1]);
  }
  // c = sqrt((cv + rw) p / (cv rho)), cv = cv(T; C, rw), T given.
  __device__ static void cs_core(const DevMech<NS>& m, const double* Y, double rw, double rho, double T, double p,
                                 double cb, double* Yb, double& rwb, double& rhob, double& Tb, double& pb) {
    const int r = E::range(m, T);
    double C[6];
    E::template coefs<5>(m, Y, r, C);
    const double cv = E::cv_of(C, rw, T);
    const double num = (cv + rw) * p, den = cv * rho;
    const double iden = 1.0 / den;
    const double g = num * iden;
    const double c = sqrt(g);
    if (!(c > 0.0)) return;
    const double gb = cb * 0.5 / c;
    const double numb = gb * iden, denb = -gb * g * iden;
    double cvb = numb * p + denb * rho;
    rwb += numb * p;
    pb += numb * (cv + rw);
    rhob += denb * cv;
    // cv = C0 - rw + T C1 + T^2 C2 + T^3 C3 + T^4 C4
    rwb -= cvb;
    Tb += cvb * dcv_dT(C, T);
    double Cb[5];
    double tp = 1.0;
#pragma unroll
    for (int n = 0; n < 5; ++n) {
      Cb[n] = cvb * tp;
      tp *= T;
    }
    coefs_rev(m, r, Cb, 5, Yb);
  }
  // RPY2Cs with T = p / (rho rw).
  __device__ static void cs_rp(const DevMech<NS>& m, const double* Y, double rw, double rho, double p, double cb,
                               double* Yb, double& rwb, double& rhob, double& pb) {
    const double rr = rho * rw, T = p / rr;  // the forward's T (it selects the range)
    double Tb = 0.0;
    cs_core(m, Y, rw, rho, T, p, cb, Yb, rwb, rhob, Tb, pb);
    // T = p / (rho rw)
    const double q = Tb / rr;
    pb += q;
    rhob -= q * T * rw;  // dT/drho = -T/rho = -T rw / rr
    rwb -= q * T * rho;
  }
  __device__ static void cs_T(const DevMech<NS>& m, const double* Y, double rw, double rho, double T, double p,
                              double cb, double* Yb, double& rwb, double& rhob, double& Tb, double& pb) {
    cs_core(m, Y, rw, rho, T, p, cb, Yb, rwb, rhob, Tb, pb);
  }
  // de/dC_n at T: e = C5 + T (C0 - rw) + T^2 C1/2 + T^3 C2/3 + T^4 C3/4 + T^5 C4/5.
  __device__ static void de_dC(double T, double* w) {
    double tp = T;
#pragma unroll
    for (int n = 0; n < 5; ++n) {
      w[n] = tp / (double)(n + 1);
      tp *= T;
    }
    w[5] = 1.0;
  }
  // RYP2E: e(T, C, rw) with T = p / (rho rw).
  __device__ static void e_rp(const DevMech<NS>& m, const double* Y, double rw, double rho, double p, double eb,
                              double* Yb, double& rwb, double& rhob, double& pb) {
    const double T = p / (rho * rw);
    const int r = E::range(m, T);
    double C[6];
    E::coefs(m, Y, r, C);
    const double cv = E::cv_of(C, rw, T);  // de/dT
    double w[6];
    de_dC(T, w);
    double Cb[6];
#pragma unroll
    for (int n = 0; n < 6; ++n) Cb[n] = eb * w[n];
    coefs_rev(m, r, Cb, 6, Yb);
    rwb -= eb * T;
    const double q = eb * cv / (rho * rw);
    pb += q;
    rhob -= q * T * rw;
    rwb -= q * T * rho;
  }
  // dh_k/dT = cp_k(T) = c0 + T (c1 + T (c2 + T (c3 + T c4))).
  __device__ static void hi_dT(const DevMech<NS>& m, double T, double* dh) {
    const int r = E::range(m, T);
#pragma unroll
    for (int k = 0; k < NS; ++k)
      dh[k] = fma(T, fma(T, fma(T, fma(T, m.cpc[r][4][k], m.cpc[r][3][k]), m.cpc[r][2][k]), m.cpc[r][1][k]),
                  m.cpc[r][0][k]);
  }
  // Implicit function theorem on e(T; C(Y), rw(Y)) = e at the converged T.
  __device__ static void rey2t(const DevMech<NS>& m, const double* Y, double rw, double T, double Tb, double& eb,
                               double* Yb, double& rwb) {
    const int r = E::range(m, T);
    double C[6];
    E::coefs(m, Y, r, C);
    const double cv = E::cv_of(C, rw, T);
    const double q = Tb / cv;  // dT = (de - de/dC dC - de/drw drw) / cv
    eb += q;
    double w[6];
    de_dC(T, w);
    double Cb[6];
#pragma unroll
    for (int n = 0; n < 6; ++n) Cb[n] = -q * w[n];
    coefs_rev(m, r, Cb, 6, Yb);
    rwb += q * T;  // de/drw = -T
  }
};

// ---------------------------------------------------------------------------
// Transport derivatives: out layout rhoD[NS], mu, xi, lambda.
// ---------------------------------------------------------------------------
template <int NS, class TR>
struct TransAdj;

template <int NS>
struct TransAdj<NS, ConstantTransport<NS>> {
  __device__ static void eval(const DevMech<NS>&, double, double, double, const double*, const double*, const double*,
                              double&, double&, double&, double*, double*) {}
};

template <int NS>
struct TransAdj<NS, SimpleTransport<NS>> {
  __device__ static void eval(const DevMech<NS>& m, double T, double rho, double p, const double* Y, const double* X,
                              const double* ob, double& Tb, double& rhob, double& pb, double* Yb, double* Xb) {
    const double L = pc_log(T);
    double smu = 0.0, slam = 0.0;
    double mk[NS], lk[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      mk[k] = pc_exp(horner4(m.visc[k], L));
      const double m2 = mk[k] * mk[k];
      smu = fma(X[k], m2 * m2 * m2, smu);
      lk[k] = pc_exp(0.25 * horner4(m.cond[k], L));
      slam = fma(X[k], lk[k], slam);
    }
    double s[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) s[k] = 0.0;
    const double pr = p * m.inv_pref;
    {
      int q = 0;
#pragma unroll
      for (int k = 0; k < NS; ++k)
#pragma unroll
        for (int j = k + 1; j < NS; ++j, ++q) {
          const double invD = pc_exp(-horner4(m.diff[q], L)) * pr;
          s[k] = fma(fmax(X[j], 1e-15), invD, s[k]);
          s[j] = fma(fmax(X[k], 1e-15), invD, s[j]);
        }
    }
    const double rw = mix_rw<NS>(m, Y);
    double Lb = 0.0, rwb = 0.0;
    double sb[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      sb[k] = 0.0;
      if (s[k] > 0.0) {
        const double is = 1.0 / s[k], iw = 1.0 / m.rW[k];
        const double wrat = rw * iw;
        const double db = ob[k];
        const double t = db * wrat * is;  // d out / d(rho (1 - Y_k))
        rhob += t * (1.0 - Y[k]);
        Yb[k] -= t * rho;
        rwb += db * rho * (1.0 - Y[k]) * iw * is;
        sb[k] = -t * rho * (1.0 - Y[k]) * is;
      }
    }
#pragma unroll
    for (int k = 0; k < NS; ++k) Yb[k] += rwb * m.rW[k];
    double prb = 0.0;
    {
      int q = 0;
#pragma unroll
      for (int k = 0; k < NS; ++k)
#pragma unroll
        for (int j = k + 1; j < NS; ++j, ++q) {
          const double e0 = pc_exp(-horner4(m.diff[q], L));
          const double invD = e0 * pr;
          const double xj = fmax(X[j], 1e-15), xk = fmax(X[k], 1e-15);
          const double invDb = sb[k] * xj + sb[j] * xk;
          if (X[j] >= 1e-15) Xb[j] += sb[k] * invD;
          if (X[k] >= 1e-15) Xb[k] += sb[j] * invD;
          prb += invDb * e0;
          Lb -= invDb * invD * horner4_d(m.diff[q], L);
        }
    }
    pb += prb * m.inv_pref;
    // mu = smu^(1/6), xi = sum X bulk mk, lambda = slam^4
    const double mu = pc_exp(pc_log(smu) * (1.0 / 6.0));
    const double smub = (smu > 0.0) ? ob[NS] * mu * (1.0 / 6.0) / smu : 0.0;
    const double sxib = ob[NS + 1];
    const double slamb = ob[NS + 2] * 4.0 * slam * slam * slam;
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      const double m2 = mk[k] * mk[k];
      const double m5 = m2 * m2 * mk[k];
      Xb[k] += smub * m2 * m2 * m2 + slamb * lk[k] + sxib * m.bulk[k] * mk[k];
      const double mkb = smub * X[k] * 6.0 * m5 + sxib * X[k] * m.bulk[k];
      Lb += mkb * mk[k] * horner4_d(m.visc[k], L);
      Lb += slamb * X[k] * lk[k] * 0.25 * horner4_d(m.cond[k], L);
    }
    Tb += Lb / T;
  }
};

// ---------------------------------------------------------------------------
// Record-cotangent accumulation (FP64 atomics into a record-shaped buffer).
// ---------------------------------------------------------------------------
struct RecBar {
  double* p;
  long long N;
  __device__ __forceinline__ void add(int fld, long long c, double v) const {
    if (v != 0.0) atomicAdd(p + (long long)fld * N + c, v);
  }
};

// ---------------------------------------------------------------------------
// Hyperbolic face flux reverse (two-shock Riemann solver, slopes on or off).
// Fb: cotangent of the face flux times the area (the F of hydro_face).
// ---------------------------------------------------------------------------
template <int NS, class EOS, int d, class Q>
__device__ void hydro_face_rev(const DevBox& b, const DevMech<NS>& m, const DevFlags& f, long long cR, long long st,
                               double A, const double* Fb, const RecBar& rb, Q& q) {
  using RC = Rec<NS>;
  using EA = EosAdj<NS, EOS>;
  const double* rec = b.rec;
  const long long N = b.ncell;
  const long long cL = cR - st, cLL = cL - st, cRR = cR + st;
  auto ld = [&](int fld, long long c) { return __ldg(rec + (long long)fld * N + c); };
  const int fun = RC::U + d;
  const int fut1 = (d == 0) ? RC::V : RC::U;
  const int fut2 = (d == 2) ? RC::V : RC::W;
  // ---- forward (same operation sequence as hydro_face) ----
  const double rLL = ld(RC::RHO, cLL), rL = ld(RC::RHO, cL), rR = ld(RC::RHO, cR), rRR = ld(RC::RHO, cRR);
  const double pLL = ld(RC::P, cLL), pL = ld(RC::P, cL), pR = ld(RC::P, cR), pRR = ld(RC::P, cRR);
  const double uLL = ld(fun, cLL), uL = ld(fun, cL), uR = ld(fun, cR), uRR = ld(fun, cRR);
  const double cLc = ld(RC::C, cL), cRc = ld(RC::C, cR);
  const double t1L = ld(fut1, cL), t1R = ld(fut1, cR), t2L = ld(fut2, cL), t2R = ld(fut2, cR);
  const double ycL = ld(RC::IC, cL), ycR = ld(RC::IC, cR);  // 1 / c (records)
  const bool slopes = f.slopes != 0;
  double t1LL = 0.0, t1RR = 0.0, t2LL = 0.0, t2RR = 0.0;
  const double dpl = pL - pLL, dpc = pR - pL, dpr = pRR - pR;
  double aL1 = 0, bL1 = 0, aL2 = 0, bL2 = 0, aR1 = 0, bR1 = 0, aR2 = 0, bR2 = 0;
  double dqL[4] = {0.0, 0.0, 0.0, 0.0}, dqR[4] = {0.0, 0.0, 0.0, 0.0};
  if (slopes) {
    t1LL = ld(fut1, cLL);
    t1RR = ld(fut1, cRR);
    t2LL = ld(fut2, cLL);
    t2RR = ld(fut2, cRR);
    aL1 = q(0.5 * dpl, cLc, ycL);
    bL1 = 0.5 * rL * (uL - uLL);
    aL2 = q(0.5 * dpc, cLc, ycL);
    bL2 = 0.5 * rL * (uR - uL);
    dqL[0] = mc_limit(aL1 - bL1, aL2 - bL2);
    dqL[1] = mc_limit(aL1 + bL1, aL2 + bL2);
    dqL[2] = mc_limit(t1L - t1LL, t1R - t1L);
    dqL[3] = mc_limit(t2L - t2LL, t2R - t2L);
    aR1 = q(0.5 * dpc, cRc, ycR);
    bR1 = 0.5 * rR * (uR - uL);
    aR2 = q(0.5 * dpr, cRc, ycR);
    bR2 = 0.5 * rR * (uRR - uR);
    dqR[0] = mc_limit(aR1 - bR1, aR2 - bR2);
    dqR[1] = mc_limit(aR1 + bR1, aR2 + bR2);
    dqR[2] = mc_limit(t1R - t1L, t1RR - t1R);
    dqR[3] = mc_limit(t2R - t2L, t2RR - t2R);
  }
  const double unl = uL + 0.5 * ((dqL[1] - dqL[0]) / rL);
  const double pl = pL + 0.5 * (dqL[0] + dqL[1]) * cLc;
  const double ut1l = t1L + 0.5 * dqL[2];
  const double ut2l = t2L + 0.5 * dqL[3];
  const double unr = uR - 0.5 * ((dqR[1] - dqR[0]) / rR);
  const double pr = pR - 0.5 * (dqR[0] + dqR[1]) * cRc;
  const double ut1r = t1R - 0.5 * dqR[2];
  const double ut2r = t2R - 0.5 * dqR[3];
  const double sL = dqL[0] + dqL[1], sR = dqR[0] + dqR[1];
  const double cL2 = cLc * cLc, cR2 = cRc * cRc;
  const double ycL2 = ld(RC::IC2, cL), ycR2 = ld(RC::IC2, cR);  // 1 / c^2 (records)
  double Yl[NS], Yr[NS];
  double rl = 0.0, rr = 0.0;
#pragma unroll
  for (int n = 0; n < NS; ++n) {
    const double yL = ld(RC::Y + n, cL), yR = ld(RC::Y + n, cR);
    double dsL = 0.0, dsR = 0.0;
    if (slopes) {
      const double yLL = ld(RC::Y + n, cLL), yRR = ld(RC::Y + n, cRR);
      const double ryL = rL * yL, ryR = rR * yR;
      dsL = mc_limit(ryL - rLL * yLL - q(yL * dpl, cL2, ycL2), ryR - ryL - q(yL * dpc, cL2, ycL2));
      dsR = mc_limit(ryR - ryL - q(yR * dpc, cR2, ycR2), rRR * yRR - ryR - q(yR * dpr, cR2, ycR2));
    }
    Yl[n] = yL * rL + 0.5 * (dsL + q(yL * sL, cLc, ycL));
    Yr[n] = yR * rR - 0.5 * (dsR + q(yR * sR, cRc, ycR));
    rl += Yl[n];
    rr += Yr[n];
  }
  {
    const double yrl = rcp_q(rl), yrr = rcp_q(rr);
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      Yl[n] = q(Yl[n], rl, yrl);
      Yr[n] = q(Yr[n], rr, yrr);
    }
  }
  const double cavg = 0.5 * (cRc + cLc);
  const double rwl = mix_rw<NS>(m, Yl), rwr = mix_rw<NS>(m, Yr);
  const double cl = EOS::cs_rp(m, Yl, rwl, rl, pl);
  const double cr = EOS::cs_rp(m, Yr, rwr, rr, pr);
  const double wsmall = 2.2250738585072014e-308;
  const double wl = fmax(wsmall, cl * rl);
  const double wr = fmax(wsmall, cr * rr);
  const double ww = wl + wr, yww = rcp_q(ww);
  const double pnum = (wr * pl + wl * pr) + wl * wr * (unl - unr);
  const double pq = q(pnum, ww, yww);
  const double pstar = fmax(wsmall, pq);
  const double ustar0 = q((wl * unl + wr * unr) + (pl - pr), ww, yww);
  const bool mask = ustar0 > 0.0;
  const bool m0 = fabs(ustar0) < kSmallU * 0.5 * (fabs(unl) + fabs(unr)) || ustar0 == 0.0;
  const double ustar = m0 ? 0.0 : ustar0;
  double uo = mask ? unl : unr;
  double po = mask ? pl : pr;
  double rspo[NS];
  double ro = 0.0;
#pragma unroll
  for (int n = 0; n < NS; ++n) {
    const double a = rl * Yl[n], bq = rr * Yr[n];
    rspo[n] = m0 ? 0.5 * (a + bq) : (mask ? a : bq);
    ro += rspo[n];
  }
  uo = m0 ? 0.5 * (unl + unr) : uo;
  po = m0 ? 0.5 * (pl + pr) : po;
  double Yo[NS];
  {
    const double y = rcp_q(ro);
#pragma unroll
    for (int n = 0; n < NS; ++n) Yo[n] = q(rspo[n], ro, y);
  }
  const double rwo = mix_rw<NS>(m, Yo);
  const double co = EOS::cs_rp(m, Yo, rwo, ro, po);
  const double drho = (pstar - po) / (co * co);
  double rsps[NS];
  double rstar = 0.0;
#pragma unroll
  for (int n = 0; n < NS; ++n) {
    rsps[n] = fmax(0.0, rspo[n] + drho * Yo[n]);
    rstar += rsps[n];
  }
  double Ys[NS];
  {
    const double y = rcp_q(rstar);
#pragma unroll
    for (int n = 0; n < NS; ++n) Ys[n] = q(rsps[n], rstar, y);
  }
  const double rws = mix_rw<NS>(m, Ys);
  const double cstar = EOS::cs_rp(m, Ys, rws, rstar, pstar);
  const double sgnm = copysign(1.0, ustar);
  const double spout0 = co - sgnm * uo;
  const double spin0 = cstar - sgnm * ustar;
  const double ushock = 0.5 * (spin0 + spout0);
  const bool mask2 = pstar < po;
  const double spout = mask2 ? spout0 : ushock;
  const double spin = mask2 ? spin0 : ushock;
  const bool tiny = fabs(spout - spin) < PCG_VERY_SMALL_NUM;
  const double scr = tiny ? kSmallNum * cavg : spout - spin;
  const double fracq = (1.0 + (spout + spin) / scr) * 0.5;
  const double frac = fmax(0.0, fmin(1.0, fracq));
  const bool mask3 = ustar > 0.0, uzero = (ustar == 0.0);
  double iv1 = mask3 ? ut1l : ut1r;
  double iv2 = mask3 ? ut2l : ut2r;
  iv1 = uzero ? 0.5 * (ut1l + ut1r) : iv1;
  iv2 = uzero ? 0.5 * (ut2l + ut2r) : iv2;
  const bool mout = spout < 0.0, min_ = spin >= 0.0;
  double iu = frac * ustar + (1.0 - frac) * uo;
  double gdp = frac * pstar + (1.0 - frac) * po;
  iu = mout ? uo : iu;
  gdp = mout ? po : gdp;
  iu = min_ ? ustar : iu;
  gdp = min_ ? pstar : gdp;
  double gq[NS];
  double rgd = 0.0;
#pragma unroll
  for (int n = 0; n < NS; ++n) {
    double g = frac * rsps[n] + (1.0 - frac) * rspo[n];
    g = mout ? rspo[n] : g;
    g = min_ ? rsps[n] : g;
    gq[n] = g;
    rgd += g;
  }
  double Yg[NS];
  {
    const double y = rcp_q(rgd);
#pragma unroll
    for (int n = 0; n < NS; ++n) Yg[n] = q(gq[n], rgd, y);
  }
  const double rwg = mix_rw<NS>(m, Yg);
  const double eg = EOS::e_rp(m, Yg, rwg, rgd, gdp);
  const double regd = rgd * eg;
  const double fl_rho = rgd * iu;
  const double rhoetot = regd + 0.5 * rgd * (iu * iu + iv1 * iv1 + iv2 * iv2);

  // ---- reverse ----
  const double frhob = Fb[URHO] * A, funb = Fb[UMX + d] * A;
  const double fut1b = Fb[(d == 0) ? UMY : UMX] * A, fut2b = Fb[(d == 2) ? UMY : UMZ] * A;
  const double fEb = Fb[UEDEN] * A, feib = Fb[UEINT] * A;
  double iub = 0.0, iv1b = 0.0, iv2b = 0.0, gdpb = 0.0, regdb = 0.0, rgdb = 0.0, flrhob = frhob;
  // fl_ei = iu regd
  iub += feib * regd;
  regdb += feib * iu;
  // fl_E = iu (rhoetot + gdp)
  iub += fEb * (rhoetot + gdp);
  const double rhoetotb = fEb * iu;
  gdpb += fEb * iu;
  // rhoetot = regd + 0.5 rgd K
  regdb += rhoetotb;
  rgdb += rhoetotb * 0.5 * (iu * iu + iv1 * iv1 + iv2 * iv2);
  iub += rhoetotb * rgd * iu;
  iv1b += rhoetotb * rgd * iv1;
  iv2b += rhoetotb * rgd * iv2;
  // fl_ut2 = fl_rho iv2, fl_ut1 = fl_rho iv1, fl_un = fl_rho iu + gdp
  flrhob += fut2b * iv2 + fut1b * iv1 + funb * iu;
  iv2b += fut2b * fl_rho;
  iv1b += fut1b * fl_rho;
  iub += funb * fl_rho;
  gdpb += funb;
  // flY_n = g_n iu
  double gb[NS];
#pragma unroll
  for (int n = 0; n < NS; ++n) {
    const double fyb = Fb[UFS + n] * A;
    gb[n] = fyb * iu;
    iub += fyb * gq[n];
  }
  // fl_rho = rgd iu
  rgdb += flrhob * iu;
  iub += flrhob * rgd;
  // regd = rgd eg
  rgdb += regdb * eg;
  {
    const double egb = regdb * rgd;
    double Ygb[NS];
#pragma unroll
    for (int n = 0; n < NS; ++n) Ygb[n] = 0.0;
    double rwgb = 0.0;
    EA::e_rp(m, Yg, rwg, rgd, gdp, egb, Ygb, rwgb, rgdb, gdpb);
    double dotp = 0.0;
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      Ygb[n] += rwgb * m.rW[n];
      dotp += Ygb[n] * Yg[n];
    }
    // Yg = g / rgd
    const double irgd = 1.0 / rgd;
#pragma unroll
    for (int n = 0; n < NS; ++n) gb[n] += Ygb[n] * irgd;
    rgdb -= dotp * irgd;
  }
  // rgd = sum g
#pragma unroll
  for (int n = 0; n < NS; ++n) gb[n] += rgdb;
  // selections of g, iu, gdp
  double rspsb[NS], rspob[NS];
  double fracb = 0.0, ustarb = 0.0, uob = 0.0, pstarb = 0.0, pob = 0.0;
#pragma unroll
  for (int n = 0; n < NS; ++n) {
    rspsb[n] = 0.0;
    rspob[n] = 0.0;
    if (min_) {
      rspsb[n] += gb[n];
    } else if (mout) {
      rspob[n] += gb[n];
    } else {
      fracb += gb[n] * (rsps[n] - rspo[n]);
      rspsb[n] += gb[n] * frac;
      rspob[n] += gb[n] * (1.0 - frac);
    }
  }
  if (min_) {
    ustarb += iub;
    pstarb += gdpb;
  } else if (mout) {
    uob += iub;
    pob += gdpb;
  } else {
    fracb += iub * (ustar - uo) + gdpb * (pstar - po);
    ustarb += iub * frac;
    uob += iub * (1.0 - frac);
    pstarb += gdpb * frac;
    pob += gdpb * (1.0 - frac);
  }
  // iv1, iv2
  double ut1lb = 0.0, ut1rb = 0.0, ut2lb = 0.0, ut2rb = 0.0;
  if (uzero) {
    ut1lb += 0.5 * iv1b;
    ut1rb += 0.5 * iv1b;
    ut2lb += 0.5 * iv2b;
    ut2rb += 0.5 * iv2b;
  } else if (mask3) {
    ut1lb += iv1b;
    ut2lb += iv2b;
  } else {
    ut1rb += iv1b;
    ut2rb += iv2b;
  }
  // frac = clamp(fracq, 0, 1)
  double spoutb = 0.0, spinb = 0.0, cavgb = 0.0;
  if (fracq >= 0.0 && fracq <= 1.0) {
    const double qb = 0.5 * fracb;  // q = (spout + spin) / scr
    const double q = (spout + spin) / scr;
    spoutb += qb / scr;
    spinb += qb / scr;
    const double scrb = -qb * q / scr;
    if (tiny) {
      cavgb += scrb * kSmallNum;
    } else {
      spoutb += scrb;
      spinb -= scrb;
    }
  }
  double spout0b = 0.0, spin0b = 0.0;
  if (mask2) {
    spout0b += spoutb;
    spin0b += spinb;
  } else {
    const double ushockb = spoutb + spinb;
    spin0b += 0.5 * ushockb;
    spout0b += 0.5 * ushockb;
  }
  double cob = spout0b;
  uob -= sgnm * spout0b;
  const double cstarb = spin0b;
  ustarb -= sgnm * spin0b;
  // cstar = cs(Ys, rws, rstar, pstar)
  {
    double Ysb[NS];
#pragma unroll
    for (int n = 0; n < NS; ++n) Ysb[n] = 0.0;
    double rwsb = 0.0, rstarb = 0.0;
    EA::cs_rp(m, Ys, rws, rstar, pstar, cstarb, Ysb, rwsb, rstarb, pstarb);
    double dotp = 0.0;
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      Ysb[n] += rwsb * m.rW[n];
      dotp += Ysb[n] * Ys[n];
    }
    const double irs = 1.0 / rstar;
    rstarb -= dotp * irs;
#pragma unroll
    for (int n = 0; n < NS; ++n) rspsb[n] += Ysb[n] * irs + rstarb;
  }
  // rsps = max(0, rspo + drho Yo)
  double drhob = 0.0;
  double Yob[NS];
#pragma unroll
  for (int n = 0; n < NS; ++n) {
    Yob[n] = 0.0;
    if (rspo[n] + drho * Yo[n] >= 0.0) {
      rspob[n] += rspsb[n];
      drhob += rspsb[n] * Yo[n];
      Yob[n] += rspsb[n] * drho;
    }
  }
  // drho = (pstar - po) / (co co)
  {
    const double ico = 1.0 / co, ic2 = ico * ico;
    pstarb += drhob * ic2;
    pob -= drhob * ic2;
    cob -= 2.0 * drhob * drho * ico;
  }
  // co = cs(Yo, rwo, ro, po)
  double rob = 0.0;
  {
    double rwob = 0.0;
    EA::cs_rp(m, Yo, rwo, ro, po, cob, Yob, rwob, rob, pob);
    double dotp = 0.0;
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      Yob[n] += rwob * m.rW[n];
      dotp += Yob[n] * Yo[n];
    }
    const double iro = 1.0 / ro;
    rob -= dotp * iro;
#pragma unroll
    for (int n = 0; n < NS; ++n) rspob[n] += Yob[n] * iro + rob;
  }
  // uo, po selections
  double unlb = 0.0, unrb = 0.0, plb = 0.0, prb = 0.0;
  if (m0) {
    unlb += 0.5 * uob;
    unrb += 0.5 * uob;
    plb += 0.5 * pob;
    prb += 0.5 * pob;
  } else if (mask) {
    unlb += uob;
    plb += pob;
  } else {
    unrb += uob;
    prb += pob;
  }
  // rspo selections
  double rlb = 0.0, rrb = 0.0;
  double Ylb[NS], Yrb[NS];
#pragma unroll
  for (int n = 0; n < NS; ++n) {
    Ylb[n] = 0.0;
    Yrb[n] = 0.0;
    const double q = rspob[n];
    if (m0) {
      rlb += 0.5 * q * Yl[n];
      Ylb[n] += 0.5 * q * rl;
      rrb += 0.5 * q * Yr[n];
      Yrb[n] += 0.5 * q * rr;
    } else if (mask) {
      rlb += q * Yl[n];
      Ylb[n] += q * rl;
    } else {
      rrb += q * Yr[n];
      Yrb[n] += q * rr;
    }
  }
  // ustar = m0 ? 0 : ustar0;  ustar0 = ((wl unl + wr unr) + (pl - pr)) / ww
  double wlb = 0.0, wrb = 0.0, wwb = 0.0;
  if (!m0) {
    const double numb = ustarb * yww;
    wwb -= ustarb * ustar0 * yww;
    wlb += numb * unl;
    unlb += numb * wl;
    wrb += numb * unr;
    unrb += numb * wr;
    plb += numb;
    prb -= numb;
  }
  // pstar = max(wsmall, pnum / ww)
  if (pq >= wsmall) {
    const double Pb = pstarb * yww;
    wwb -= pstarb * pq * yww;
    wrb += Pb * pl;
    plb += Pb * wr;
    wlb += Pb * pr;
    prb += Pb * wl;
    const double du = unl - unr;
    wlb += Pb * wr * du;
    wrb += Pb * wl * du;
    unlb += Pb * wl * wr;
    unrb -= Pb * wl * wr;
  }
  wlb += wwb;
  wrb += wwb;
  double clb = 0.0, crb = 0.0;
  if (cl * rl >= wsmall) {
    clb += wlb * rl;
    rlb += wlb * cl;
  }
  if (cr * rr >= wsmall) {
    crb += wrb * rr;
    rrb += wrb * cr;
  }
  // cl = cs(Yl, rwl, rl, pl), cr likewise
  {
    double rwlb = 0.0, rwrb = 0.0;
    EA::cs_rp(m, Yl, rwl, rl, pl, clb, Ylb, rwlb, rlb, plb);
    EA::cs_rp(m, Yr, rwr, rr, pr, crb, Yrb, rwrb, rrb, prb);
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      Ylb[n] += rwlb * m.rW[n];
      Yrb[n] += rwrb * m.rW[n];
    }
  }
  double cLcb = 0.5 * cavgb, cRcb = 0.5 * cavgb;
  // Yl = spl / rl (spl before normalisation is rl Yl)
  double splb[NS], sprb[NS];
  {
    double dl = 0.0, dr = 0.0;
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      dl += Ylb[n] * Yl[n];
      dr += Yrb[n] * Yr[n];
    }
    const double irl = 1.0 / rl, irr = 1.0 / rr;
    rlb -= dl * irl;
    rrb -= dr * irr;
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      splb[n] = Ylb[n] * irl + rlb;
      sprb[n] = Yrb[n] * irr + rrb;
    }
  }
  // face states and slopes
  double dqLb[4] = {0.0, 0.0, 0.0, 0.0}, dqRb[4] = {0.0, 0.0, 0.0, 0.0};
  double rLLb = 0.0, rLb = 0.0, rRb = 0.0, rRRb = 0.0, dplb = 0.0, dpcb = 0.0, dprb = 0.0;
  double cL2b = 0.0, cR2b = 0.0, sLb = 0.0, sRb = 0.0;
#pragma unroll
  for (int n = 0; n < NS; ++n) {
    const double yL = ld(RC::Y + n, cL), yR = ld(RC::Y + n, cR);
    double yLb = 0.0, yRb = 0.0;
    // spl = yL rL + 0.5 (dsL + yL sL / cLc)
    const double sb = splb[n];
    yLb += sb * rL + 0.5 * sb * sL * ycL;
    rLb += sb * yL;
    const double dsLb = 0.5 * sb;
    sLb += 0.5 * sb * yL * ycL;
    cLcb -= 0.5 * sb * yL * sL * ycL2;
    // spr = yR rR - 0.5 (dsR + yR sR / cRc)
    const double sr = sprb[n];
    yRb += sr * rR - 0.5 * sr * sR * ycR;
    rRb += sr * yR;
    const double dsRb = -0.5 * sr;
    sRb -= 0.5 * sr * yR * ycR;
    cRcb += 0.5 * sr * yR * sR * ycR2;
    if (slopes) {
      const double yLL = ld(RC::Y + n, cLL), yRR = ld(RC::Y + n, cRR);
      const double ryL = rL * yL, ryR = rR * yR;
      double ryLb = 0.0, ryRb = 0.0, yLLb = 0.0, yRRb = 0.0;
      {
        const double a = ryL - rLL * yLL - q(yL * dpl, cL2, ycL2);
        const double bq = ryR - ryL - q(yL * dpc, cL2, ycL2);
        double ab = 0.0, bb = 0.0;
        mc_limit_rev(a, bq, dsLb, ab, bb);
        ryLb += ab - bb;
        ryRb += bb;
        rLLb -= ab * yLL;
        yLLb -= ab * rLL;
        yLb -= (ab * dpl + bb * dpc) * ycL2;
        dplb -= ab * yL * ycL2;
        dpcb -= bb * yL * ycL2;
        cL2b += (ab * yL * dpl + bb * yL * dpc) * ycL2 * ycL2;
      }
      {
        const double a = ryR - ryL - q(yR * dpc, cR2, ycR2);
        const double bq = rRR * yRR - ryR - q(yR * dpr, cR2, ycR2);
        double ab = 0.0, bb = 0.0;
        mc_limit_rev(a, bq, dsRb, ab, bb);
        ryRb += ab - bb;
        ryLb -= ab;
        yRb -= (ab * dpc + bb * dpr) * ycR2;
        dpcb -= ab * yR * ycR2;
        dprb -= bb * yR * ycR2;
        cR2b += (ab * yR * dpc + bb * yR * dpr) * ycR2 * ycR2;
        rRRb += bb * yRR;
        yRRb += bb * rRR;
      }
      rLb += ryLb * yL;
      yLb += ryLb * rL;
      rRb += ryRb * yR;
      yRb += ryRb * rR;
      rb.add(RC::Y + n, cLL, yLLb);
      rb.add(RC::Y + n, cRR, yRRb);
    }
    rb.add(RC::Y + n, cL, yLb);
    rb.add(RC::Y + n, cR, yRb);
  }
  cLcb += 2.0 * cL2b * cLc;
  cRcb += 2.0 * cR2b * cRc;
  dqLb[0] += sLb;
  dqLb[1] += sLb;
  dqRb[0] += sRb;
  dqRb[1] += sRb;
  double uLb = 0.0, uRb = 0.0, pLb = 0.0, pRb = 0.0, t1Lb = 0.0, t1Rb = 0.0, t2Lb = 0.0, t2Rb = 0.0;
  // unl = uL + 0.5 (dqL1 - dqL0) / rL
  const double irL = 1.0 / rL, irR = 1.0 / rR;
  uLb += unlb;
  dqLb[1] += 0.5 * unlb * irL;
  dqLb[0] -= 0.5 * unlb * irL;
  rLb -= unlb * 0.5 * (dqL[1] - dqL[0]) * irL * irL;
  // pl = pL + 0.5 (dqL0 + dqL1) cLc
  pLb += plb;
  dqLb[0] += 0.5 * plb * cLc;
  dqLb[1] += 0.5 * plb * cLc;
  cLcb += plb * 0.5 * (dqL[0] + dqL[1]);
  t1Lb += ut1lb;
  dqLb[2] += 0.5 * ut1lb;
  t2Lb += ut2lb;
  dqLb[3] += 0.5 * ut2lb;
  // unr = uR - 0.5 (dqR1 - dqR0) / rR
  uRb += unrb;
  dqRb[1] -= 0.5 * unrb * irR;
  dqRb[0] += 0.5 * unrb * irR;
  rRb += unrb * 0.5 * (dqR[1] - dqR[0]) * irR * irR;
  pRb += prb;
  dqRb[0] -= 0.5 * prb * cRc;
  dqRb[1] -= 0.5 * prb * cRc;
  cRcb -= prb * 0.5 * (dqR[0] + dqR[1]);
  t1Rb += ut1rb;
  dqRb[2] -= 0.5 * ut1rb;
  t2Rb += ut2rb;
  dqRb[3] -= 0.5 * ut2rb;
  double uLLb = 0.0, uRRb = 0.0;
  if (slopes) {
    double aL1b = 0, bL1b = 0, aL2b = 0, bL2b = 0, aR1b = 0, bR1b = 0, aR2b = 0, bR2b = 0;
    double t1LLb = 0, t1RRb = 0, t2LLb = 0, t2RRb = 0;
    {
      double xb = 0.0, yb = 0.0;
      mc_limit_rev(aL1 - bL1, aL2 - bL2, dqLb[0], xb, yb);
      aL1b += xb;
      bL1b -= xb;
      aL2b += yb;
      bL2b -= yb;
      xb = yb = 0.0;
      mc_limit_rev(aL1 + bL1, aL2 + bL2, dqLb[1], xb, yb);
      aL1b += xb;
      bL1b += xb;
      aL2b += yb;
      bL2b += yb;
      xb = yb = 0.0;
      mc_limit_rev(t1L - t1LL, t1R - t1L, dqLb[2], xb, yb);
      t1Lb += xb - yb;
      t1LLb -= xb;
      t1Rb += yb;
      xb = yb = 0.0;
      mc_limit_rev(t2L - t2LL, t2R - t2L, dqLb[3], xb, yb);
      t2Lb += xb - yb;
      t2LLb -= xb;
      t2Rb += yb;
      xb = yb = 0.0;
      mc_limit_rev(aR1 - bR1, aR2 - bR2, dqRb[0], xb, yb);
      aR1b += xb;
      bR1b -= xb;
      aR2b += yb;
      bR2b -= yb;
      xb = yb = 0.0;
      mc_limit_rev(aR1 + bR1, aR2 + bR2, dqRb[1], xb, yb);
      aR1b += xb;
      bR1b += xb;
      aR2b += yb;
      bR2b += yb;
      xb = yb = 0.0;
      mc_limit_rev(t1R - t1L, t1RR - t1R, dqRb[2], xb, yb);
      t1Rb += xb - yb;
      t1Lb -= xb;
      t1RRb += yb;
      xb = yb = 0.0;
      mc_limit_rev(t2R - t2L, t2RR - t2R, dqRb[3], xb, yb);
      t2Rb += xb - yb;
      t2Lb -= xb;
      t2RRb += yb;
    }
    // a = 0.5 dp / c, b = 0.5 r du
    dplb += 0.5 * aL1b * ycL;
    cLcb -= aL1b * aL1 * ycL;
    dpcb += 0.5 * aL2b * ycL;
    cLcb -= aL2b * aL2 * ycL;
    rLb += 0.5 * bL1b * (uL - uLL) + 0.5 * bL2b * (uR - uL);
    uLb += 0.5 * bL1b * rL - 0.5 * bL2b * rL;
    uLLb -= 0.5 * bL1b * rL;
    uRb += 0.5 * bL2b * rL;
    dpcb += 0.5 * aR1b * ycR;
    cRcb -= aR1b * aR1 * ycR;
    dprb += 0.5 * aR2b * ycR;
    cRcb -= aR2b * aR2 * ycR;
    rRb += 0.5 * bR1b * (uR - uL) + 0.5 * bR2b * (uRR - uR);
    uRb += 0.5 * bR1b * rR - 0.5 * bR2b * rR;
    uLb -= 0.5 * bR1b * rR;
    uRRb += 0.5 * bR2b * rR;
    rb.add(fut1, cLL, t1LLb);
    rb.add(fut1, cRR, t1RRb);
    rb.add(fut2, cLL, t2LLb);
    rb.add(fut2, cRR, t2RRb);
  }
  // dp differences
  pLb += dplb - dpcb;
  pRb += dpcb - dprb;
  const double pLLb = -dplb, pRRb = dprb;
  rb.add(RC::RHO, cLL, rLLb);
  rb.add(RC::RHO, cL, rLb);
  rb.add(RC::RHO, cR, rRb);
  rb.add(RC::RHO, cRR, rRRb);
  rb.add(RC::P, cLL, pLLb);
  rb.add(RC::P, cL, pLb);
  rb.add(RC::P, cR, pRb);
  rb.add(RC::P, cRR, pRRb);
  rb.add(fun, cLL, uLLb);
  rb.add(fun, cL, uLb);
  rb.add(fun, cR, uRb);
  rb.add(fun, cRR, uRRb);
  rb.add(RC::C, cL, cLcb);
  rb.add(RC::C, cR, cRcb);
  rb.add(fut1, cL, t1Lb);
  rb.add(fut1, cR, t1Rb);
  rb.add(fut2, cL, t2Lb);
  rb.add(fut2, cR, t2Rb);
}

// ---------------------------------------------------------------------------
// Diffusion face flux reverse (pc_diffusion_flux + SpeciesEnergyFlux).
// ---------------------------------------------------------------------------
template <int NS, int d>
__device__ void diffusion_face_rev(const DevBox& b, const DevFlags& f, const Geo& g, long long cR,
                                   const long long stv[3], const double* Fb, const RecBar& rb) {
  using RC = Rec<NS>;
  const double* rec = b.rec;
  const long long N = b.ncell;
  auto ld = [&](int fld, long long c) { return __ldg(rec + (long long)fld * N + c); };
  const long long cL = cR - stv[d];
  const bool harm = f.harmonic != 0;
  const double muR = ld(RC::MU, cR), muL = ld(RC::MU, cL);
  const double xiR = ld(RC::XI, cR), xiL = ld(RC::XI, cL);
  const double lamR = ld(RC::LAM, cR), lamL = ld(RC::LAM, cL);
  const double mu = face_coef(muR, muL, harm);
  const double xi = face_coef(xiR, xiL, harm);
  const double lam = face_coef(lamR, lamL, harm);
  double grad[3][3];
  const double uR[3] = {ld(RC::U, cR), ld(RC::V, cR), ld(RC::W, cR)};
  const double uL[3] = {ld(RC::U, cL), ld(RC::V, cL), ld(RC::W, cL)};
#pragma unroll
  for (int c = 0; c < 3; ++c) grad[c][d] = g.dxinv[d] * (uR[c] - uL[c]);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (a == d) continue;
    const long long sa = stv[a];
    const double q4 = 0.25 * g.dxinv[a];
    const int ca = RC::U + a, cd = RC::U + d;
    grad[a][a] = (ld(ca, cR + sa) + ld(ca, cL + sa) - ld(ca, cR - sa) - ld(ca, cL - sa)) * q4;
    grad[d][a] = (ld(cd, cR + sa) + ld(cd, cL + sa) - ld(cd, cR - sa) - ld(cd, cL - sa)) * q4;
  }
  const double divu = grad[0][0] + grad[1][1] + grad[2][2];
  double tau[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (a == d)
      tau[a] = mu * (2.0 * grad[d][d] - 2.0 / 3.0 * divu) + xi * divu;
    else
      tau[a] = mu * (grad[d][a] + grad[a][d]);
  }
  const double TR = ld(RC::T, cR), TL = ld(RC::T, cL);
  const double dTdd = g.dxinv[d] * (TR - TL);
  const double A = g.area[d];
  const bool spec = f.diffuse_spec != 0;
  const bool ener = (f.diffuse_temp != 0) || (f.diffuse_enth != 0);
  const double fEb = ener ? Fb[UEDEN] * A : 0.0;
  double taub[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) taub[a] = f.diffuse_vel ? -Fb[UMX + a] * A : 0.0;
  if (NS > 1 || spec || ener) {
    const double pR = ld(RC::P, cR), pL = ld(RC::P, cL);
    const double dpdx = g.dxinv[d] * (pR - pL);
    const double pm = 0.5 * (pR + pL);
    const double dlnp = dpdx / pm;
    double Vd[NS], Yf[NS], hf[NS], D[NS], inner[NS], Xf[NS];
    double Vc = 0.0;
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      const double x1 = ld(RC::X + n, cR), x2 = ld(RC::X + n, cL);
      const double y1 = ld(RC::Y + n, cR), y2 = ld(RC::Y + n, cL);
      Xf[n] = 0.5 * (x1 + x2);
      Yf[n] = 0.5 * (y1 + y2);
      hf[n] = 0.5 * (ld(RC::H + n, cR) + ld(RC::H + n, cL));
      const double dXdx = g.dxinv[d] * (x1 - x2);
      D[n] = face_coef(ld(RC::D + n, cR), ld(RC::D + n, cL), harm);
      inner[n] = dXdx + (Xf[n] - Yf[n]) * dlnp;
      Vd[n] = -D[n] * inner[n];
      Vc += Vd[n];
    }
    double Vcb = 0.0, dlnpb = 0.0;
    double Vdb[NS], Yfb[NS], hfb[NS];
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      const double vb = spec ? Fb[UFS + n] * A : 0.0;
      // fE -= Yf hf Vc;  v = Vd - Yf Vc
      Yfb[n] = -fEb * hf[n] * Vc - vb * Vc;
      hfb[n] = -fEb * Yf[n] * Vc;
      Vcb -= fEb * Yf[n] * hf[n] + vb * Yf[n];
      Vdb[n] = vb;
    }
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      // fE += Vd hf;  Vc += Vd
      Vdb[n] += fEb * hf[n] + Vcb;
      hfb[n] += fEb * Vd[n];
      // Vd = -D inner
      const double Db = -Vdb[n] * inner[n];
      const double ib = -Vdb[n] * D[n];
      const double Xfb = ib * dlnp;
      Yfb[n] -= ib * dlnp;
      dlnpb += ib * (Xf[n] - Yf[n]);
      const double dXb = ib * g.dxinv[d];
      double DRb = 0.0, DLb = 0.0;
      face_coef_rev(ld(RC::D + n, cR), ld(RC::D + n, cL), harm, Db, DRb, DLb);
      rb.add(RC::D + n, cR, DRb);
      rb.add(RC::D + n, cL, DLb);
      rb.add(RC::X + n, cR, 0.5 * Xfb + dXb);
      rb.add(RC::X + n, cL, 0.5 * Xfb - dXb);
      rb.add(RC::Y + n, cR, 0.5 * Yfb[n]);
      rb.add(RC::Y + n, cL, 0.5 * Yfb[n]);
      rb.add(RC::H + n, cR, 0.5 * hfb[n]);
      rb.add(RC::H + n, cL, 0.5 * hfb[n]);
    }
    // dlnp = dpdx / pm
    const double ipm = 1.0 / pm;
    const double dpdxb = dlnpb * ipm;
    const double pmb = -dlnpb * dlnp * ipm;
    rb.add(RC::P, cR, g.dxinv[d] * dpdxb + 0.5 * pmb);
    rb.add(RC::P, cL, -g.dxinv[d] * dpdxb + 0.5 * pmb);
  }
  // fE = 0.5 (-sum tau_c (uR_c + uL_c)) - lam dTdd
  double uRb[3], uLb[3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    taub[c] -= 0.5 * fEb * (uR[c] + uL[c]);
    uRb[c] = -0.5 * fEb * tau[c];
    uLb[c] = -0.5 * fEb * tau[c];
  }
  const double lamb = -fEb * dTdd;
  const double dTb = -fEb * lam * g.dxinv[d];
  rb.add(RC::T, cR, dTb);
  rb.add(RC::T, cL, -dTb);
  // tau
  double mub = 0.0, xib = 0.0, divub = 0.0;
  double gradb[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (a == d) {
      mub += taub[a] * (2.0 * grad[d][d] - 2.0 / 3.0 * divu);
      gradb[d][d] += taub[a] * mu * 2.0;
      divub += taub[a] * (-2.0 / 3.0 * mu + xi);
      xib += taub[a] * divu;
    } else {
      mub += taub[a] * (grad[d][a] + grad[a][d]);
      gradb[d][a] += taub[a] * mu;
      gradb[a][d] += taub[a] * mu;
    }
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) gradb[a][a] += divub;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    uRb[c] += g.dxinv[d] * gradb[c][d];
    uLb[c] -= g.dxinv[d] * gradb[c][d];
  }
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (a == d) continue;
    const long long sa = stv[a];
    const double q4 = 0.25 * g.dxinv[a];
    const int ca = RC::U + a, cd = RC::U + d;
    const double ga = gradb[a][a] * q4, gd = gradb[d][a] * q4;
    rb.add(ca, cR + sa, ga);
    rb.add(ca, cL + sa, ga);
    rb.add(ca, cR - sa, -ga);
    rb.add(ca, cL - sa, -ga);
    rb.add(cd, cR + sa, gd);
    rb.add(cd, cL + sa, gd);
    rb.add(cd, cR - sa, -gd);
    rb.add(cd, cL - sa, -gd);
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    rb.add(RC::U + c, cR, uRb[c]);
    rb.add(RC::U + c, cL, uLb[c]);
  }
  double ab = 0.0, bb = 0.0;
  face_coef_rev(muR, muL, harm, mub, ab, bb);
  rb.add(RC::MU, cR, ab);
  rb.add(RC::MU, cL, bb);
  ab = bb = 0.0;
  face_coef_rev(xiR, xiL, harm, xib, ab, bb);
  rb.add(RC::XI, cR, ab);
  rb.add(RC::XI, cL, bb);
  ab = bb = 0.0;
  face_coef_rev(lamR, lamL, harm, lamb, ab, bb);
  rb.add(RC::LAM, cR, ab);
  rb.add(RC::LAM, cL, bb);
}

// Cotangent arrays of one box: rbar (RHS cotangent, valid region) in,
// ubar (state cotangent, grow(valid, 2)) out.
struct AdjBox {
  const double* rbar;
  long long rj, rk, rn;
  int rb[3];
  int pad0;
  double* ubar;
  long long uj, uk, un;
  int ub[3];
  int pad1;
};

// ---------------------------------------------------------------------------
// Pass 2 of the adjoint: one thread per face.  items = (box, direction,
// first face of a 128-face chunk); the faces of direction d of a box are
// those with the high-side cell in [lo_d, hi_d + 1] and the transverse cells
// in the valid box.
// ---------------------------------------------------------------------------
constexpr int kAdjThreads = 128;

template <int NS, class EOS, int d, class Q>
__device__ __forceinline__ void face_adjoint_dir(const DevBox& b, const AdjBox& a, const DevMech<NS>& m,
                                                 const DevFlags& f, const Geo& g, long long fi, const RecBar& rb,
                                                 Q& q) {
  constexpr int NVAR = 7 + NS;
  const int nf0 = b.hi[0] - b.lo[0] + 1 + (d == 0), nf1 = b.hi[1] - b.lo[1] + 1 + (d == 1);
  const int nf2 = b.hi[2] - b.lo[2] + 1 + (d == 2);
  if (fi >= (long long)nf0 * nf1 * nf2) return;
  const int i = b.lo[0] + (int)(fi % nf0), j = b.lo[1] + (int)((fi / nf0) % nf1),
            k = b.lo[2] + (int)(fi / ((long long)nf0 * nf1));
  // Fbar = (rbar_R - rbar_L) / V with rbar = 0 outside the valid box.
  const int iv[3] = {i, j, k};
  const bool Rin = iv[d] <= b.hi[d], Lin = iv[d] - 1 >= b.lo[d];
  double Fb[NVAR];
  const double* pR = a.rbar + (i - a.rb[0]) + (long long)(j - a.rb[1]) * a.rj + (long long)(k - a.rb[2]) * a.rk;
  const long long sd = (d == 0) ? 1 : (d == 1) ? a.rj : a.rk;
  const double iv_vol = 1.0 / g.vol;
  bool any = false;
#pragma unroll
  for (int n = 0; n < NVAR; ++n) {
    const double r1 = Rin ? __ldg(pR + n * a.rn) : 0.0;
    const double r0 = Lin ? __ldg(pR - sd + n * a.rn) : 0.0;
    Fb[n] = (r1 - r0) * iv_vol;
    any |= Fb[n] != 0.0;
  }
  if (!any) return;
  const long long stv[3] = {1, b.n2[0], (long long)b.n2[0] * b.n2[1]};
  const long long cR = (i - b.g2lo[0]) + (j - b.g2lo[1]) * stv[1] + (k - b.g2lo[2]) * stv[2];
  if (f.do_hydro) hydro_face_rev<NS, EOS, d>(b, m, f, cR, stv[d], g.area[d], Fb, rb, q);
  const bool diff = f.diffuse_vel || f.diffuse_temp || f.diffuse_spec || f.diffuse_enth;
  if (diff) diffusion_face_rev<NS, d>(b, f, g, cR, stv, Fb, rb);
}

// kExact = false: quotients by div_fast, lanes that need a real division
// counted in counters[kCounterSlowAdj]; kExact = true: the exact twin, which
// returns at once unless that count is nonzero and then (after the record
// cotangents have been cleared again, zero_recbar_if_slow) accumulates them
// anew with IEEE quotients.
template <int NS, class EOS, bool kExact = false>
__global__ void __launch_bounds__(kAdjThreads)
    face_adjoint_kernel(const DevBox* __restrict__ boxes, const AdjBox* __restrict__ adj,
                        const int4* __restrict__ items, double* __restrict__ recbar_base,
                        const long long* __restrict__ recbar_off, const __grid_constant__ DevMech<NS> m,
                        const DevFlags f, const Geo g, unsigned long long* __restrict__ counters) {
  if (kExact && __ldcg(&counters[kCounterSlowAdj]) == 0ull) return;
  const int4 it = items[blockIdx.x];
  const DevBox& b = boxes[it.x];
  const RecBar rb{recbar_base + recbar_off[it.x], b.ncell};
  const long long fi = (long long)it.z * kAdjThreads + threadIdx.x;
  Quot<kExact> quo;
  if (it.y == 0)
    face_adjoint_dir<NS, EOS, 0>(b, adj[it.x], m, f, g, fi, rb, quo);
  else if (it.y == 1)
    face_adjoint_dir<NS, EOS, 1>(b, adj[it.x], m, f, g, fi, rb, quo);
  else
    face_adjoint_dir<NS, EOS, 2>(b, adj[it.x], m, f, g, fi, rb, quo);
  if (!kExact) warp_count(&counters[kCounterSlowAdj], quo.slow);
}

// Clears the record cotangents before the exact twin of the face adjoint,
// when the fast pass counted a lane that needs a real division.
static __global__ void zero_recbar_if_slow(double* __restrict__ recbar, long long n,
                                    const unsigned long long* __restrict__ counters) {
  if (__ldcg(&counters[kCounterSlowAdj]) == 0ull) return;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    recbar[i] = 0.0;
}

// ---------------------------------------------------------------------------
// Pass 3 of the adjoint: record cotangents -> state cotangents, one thread
// per cell of grow(valid, 2) (same items as the forward pass 1).
// ---------------------------------------------------------------------------
template <int NS, class EOS, class TR>
__global__ void __launch_bounds__(kCellThreads)
    cell_adjoint_kernel(const DevBox* __restrict__ boxes, const AdjBox* __restrict__ adj,
                        const int2* __restrict__ items, const double* __restrict__ recbar_base,
                        const long long* __restrict__ recbar_off, const __grid_constant__ DevMech<NS> m,
                        const DevFlags f) {
  using RC = Rec<NS>;
  using EA = EosAdj<NS, EOS>;
  constexpr int NVAR = 7 + NS;
  const int2 it = items[blockIdx.x];
  const DevBox& b = boxes[it.x];
  const AdjBox& a = adj[it.x];
  const long long c = (long long)it.y + threadIdx.x;
  if (c >= b.ncell) return;
  const double* rbar = recbar_base + recbar_off[it.x] + c;
  const long long N = b.ncell;
  auto rbr = [&](int fld) { return rbar[(long long)fld * N]; };
  const int nx = b.n2[0], ny = b.n2[1];
  const int i = b.g2lo[0] + (int)(c % nx);
  const int j = b.g2lo[1] + (int)((c / nx) % ny);
  const int k = b.g2lo[2] + (int)(c / ((long long)nx * ny));
  const double* s = b.S + (i - b.sb[0]) + (long long)(j - b.sb[1]) * b.sj + (long long)(k - b.sb[2]) * b.sk;
  const long long sn = b.sn;
  // ---- forward (pass 1) ----
  const double rho = __ldg(s + URHO * sn);
  const double rhoinv = 1.0 / rho;
  const double mx = __ldg(s + UMX * sn), my = __ldg(s + UMY * sn), mz = __ldg(s + UMZ * sn);
  const double vx = mx * rhoinv, vy = my * rhoinv, vz = mz * rhoinv;
  const double E = __ldg(s + UEDEN * sn);
  const double kineng = 0.5 * rho * (vx * vx + vy * vy + vz * vz);
  const double e = (E - kineng) * rhoinv;
  double Y[NS];
  bool clip[NS];
#pragma unroll
  for (int n = 0; n < NS; ++n) {
    double y = __ldg(s + (UFS + n) * sn) / rho;
    clip[n] = -1e-4 * 2.220446049250313e-16 < y && y < 1e-4 * 2.220446049250313e-16;
    if (clip[n]) y = 0.0;
    Y[n] = y;
  }
  const double rw = mix_rw<NS>(m, Y);
  bool ok = true;
  const double T = EOS::rey2t(m, Y, rw, e, __ldg(s + UTEMP * sn), f.newton_maxit, ok);
  const double p = rho * rw * T;
  const bool inner = i >= b.lo[0] - 1 && i <= b.hi[0] + 1 && j >= b.lo[1] - 1 && j <= b.hi[1] + 1 &&
                     k >= b.lo[2] - 1 && k <= b.hi[2] + 1;
  // ---- reverse ----
  double Yb[NS];
#pragma unroll
  for (int n = 0; n < NS; ++n) Yb[n] = rbr(RC::Y + n);
  double rhob = rbr(RC::RHO), pb = rbr(RC::P), Tb = 0.0, rwb = 0.0;
  double vxb = rbr(RC::U), vyb = rbr(RC::V), vzb = rbr(RC::W);
  if (inner) {
    Tb += rbr(RC::T);
    double X[NS], Xb[NS];
    y2x(m, Y, rw, X);
#pragma unroll
    for (int n = 0; n < NS; ++n) Xb[n] = rbr(RC::X + n);
    // h = hi(T)
    {
      double dh[NS];
      EA::hi_dT(m, T, dh);
#pragma unroll
      for (int n = 0; n < NS; ++n) Tb += rbr(RC::H + n) * dh[n];
    }
    // transport
    {
      double ob[NS + 3];
#pragma unroll
      for (int n = 0; n < NS + 3; ++n) ob[n] = rbr(RC::D + n);
      TransAdj<NS, TR>::eval(m, T, rho, p, Y, X, ob, Tb, rhob, pb, Yb, Xb);
    }
    // X_n = Y_n rW_n / rw
    const double irw = 1.0 / rw;
    double dotp = 0.0;
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      Yb[n] += Xb[n] * m.rW[n] * irw;
      dotp += Xb[n] * X[n];
    }
    rwb -= dotp * irw;
  }
  // c = cs_T(Y, rw, rho, T, p)
  EA::cs_T(m, Y, rw, rho, T, p, rbr(RC::C), Yb, rwb, rhob, Tb, pb);
  // p = rho rw T
  rhob += pb * rw * T;
  rwb += pb * rho * T;
  Tb += pb * rho * rw;
  // T = T(e, Y) by the implicit-function theorem
  double eb = 0.0;
  EA::rey2t(m, Y, rw, T, Tb, eb, Yb, rwb);
#pragma unroll
  for (int n = 0; n < NS; ++n) Yb[n] += rwb * m.rW[n];
  // Y_n = rhoY_n / rho
  double ub[NVAR];
#pragma unroll
  for (int n = 0; n < NVAR; ++n) ub[n] = 0.0;
#pragma unroll
  for (int n = 0; n < NS; ++n) {
    if (!clip[n]) {
      ub[UFS + n] = Yb[n] * rhoinv;
      rhob -= Yb[n] * Y[n] * rhoinv;
    }
  }
  // e = (E - kineng) rhoinv
  ub[UEDEN] = eb * rhoinv;
  const double kb = -eb * rhoinv;
  double rinvb = eb * (E - kineng);
  // kineng = 0.5 rho |v|^2
  rhob += kb * 0.5 * (vx * vx + vy * vy + vz * vz);
  vxb += kb * rho * vx;
  vyb += kb * rho * vy;
  vzb += kb * rho * vz;
  // v = m rhoinv
  ub[UMX] = vxb * rhoinv;
  ub[UMY] = vyb * rhoinv;
  ub[UMZ] = vzb * rhoinv;
  rinvb += vxb * mx + vyb * my + vzb * mz;
  rhob -= rinvb * rhoinv * rhoinv;
  ub[URHO] = rhob;
  double* o = a.ubar + (i - a.ub[0]) + (long long)(j - a.ub[1]) * a.uj + (long long)(k - a.ub[2]) * a.uk;
#pragma unroll
  for (int n = 0; n < NVAR; ++n) o[n * a.un] = ub[n];
}

}  // namespace pcg
