// pc_oracle.hpp — ORACLE (test infrastructure, never shipped or measured).
//
// CPU restatement of PeleC's method-of-lines right-hand side on one regular
// (non-EB) box, PeleC::getMOLSrcTerm (Source/Diffusion.cpp:4-681).  It keeps
// the reference's pass structure and floating-point operation order:
//   ctoprim over gbox=grow(vbox,4)                 Diffusion.cpp:132-145
//   transport coefficients over gbox               Diffusion.cpp:180-220
//   diffusion fluxes on eboxes=surroundingNodes(cbox,d), cbox=grow(vbox,3)
//                                                  Diffusion.cpp:222-275
//   zeroing of switched-off diffusion components   Diffusion.cpp:321-341
//   hyperbolic fluxes (slopes + Riemann), +=       Diffusion.cpp:344-369
//   flux divergence over cbox, copy on vbox        Diffusion.cpp:530-541,672
// Only tests/, the package smoke check and bench.py's CPU-baseline leg use
// this code, as the checker and as the timed CPU baseline.
//
// Parity status: PINNED for everything that lives in the reference tree.
// oracle/ref_build.py compiles the reference's own hot-path sources where
// they lie (MOL.cpp, Riemann.H, Diffterm.H, Utilities.H, TransCoeff.H,
// Timestep.H) against stand-ins for the absent AMReX and PelePhysics
// headers, and tests/test_ref_pinned.py checks that this restatement gives
// the same bits on every output (full C1 and C2 boxes, the flag matrix,
// face fluxes, single faces and cells, computeTemp, estTimeStep).
// UNPINNED: what PelePhysics supplies — the EOS (GammaLaw, NASA-7 ideal
// mixture) and the transport (Constant, mixture-averaged "Simple") are
// restated from their published physics, and the species tables are the
// caller's (pc_mechanism); the reference build runs these same restatements.
//
// The transport's exp and log are pc_exp.h's (pelec_gb300/csrc), the
// table-driven functions the kernels call too, instead of the host libm's:
// within one ulp of the correctly rounded values (tests/test_oracle.py), and
// the same bits on every host and on the GPU.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#include "pc_exp.h"
#include "pelec_mol.h"

namespace orc {

// Universal gas constant, erg/(mol K) (CODATA 2018 value in cgs units).
constexpr double RU = 8.31446261815324e7;

// Source/IndexDefines.H:6-42,60,69-78 (NUM_ADV = NUM_AUX = NUM_LIN = 0).
enum { URHO = 0, UMX = 1, UMY = 2, UMZ = 3, UEDEN = 4, UEINT = 5, UTEMP = 6, UFS = 7 };
enum { QRHO = 0, QU = 1, QV = 2, QW = 3, QGAME = 4, QPRES = 5, QREINT = 6, QTEMP = 7, QFS = 8 };
enum { QGAMC = 0, QC = 1, QCSML = 2, QDPDR = 3, QDPDE = 4, QRSPEC = 5, NQAUX = 6 };

// Source/Constants.H:10-24.
inline double smallu() { return 1.0e-12; }
inline double small_num() { return 1.0e-8; }
inline double very_small_num() { return std::numeric_limits<double>::epsilon() * 1e-100; }

struct Box {
  int lo[3], hi[3];
  long long npts() const {
    long long n = 1;
    for (int d = 0; d < 3; ++d) n *= (hi[d] - lo[d] + 1);
    return n;
  }
};
inline Box grow(Box b, int n) {
  for (int d = 0; d < 3; ++d) { b.lo[d] -= n; b.hi[d] += n; }
  return b;
}
inline Box grow_dir(Box b, int dir, int n) { b.lo[dir] -= n; b.hi[dir] += n; return b; }
inline Box surrounding_nodes(Box b, int dir) { b.hi[dir] += 1; return b; }

// Array4-style view: i fastest, component slowest.
template <class R>
struct Arr {
  R* p = nullptr;
  long long js = 0, ks = 0, ns = 0;
  int b[3] = {0, 0, 0};
  R& operator()(int i, int j, int k, int n = 0) const {
    return p[(i - b[0]) + (long long)(j - b[1]) * js + (long long)(k - b[2]) * ks + (long long)n * ns];
  }
};

// Owning FArrayBox-style container.
template <class R>
struct Fab {
  Box bx{};
  int nc = 0;
  std::vector<R> v;
  Fab(const Box& b, int ncomp) : bx(b), nc(ncomp), v((size_t)b.npts() * ncomp, R(0)) {}
  Arr<R> arr() {
    Arr<R> a;
    a.p = v.data();
    a.js = bx.hi[0] - bx.lo[0] + 1;
    a.ks = a.js * (bx.hi[1] - bx.lo[1] + 1);
    a.ns = a.ks * (bx.hi[2] - bx.lo[2] + 1);
    for (int d = 0; d < 3; ++d) a.b[d] = bx.lo[d];
    return a;
  }
};

template <class F>
inline void for_box(const Box& b, F&& f) {
#pragma omp parallel for schedule(static)
  for (int k = b.lo[2]; k <= b.hi[2]; ++k)
    for (int j = b.lo[1]; j <= b.hi[1]; ++j)
      for (int i = b.lo[0]; i <= b.hi[0]; ++i) f(i, j, k);
}

// ---------------------------------------------------------------------------
// Equations of state.  Method names follow the PelePhysics EOS calls made on
// the hot path (Utilities.H:300-305, Riemann.H:51-178, Diffterm.H:41-52).
// ---------------------------------------------------------------------------

// Both equations of state are written around rWbar = R/Wbar = sum_k Y_k R/W_k
// (accumulated with fused multiply-adds in species order); every polynomial
// is evaluated by Horner's rule with std::fma.  The arithmetic is fixed
// exactly (IEEE fma, division and square root are correctly rounded), so an
// implementation that performs the same operations reproduces these values
// bit for bit.
// The equation-of-state and transport code below is templated on its scalar
// type R: double everywhere in the oracle, and a counting double in the
// flop-counting build of the reference harness (ref_shim/flop_count.hpp).
// exp and log are the shared pc_exp.h implementations (oexp / olog; the
// counting type overloads them).
inline double oexp(double x) { return pc_math::exp(x); }
inline double olog(double x) { return pc_math::log(x); }
#ifdef PC_COUNT_FLOPS
}  // namespace orc
namespace pcc {
inline CReal oexp(CReal x) {
  PCC_COUNT(exp);
  return CReal(pc_math::exp(x.v));
}
inline CReal olog(CReal x) {
  PCC_COUNT(log);
  return CReal(pc_math::log(x.v));
}
}  // namespace pcc
namespace orc {
#endif

template <int NS, class R>
inline R mix_rw(const pc_mechanism* m, const R* Y) {
  R s = 0.0;
  for (int k = 0; k < NS; ++k) s = std::fma(Y[k], RU / m->mw[k], s);
  return s;
}
// X_k = Y_k Wbar / W_k = Y_k (R/W_k) / rWbar.
template <int NS, class R>
inline void mix_y2x(const pc_mechanism* m, const R* Y, R* X) {
  const R rw = mix_rw<NS>(m, Y);
  for (int k = 0; k < NS; ++k) X[k] = Y[k] * (RU / m->mw[k]) / rw;
}

// Calorically perfect gas: e = cv T, cv = R / ((gamma-1) Wbar), p = (gamma-1) rho e.
template <int NS>
struct GammaLaw {
  const pc_mechanism* m;
  template <class R>
  void Y2WBAR(const R* Y, R& wbar) const { wbar = RU / mix_rw<NS>(m, Y); }
  template <class R>
  void REY2T(R /*rho*/, R e, const R* Y, R& T, int& /*iters*/, bool& ok) const {
    T = e * (m->gamma - 1.0) / mix_rw<NS>(m, Y);
    ok = true;
  }
  template <class R>
  void RTY2P(R rho, R T, const R* Y, R& p) const { p = rho * mix_rw<NS>(m, Y) * T; }
  template <class R>
  void RTY2Cs(R rho, R T, const R* Y, R& cs) const {
    R p;
    RTY2P(rho, T, Y, p);
    cs = std::sqrt(m->gamma * p / rho);
  }
  template <class R>
  void RTY2G(R, R, const R*, R& g) const { g = m->gamma; }
  template <class R>
  void RTY2dpde_dpdre(R rho, R T, const R* Y, R& dpde, R& dpdr_e) const {
    dpde = (m->gamma - 1.0) * rho;
    dpdr_e = mix_rw<NS>(m, Y) * T;
  }
  template <class R>
  void RPY2Cs(R rho, R p, const R*, R& cs) const { cs = std::sqrt(m->gamma * p / rho); }
  template <class R>
  void RYP2E(R rho, const R*, R p, R& e) const { e = p / ((m->gamma - 1.0) * rho); }
  template <class R>
  void Y2X(const R* Y, R* X) const { mix_y2x<NS>(m, Y, X); }
  template <class R>
  void T2Hi(R T, R* h) const {
    for (int k = 0; k < NS; ++k) h[k] = (m->gamma / (m->gamma - 1.0) * RU / m->mw[k]) * T;
  }
  template <class R>
  void TY2CpCv(R, const R* Y, R& cp, R& cv) const {
    const R rw = mix_rw<NS>(m, Y);
    cv = rw / (m->gamma - 1.0);
    cp = cv + rw;
  }
};

// Ideal-gas mixture with NASA-7 species polynomials (CHEMKIN convention,
// e = sum_k Y_k e_k(T), Docs/sphinx/Algorithms.rst:523-529).  With the
// species coefficients folded into mixture coefficients
//   C_n = sum_k Y_k (R/W_k) a_{n,k}   (n = 0..5, range of T),
// cv(T) = (C0 - rWbar) + C1 T + C2 T^2 + C3 T^3 + C4 T^4 and
// e(T)  = C5 + T (C0 - rWbar) + C1 T^2/2 + C2 T^3/3 + C3 T^4/4 + C4 T^5/5.
// One range split tmid shared by all species (nasa_tmid[0]).
template <int NS>
struct IdealMix {
  const pc_mechanism* m;
  int maxit;
  template <class R>
  int range(R T) const { return (T < m->nasa_tmid[0]) ? 0 : 1; }
  template <class R>
  void coefs(const R* Y, int r, R C[6]) const {
    const double(*a)[7] = r == 0 ? m->nasa_lo : m->nasa_hi;
    for (int n = 0; n < 6; ++n) {
      R s = 0.0;
      for (int k = 0; k < NS; ++k) s = std::fma(Y[k], (RU / m->mw[k]) * a[k][n], s);
      C[n] = s;
    }
  }
  template <class R>
  static R cv_of(const R C[6], R rw, R T) {
    return (C[0] - rw) + T * std::fma(T, std::fma(T, std::fma(T, C[4], C[3]), C[2]), C[1]);
  }
  template <class R>
  static R e_of(const R C[6], R rw, R T) {
    const R p = std::fma(
        T, std::fma(T, std::fma(T, std::fma(T, C[4] * 0.2, C[3] * 0.25), C[2] * (1.0 / 3.0)), C[1] * 0.5), C[0] - rw);
    return std::fma(T, p, C[5]);
  }
  template <class R>
  void Y2WBAR(const R* Y, R& wbar) const { wbar = RU / mix_rw<NS>(m, Y); }
  // Temperature from internal energy by Newton's method on e(T) = e_in,
  // started from the caller's guess (U(UTEMP), Utilities.H:285).  Steps are
  // clamped to +-1000 K and T is kept >= 10 K; the solve stops once
  // |T_new - T| <= 1e-12 T_new, or fails after maxit iterations.
  template <class R>
  void REY2T(R /*rho*/, R ein, const R* Y, R& T, int& iters, bool& ok) const {
    const R rw = mix_rw<NS>(m, Y);
    R t = T;
    if (!(t > 0.0) || !std::isfinite(t)) t = 1000.0;
    int r = range(t);
    R C[6];
    coefs(Y, r, C);
    ok = false;
    int it = 0;
    for (; it < maxit; ++it) {
      const int rn = range(t);
      if (rn != r) {
        r = rn;
        coefs(Y, r, C);
      }
      const R e = e_of(C, rw, t);
      const R cv = cv_of(C, rw, t);
      R dt = (ein - e) / cv;
      if (dt > 1000.0) dt = 1000.0;
      if (dt < -1000.0) dt = -1000.0;
      R tn = t + dt;
      if (tn < 10.0) tn = 10.0;
      const bool conv = std::fabs(tn - t) <= 1e-12 * tn;
      t = tn;
      if (conv) { ok = true; ++it; break; }
    }
    iters = it;
    T = t;
  }
  template <class R>
  void RTY2P(R rho, R T, const R* Y, R& p) const { p = rho * mix_rw<NS>(m, Y) * T; }
  // c^2 = (cp/cv) p / rho with cp = cv + R/Wbar, evaluated as (cp p) / (cv rho).
  template <class R>
  R cs_at(R rho, R p, R T, const R* Y, R rw) const {
    R C[6];
    coefs(Y, range(T), C);
    const R cv = cv_of(C, rw, T);
    return std::sqrt((cv + rw) * p / (cv * rho));
  }
  template <class R>
  void RTY2Cs(R rho, R T, const R* Y, R& cs) const {
    const R rw = mix_rw<NS>(m, Y);
    cs = cs_at(rho, rho * rw * T, T, Y, rw);
  }
  template <class R>
  void RTY2G(R, R T, const R* Y, R& g) const {
    const R rw = mix_rw<NS>(m, Y);
    R C[6];
    coefs(Y, range(T), C);
    const R cv = cv_of(C, rw, T);
    g = (cv + rw) / cv;
  }
  template <class R>
  void RTY2dpde_dpdre(R rho, R T, const R* Y, R& dpde, R& dpdr_e) const {
    const R rw = mix_rw<NS>(m, Y);
    R C[6];
    coefs(Y, range(T), C);
    dpde = rho * rw / cv_of(C, rw, T);
    dpdr_e = rw * T;
  }
  template <class R>
  void RPY2Cs(R rho, R p, const R* Y, R& cs) const {
    const R rw = mix_rw<NS>(m, Y);
    cs = cs_at(rho, p, p / (rho * rw), Y, rw);
  }
  template <class R>
  void RYP2E(R rho, const R* Y, R p, R& e) const {
    const R rw = mix_rw<NS>(m, Y);
    const R T = p / (rho * rw);
    R C[6];
    coefs(Y, range(T), C);
    e = e_of(C, rw, T);
  }
  template <class R>
  void Y2X(const R* Y, R* X) const { mix_y2x<NS>(m, Y, X); }
  // h_k = R/W_k T (h/RT)_k = e5_k + T (c0 + T (c1/2 + T (c2/3 + T (c3/4 + T c4/5)))), c = R/W_k a.
  template <class R>
  void T2Hi(R T, R* h) const {
    const double(*a)[7] = range(T) == 0 ? m->nasa_lo : m->nasa_hi;
    for (int k = 0; k < NS; ++k) {
      const double r = RU / m->mw[k];
      const double c[6] = {r * a[k][0], r * a[k][1], r * a[k][2], r * a[k][3], r * a[k][4], r * a[k][5]};
      const R p = std::fma(
          T, std::fma(T, std::fma(T, std::fma(T, R(c[4] * 0.2), R(c[3] * 0.25)), R(c[2] * (1.0 / 3.0))), R(c[1] * 0.5)),
          R(c[0]));
      h[k] = std::fma(T, p, R(c[5]));
    }
  }
  // Mixture e and cv at T (used by tests).
  template <class R>
  void TY2E_Cv(R T, const R* Y, R& e, R& cv) const {
    const R rw = mix_rw<NS>(m, Y);
    R C[6];
    coefs(Y, range(T), C);
    e = e_of(C, rw, T);
    cv = cv_of(C, rw, T);
  }
  template <class R>
  void TY2CpCv(R T, const R* Y, R& cp, R& cv) const {
    const R rw = mix_rw<NS>(m, Y);
    R C[6];
    coefs(Y, range(T), C);
    cv = cv_of(C, rw, T);
    cp = cv + rw;
  }
};

// ---------------------------------------------------------------------------
// Transport (pc_transcoeff, Source/TransCoeff.H:7-37; the problem hook is the
// default no-op, ProblemSpecificFunctions.H:141-161).
// ---------------------------------------------------------------------------
template <int NS, class EOS>
struct ConstantTransport {
  const pc_mechanism* m;
  template <class R>
  void transport(const EOS&, R, R, const R*, R* Ddiag, R& mu, R& xi, R& lam) const {
    mu = m->const_mu;
    xi = m->const_xi;
    lam = m->const_lambda;
    for (int k = 0; k < NS; ++k) Ddiag[k] = m->const_rhoD;
  }
};

// Mixture-averaged transport (Docs/sphinx/Algorithms.rst:540-566):
//   mu = (sum X_m mu_m^6)^(1/6), lambda = (sum X_m lambda_m^(1/4))^4,
//   rhoD_m = rho (W_m/Wbar) D_m,mix, D_m,mix = (1-Y_m) / sum_{j!=m} X_j / D_mj(T,p),
// so that the flux rhoD_m grad X_m used by SpeciesEnergyFlux is the
// Hirschfelder-Curtiss mass flux,
// pure-species fits ln q = sum_n c_n (ln T)^n.  D_mj(T,p) = D_mj(T) p_ref/p.
// Mole fractions in the diffusion sum are floored at 1e-15 so a pure
// species keeps a finite mixture coefficient.  Bulk viscosity is
// xi = sum_m X_m bulk_ratio_m mu_m.  Binary fits are symmetric; the upper
// triangle (k < j) is used.  mu_k^6 is formed as ((mu_k^2)^2) mu_k^2.
template <int NS, class EOS>
struct SimpleTransport {
  const pc_mechanism* m;
  template <class R>
  static R fit(const double* c, R L) { return std::fma(L, std::fma(L, std::fma(L, R(c[3]), R(c[2])), R(c[1])), R(c[0])); }
  template <class R>
  void transport(const EOS& eos, R T, R rho, const R* Y, R* Ddiag, R& mu, R& xi, R& lam) const {
    R X[NS];
    eos.Y2X(Y, X);
    R p;
    eos.RTY2P(rho, T, Y, p);
    const R L = olog(T);
    R smu = 0.0, slam = 0.0, sxi = 0.0;
    for (int k = 0; k < NS; ++k) {
      const R mk = oexp(fit(m->visc_fit[k], L));
      const R m2 = mk * mk;
      smu = std::fma(X[k], m2 * m2 * m2, smu);
      slam = std::fma(X[k], oexp(0.25 * fit(m->cond_fit[k], L)), slam);
      sxi = std::fma(X[k], m->bulk_ratio[k] * mk, sxi);
    }
    mu = oexp(olog(smu) * (1.0 / 6.0));
    const R l2 = slam * slam;
    lam = l2 * l2;
    xi = sxi;
    // 1/D_kj(T,p) = exp(-fit) p / p_ref, accumulated over j != k in order.
    const R pr = p * (1.0 / m->diff_pref);
    for (int k = 0; k < NS; ++k) {
      R s = 0.0;
      for (int j = 0; j < NS; ++j) {
        if (j == k) continue;
        const R invD = oexp(-fit(m->diff_fit[std::min(j, k)][std::max(j, k)], L)) * pr;
        s = std::fma(std::max(X[j], R(1e-15)), invD, s);
      }
      // W_k / Wbar = (R/Wbar) / (R/W_k): rhoD_k grad X_k is then the
      // Hirschfelder-Curtiss mass flux rho (W_k/Wbar) D_k,mix grad X_k.
      const R wrat = mix_rw<NS>(m, Y) / (RU / m->mw[k]);
      Ddiag[k] = (s > 0.0) ? R(rho * (1.0 - Y[k]) * wrat / s) : R(0.0);
    }
  }
};

// ---------------------------------------------------------------------------
// Pointwise kernels of the hot path.
// ---------------------------------------------------------------------------

// pc_ctoprim, Source/Utilities.H:239-320 (no rotating frame).
template <int NS, class EOS>
inline void ctoprim(int i, int j, int k, const Arr<const double>& u, const Arr<double>& q, const Arr<double>& qa,
                    const EOS& eos, long long& newton_fail) {
  const double rho = u(i, j, k, URHO);
  const double rhoinv = 1.0 / rho;
  const double vx = u(i, j, k, UMX) * rhoinv;
  const double vy = u(i, j, k, UMY) * rhoinv;
  const double vz = u(i, j, k, UMZ) * rhoinv;
  const double kineng = 0.5 * rho * (vx * vx + vy * vy + vz * vz) - 0.5 * rho * 0.0 * 0.0 * 0.0 * 0.0;
  q(i, j, k, QRHO) = rho;
  q(i, j, k, QU) = vx;
  q(i, j, k, QV) = vy;
  q(i, j, k, QW) = vz;
  for (int n = 0; n < NS; n++) q(i, j, k, QFS + n) = u(i, j, k, UFS + n) / rho;
  const double e = (u(i, j, k, UEDEN) - kineng) * rhoinv;
  double T = u(i, j, k, UTEMP);
  double massfrac[NS];
  for (int sp = 0; sp < NS; ++sp) {
    const double y = q(i, j, k, sp + QFS);
    if ((-1e-4 * std::numeric_limits<double>::epsilon() < y) && (y < 1e-4 * std::numeric_limits<double>::epsilon()))
      q(i, j, k, sp + QFS) = 0.0;
    massfrac[sp] = q(i, j, k, sp + QFS);
  }
  double dpdr_e, dpde, gam1, cs, wbar, p;
  int iters = 0;
  bool ok = true;
  eos.Y2WBAR(massfrac, wbar);
  eos.REY2T(rho, e, massfrac, T, iters, ok);
  if (!ok) {
#pragma omp atomic
    newton_fail += 1;
  }
  eos.RTY2P(rho, T, massfrac, p);
  eos.RTY2Cs(rho, T, massfrac, cs);
  eos.RTY2G(rho, T, massfrac, gam1);
  eos.RTY2dpde_dpdre(rho, T, massfrac, dpde, dpdr_e);
  q(i, j, k, QTEMP) = T;
  q(i, j, k, QREINT) = e * rho;
  q(i, j, k, QPRES) = p;
  q(i, j, k, QGAME) = p / (e * rho) + 1.0;
  qa(i, j, k, QDPDR) = dpdr_e;
  qa(i, j, k, QDPDE) = dpde;
  qa(i, j, k, QGAMC) = gam1;
  qa(i, j, k, QC) = cs;
  qa(i, j, k, QCSML) = std::max(small_num(), small_num() * cs);
  qa(i, j, k, QRSPEC) = RU / wbar;
}

// pc_move_transcoefs_to_ec, Source/Utilities.H:322-342.
inline double face_coef(double a, double b, bool harmonic) {
  if (harmonic) return (a * b > 0.0) ? 2.0 * (a * b) / (a + b) : 0.0;
  return 0.5 * (a + b);
}

// pc_diffusion_flux + SpeciesEnergyFlux<ideal>, Source/Diffterm.H:20-75,344-461.
template <int NS, class EOS>
inline void diffusion_flux(int i, int j, int k, int dir, const Arr<double>& q, const double* coef, double area,
                           const Arr<double>& flx, const double dxinv[3], const EOS& eos) {
  const int dComp_mu = NS, dComp_xi = NS + 1, dComp_lambda = NS + 2;
  const int im = i - (dir == 0), jm = j - (dir == 1), km = k - (dir == 2);
  double taux = 0.0, tauy = 0.0, tauz = 0.0;
  if (dir == 0) {
    const double dudx = dxinv[0] * (q(i, j, k, QU) - q(im, jm, km, QU));
    const double dvdx = dxinv[0] * (q(i, j, k, QV) - q(im, jm, km, QV));
    const double dwdx = dxinv[0] * (q(i, j, k, QW) - q(im, jm, km, QW));
    const double dudy = (q(i, j + 1, k, QU) + q(i - 1, j + 1, k, QU) - q(i, j - 1, k, QU) - q(i - 1, j - 1, k, QU)) *
                        (0.25 * dxinv[1]);
    const double dvdy = (q(i, j + 1, k, QV) + q(i - 1, j + 1, k, QV) - q(i, j - 1, k, QV) - q(i - 1, j - 1, k, QV)) *
                        (0.25 * dxinv[1]);
    const double dudz = (q(i, j, k + 1, QU) + q(i - 1, j, k + 1, QU) - q(i, j, k - 1, QU) - q(i - 1, j, k - 1, QU)) *
                        (0.25 * dxinv[2]);
    const double dwdz = (q(i, j, k + 1, QW) + q(i - 1, j, k + 1, QW) - q(i, j, k - 1, QW) - q(i - 1, j, k - 1, QW)) *
                        (0.250 * dxinv[2]);
    const double divu = dudx + dvdy + dwdz;
    taux = coef[dComp_mu] * (2.0 * dudx - 2.0 / 3.0 * divu) + coef[dComp_xi] * divu;
    tauy = coef[dComp_mu] * (dudy + dvdx);
    tauz = coef[dComp_mu] * (dudz + dwdx);
  } else if (dir == 1) {
    const double dudy = dxinv[1] * (q(i, j, k, QU) - q(im, jm, km, QU));
    const double dvdy = dxinv[1] * (q(i, j, k, QV) - q(im, jm, km, QV));
    const double dwdy = dxinv[1] * (q(i, j, k, QW) - q(im, jm, km, QW));
    const double dudx = (q(i + 1, j, k, QU) + q(i + 1, j - 1, k, QU) - q(i - 1, j, k, QU) - q(i - 1, j - 1, k, QU)) *
                        (0.25 * dxinv[0]);
    const double dvdx = (q(i + 1, j, k, QV) + q(i + 1, j - 1, k, QV) - q(i - 1, j, k, QV) - q(i - 1, j - 1, k, QV)) *
                        (0.25 * dxinv[0]);
    const double dvdz = (q(i, j, k + 1, QV) + q(i, j - 1, k + 1, QV) - q(i, j, k - 1, QV) - q(i, j - 1, k - 1, QV)) *
                        (0.25 * dxinv[2]);
    const double dwdz = (q(i, j, k + 1, QW) + q(i, j - 1, k + 1, QW) - q(i, j, k - 1, QW) - q(i, j - 1, k - 1, QW)) *
                        (0.25 * dxinv[2]);
    const double divu = dudx + dvdy + dwdz;
    taux = coef[dComp_mu] * (dudy + dvdx);
    tauy = coef[dComp_mu] * (2.0 * dvdy - 2.0 / 3.0 * divu) + coef[dComp_xi] * divu;
    tauz = coef[dComp_mu] * (dwdy + dvdz);
  } else {
    const double dudz = dxinv[2] * (q(i, j, k, QU) - q(im, jm, km, QU));
    const double dvdz = dxinv[2] * (q(i, j, k, QV) - q(im, jm, km, QV));
    const double dwdz = dxinv[2] * (q(i, j, k, QW) - q(im, jm, km, QW));
    const double dudx = (q(i + 1, j, k, QU) + q(i + 1, j, k - 1, QU) - q(i - 1, j, k, QU) - q(i - 1, j, k - 1, QU)) *
                        (0.25 * dxinv[0]);
    const double dwdx = (q(i + 1, j, k, QW) + q(i + 1, j, k - 1, QW) - q(i - 1, j, k, QW) - q(i - 1, j, k - 1, QW)) *
                        (0.25 * dxinv[0]);
    const double dvdy = (q(i, j + 1, k, QV) + q(i, j + 1, k - 1, QV) - q(i, j - 1, k, QV) - q(i, j - 1, k - 1, QV)) *
                        (0.25 * dxinv[1]);
    const double dwdy = (q(i, j + 1, k, QW) + q(i, j + 1, k - 1, QW) - q(i, j - 1, k, QW) - q(i, j - 1, k - 1, QW)) *
                        (0.25 * dxinv[1]);
    const double divu = dudx + dvdy + dwdz;
    taux = coef[dComp_mu] * (dudz + dwdx);
    tauy = coef[dComp_mu] * (dvdz + dwdy);
    tauz = coef[dComp_mu] * (2.0 * dwdz - 2.0 / 3.0 * divu) + coef[dComp_xi] * divu;
  }
  const double dTdd = dxinv[dir] * (q(i, j, k, QTEMP) - q(im, jm, km, QTEMP));
  flx(i, j, k, UMX) = -taux;
  flx(i, j, k, UMY) = -tauy;
  flx(i, j, k, UMZ) = -tauz;
  flx(i, j, k, UEDEN) = 0.5 * (-taux * (q(i, j, k, QU) + q(im, jm, km, QU)) - tauy * (q(i, j, k, QV) + q(im, jm, km, QV)) -
                               tauz * (q(i, j, k, QW) + q(im, jm, km, QW))) -
                        coef[dComp_lambda] * dTdd;
  // SpeciesEnergyFlux<ideal EOS>
  {
    double mass1[NS], mass2[NS], mole1[NS], mole2[NS], hi1[NS], hi2[NS];
    for (int n = 0; n < NS; ++n) mass1[n] = q(i, j, k, n + QFS);
    eos.Y2X(mass1, mole1);
    for (int n = 0; n < NS; ++n) mass2[n] = q(im, jm, km, n + QFS);
    eos.Y2X(mass2, mole2);
    eos.T2Hi(q(i, j, k, QTEMP), hi1);
    eos.T2Hi(q(im, jm, km, QTEMP), hi2);
    double Vc = 0.0;
    const double dpdx = dxinv[dir] * (q(i, j, k, QPRES) - q(im, jm, km, QPRES));
    const double dlnp = dpdx / (0.5 * (q(i, j, k, QPRES) + q(im, jm, km, QPRES)));
    for (int n = 0; n < NS; ++n) {
      const double Xface = 0.5 * (mole1[n] + mole2[n]);
      const double Yface = 0.5 * (mass1[n] + mass2[n]);
      const double hface = 0.5 * (hi1[n] + hi2[n]);
      const double dXdx = dxinv[dir] * (mole1[n] - mole2[n]);
      const double Vd = -coef[n] * (dXdx + (Xface - Yface) * dlnp);
      flx(i, j, k, UFS + n) = Vd;
      Vc += Vd;
      flx(i, j, k, UEDEN) += Vd * hface;
    }
    for (int n = 0; n < NS; ++n) {
      const double Yface = 0.5 * (mass1[n] + mass2[n]);
      const double hface = 0.5 * (hi1[n] + hi2[n]);
      flx(i, j, k, UFS + n) -= Yface * Vc;
      flx(i, j, k, UEDEN) -= Yface * hface * Vc;
    }
  }
  flx(i, j, k, UMX) *= area;
  flx(i, j, k, UMY) *= area;
  flx(i, j, k, UMZ) *= area;
  flx(i, j, k, UEDEN) *= area;
  for (int n = 0; n < NS; ++n) flx(i, j, k, UFS + n) *= area;
}

// mol_slope, Source/MOL.H:28-113 (all cells regular).
template <int NS>
inline void mol_slope(int i, int j, int k, int dir, const int q_idx[3], const Arr<double>& q, const Arr<double>& qaux,
                      const Arr<double>& dq) {
  const int QVAR = 8 + NS;
  const int im = i - (dir == 0), jm = j - (dir == 1), km = k - (dir == 2);
  const int ip = i + (dir == 0), jp = j + (dir == 1), kp = k + (dir == 2);
  double dlft[8 + NS], drgt[8 + NS];
  for (int n = 0; n < QVAR; ++n) dlft[n] = drgt[n] = 0.0;
  const double c = qaux(i, j, k, QC);
  dlft[0] = 0.5 * (q(i, j, k, QPRES) - q(im, jm, km, QPRES)) / c -
            0.5 * q(i, j, k, QRHO) * (q(i, j, k, q_idx[0]) - q(im, jm, km, q_idx[0]));
  dlft[1] = 0.5 * (q(i, j, k, QPRES) - q(im, jm, km, QPRES)) / c +
            0.5 * q(i, j, k, QRHO) * (q(i, j, k, q_idx[0]) - q(im, jm, km, q_idx[0]));
  dlft[2] = q(i, j, k, q_idx[1]) - q(im, jm, km, q_idx[1]);
  dlft[3] = q(i, j, k, q_idx[2]) - q(im, jm, km, q_idx[2]);
  drgt[0] = 0.5 * (q(ip, jp, kp, QPRES) - q(i, j, k, QPRES)) / c -
            0.5 * q(i, j, k, QRHO) * (q(ip, jp, kp, q_idx[0]) - q(i, j, k, q_idx[0]));
  drgt[1] = 0.5 * (q(ip, jp, kp, QPRES) - q(i, j, k, QPRES)) / c +
            0.5 * q(i, j, k, QRHO) * (q(ip, jp, kp, q_idx[0]) - q(i, j, k, q_idx[0]));
  drgt[2] = q(ip, jp, kp, q_idx[1]) - q(i, j, k, q_idx[1]);
  drgt[3] = q(ip, jp, kp, q_idx[2]) - q(i, j, k, q_idx[2]);
  for (int n = 0; n < NS; n++) {
    dlft[QFS + n] = q(i, j, k, QRHO) * q(i, j, k, QFS + n) - q(im, jm, km, QRHO) * q(im, jm, km, QFS + n) -
                    q(i, j, k, QFS + n) * (q(i, j, k, QPRES) - q(im, jm, km, QPRES)) / (c * c);
    drgt[QFS + n] = q(ip, jp, kp, QRHO) * q(ip, jp, kp, QFS + n) - q(i, j, k, QRHO) * q(i, j, k, QFS + n) -
                    q(i, j, k, QFS + n) * (q(ip, jp, kp, QPRES) - q(i, j, k, QPRES)) / (c * c);
  }
  for (int n = 0; n < QVAR; n++) {
    const double dcen = 0.5 * (dlft[n] + drgt[n]);
    const double dlim = dlft[n] * drgt[n] >= 0.0 ? 2.0 * std::min(std::fabs(dlft[n]), std::fabs(drgt[n])) : 0.0;
    dq(i, j, k, n) = std::copysign(1.0, dcen) * std::min(dlim, std::fabs(dcen));
  }
}

// riemann, Source/Riemann.H:6-200 (bc_test_val = 1, no rotating frame).
template <int NS, class EOS>
inline void riemann(double rl, double ul, double vl, double v2l, double pl, const double* spl, double rr, double ur,
                    double vr, double v2r, double pr, const double* spr, double cav, double& ustar, double& uflx_rho,
                    double* uflx_rhoY, double& uflx_u, double& uflx_v, double& uflx_w, double& uflx_eden,
                    double& uflx_eint, const EOS& eos) {
  const double wsmall = std::numeric_limits<double>::min();
  double gdnv_state_massfrac[NS];
  for (int n = 0; n < NS; n++) gdnv_state_massfrac[n] = spl[n];
  double cl = 0.0;
  eos.RPY2Cs(rl, pl, gdnv_state_massfrac, cl);
  for (int n = 0; n < NS; n++) gdnv_state_massfrac[n] = spr[n];
  double cr = 0.0;
  eos.RPY2Cs(rr, pr, gdnv_state_massfrac, cr);
  const double wl = std::max(wsmall, cl * rl);
  const double wr = std::max(wsmall, cr * rr);
  const double pstar = std::max(std::numeric_limits<double>::min(), ((wr * pl + wl * pr) + wl * wr * (ul - ur)) / (wl + wr));
  ustar = ((wl * ul + wr * ur) + (pl - pr)) / (wl + wr);
  bool mask = ustar > 0.0;
  double ro = 0.0;
  double rspo[NS];
  for (int n = 0; n < NS; n++) {
    rspo[n] = mask ? rl * spl[n] : rr * spr[n];
    ro += rspo[n];
  }
  double uo = mask ? ul : ur;
  double po = mask ? pl : pr;
  mask = std::fabs(ustar) < smallu() * 0.5 * (std::fabs(ul) + std::fabs(ur)) || ustar == 0.0;
  ustar = mask ? 0.0 : ustar;
  ro = 0.0;
  for (int n = 0; n < NS; n++) {
    rspo[n] = mask ? 0.5 * (rl * spl[n] + rr * spr[n]) : rspo[n];
    ro += rspo[n];
  }
  uo = mask ? 0.5 * (ul + ur) : uo;
  po = mask ? 0.5 * (pl + pr) : po;
  double gdnv_state_rho = ro;
  double gdnv_state_p = po;
  for (int n = 0; n < NS; n++) gdnv_state_massfrac[n] = rspo[n] / ro;
  double gdnv_state_e;
  eos.RYP2E(gdnv_state_rho, gdnv_state_massfrac, gdnv_state_p, gdnv_state_e);
  double co;
  eos.RPY2Cs(gdnv_state_rho, gdnv_state_p, gdnv_state_massfrac, co);
  const double drho = (pstar - po) / (co * co);
  double rstar = 0.0;
  double rspstar[NS];
  for (int n = 0; n < NS; n++) {
    const double spon = rspo[n] / ro;
    rspstar[n] = std::max(0.0, rspo[n] + drho * spon);
    rstar += rspstar[n];
  }
  gdnv_state_rho = rstar;
  gdnv_state_p = pstar;
  for (int n = 0; n < NS; n++) gdnv_state_massfrac[n] = rspstar[n] / rstar;
  eos.RYP2E(gdnv_state_rho, gdnv_state_massfrac, gdnv_state_p, gdnv_state_e);
  double cstar;
  eos.RPY2Cs(gdnv_state_rho, gdnv_state_p, gdnv_state_massfrac, cstar);
  const double sgnm = std::copysign(1.0, ustar);
  double spout = co - sgnm * uo;
  double spin = cstar - sgnm * ustar;
  const double ushock = 0.5 * (spin + spout);
  mask = pstar < po;
  spout = mask ? spout : ushock;
  spin = mask ? spin : ushock;
  const double scr = (std::fabs(spout - spin) < very_small_num()) ? small_num() * cav : spout - spin;
  const double frac = std::max(0.0, std::min(1.0, (1.0 + (spout + spin) / scr) * 0.5));
  mask = ustar > 0.0;
  double qint_iv1 = mask ? vl : vr;
  double qint_iv2 = mask ? v2l : v2r;
  mask = (ustar == 0.0);
  qint_iv1 = mask ? 0.5 * (vl + vr) : qint_iv1;
  qint_iv2 = mask ? 0.5 * (v2l + v2r) : qint_iv2;
  double rgd = 0.0;
  double rspgd[NS];
  for (int n = 0; n < NS; n++) {
    rspgd[n] = frac * rspstar[n] + (1.0 - frac) * rspo[n];
    rgd += rspgd[n];
  }
  double qint_iu = frac * ustar + (1.0 - frac) * uo;
  double qint_gdpres = frac * pstar + (1.0 - frac) * po;
  gdnv_state_rho = rgd;
  gdnv_state_p = qint_gdpres;
  for (int n = 0; n < NS; n++) gdnv_state_massfrac[n] = rspgd[n] / rgd;
  eos.RYP2E(gdnv_state_rho, gdnv_state_massfrac, gdnv_state_p, gdnv_state_e);
  mask = (spout < 0.0);
  rgd = 0.0;
  for (int n = 0; n < NS; n++) {
    rspgd[n] = mask ? rspo[n] : rspgd[n];
    rgd += rspgd[n];
  }
  qint_iu = mask ? uo : qint_iu;
  qint_gdpres = mask ? po : qint_gdpres;
  mask = (spin >= 0.0);
  rgd = 0.0;
  for (int n = 0; n < NS; n++) {
    rspgd[n] = mask ? rspstar[n] : rspgd[n];
    rgd += rspgd[n];
  }
  qint_iu = mask ? ustar : qint_iu;
  qint_gdpres = mask ? pstar : qint_gdpres;
  gdnv_state_rho = rgd;
  gdnv_state_p = qint_gdpres;
  for (int n = 0; n < NS; n++) gdnv_state_massfrac[n] = rspgd[n] / rgd;
  eos.RYP2E(gdnv_state_rho, gdnv_state_massfrac, gdnv_state_p, gdnv_state_e);
  const double regd = gdnv_state_rho * gdnv_state_e;
  qint_iu = 1 * qint_iu;
  uflx_rho = rgd * qint_iu;
  for (int n = 0; n < NS; n++) uflx_rhoY[n] = rspgd[n] * qint_iu;
  uflx_u = uflx_rho * qint_iu + qint_gdpres;
  uflx_v = uflx_rho * qint_iv1;
  uflx_w = uflx_rho * qint_iv2;
  const double rhoetot = regd + 0.5 * rgd * (qint_iu * qint_iu + qint_iv1 * qint_iv1 + qint_iv2 * qint_iv2) -
                         0.5 * rgd * 0.0 * 0.0 * 0.0 * 0.0;
  uflx_eden = qint_iu * (rhoetot + qint_gdpres);
  uflx_eint = qint_iu * regd;
}

// laxfriedrich_flux, Source/Riemann.H:202-307 (no rotating frame).
template <int NS, class EOS>
inline void laxfriedrich_flux(double rl, double ul, double vl, double v2l, double pl, const double* spl, double rr,
                              double ur, double vr, double v2r, double pr, const double* spr, double& ustar,
                              double& maxeigval, double& uflx_rho, double* uflx_rhoY, double& uflx_u, double& uflx_v,
                              double& uflx_w, double& uflx_eden, double& uflx_eint, const EOS& eos) {
  const double wsmall = std::numeric_limits<double>::min();
  double cl = 0.0, cr = 0.0, el = 0.0, er = 0.0;
  double mfrac_l[NS], mfrac_r[NS];
  for (int n = 0; n < NS; n++) { mfrac_l[n] = spl[n]; mfrac_r[n] = spr[n]; }
  eos.RPY2Cs(rl, pl, mfrac_l, cl);
  eos.RPY2Cs(rr, pr, mfrac_r, cr);
  eos.RYP2E(rl, mfrac_l, pl, el);
  eos.RYP2E(rr, mfrac_r, pr, er);
  const double r_elt = rl * (el + 0.5 * (ul * ul + vl * vl + v2l * v2l) - 0.5 * 0.0 * 0.0 * 0.0 * 0.0);
  const double r_ert = rr * (er + 0.5 * (ur * ur + vr * vr + v2r * v2r) - 0.5 * 0.0 * 0.0 * 0.0 * 0.0);
  const double wl = std::max(wsmall, cl * rl);
  const double wr = std::max(wsmall, cr * rr);
  ustar = ((wl * ul + wr * ur) + (pl - pr)) / (wl + wr);
  const bool mask = std::fabs(ustar) < smallu() * 0.5 * (std::fabs(ul) + std::fabs(ur)) || ustar == 0.0;
  ustar = mask ? 0.0 : ustar;
  const double chalf = 0.5 * (cr + cl);
  const double max_wavespd = std::fabs(ustar) + chalf;
  maxeigval = max_wavespd;
  uflx_rho = 0.0;
  for (int n = 0; n < NS; n++) {
    uflx_rhoY[n] = 0.5 * ((rl * ul * spl[n] + rr * ur * spr[n]) - max_wavespd * (rr * spr[n] - rl * spl[n]));
    uflx_rho += uflx_rhoY[n];
  }
  uflx_u = 0.5 * ((rl * ul * ul + pl + rr * ur * ur + pr) - max_wavespd * (rr * ur - rl * ul));
  uflx_v = 0.5 * ((rl * vl * ul + rr * vr * ur) - max_wavespd * (rr * vr - rl * vl));
  uflx_w = 0.5 * ((rl * v2l * ul + rr * v2r * ur) - max_wavespd * (rr * v2r - rl * v2l));
  uflx_eden = 0.5 * (((r_elt + pl) * ul + (r_ert + pr) * ur) - max_wavespd * (r_ert - r_elt));
  uflx_eint = 0.5 * ((rl * el * ul + rr * er * ur) - max_wavespd * (rr * er - rl * el));
}

// pc_compute_hyp_mol_flux, Source/MOL.cpp:5-204 (regular cells).
template <int NS, class EOS>
inline void hyp_mol_flux(const Box& cbox, const Arr<double>& q, const Arr<double>& qaux, const Arr<double> flx[3],
                         const double area[3], int mol_iorder, bool use_laxf_flux, const EOS& eos) {
  const int QVAR = 8 + NS;
  const int NVAR = 7 + NS;
  for (int dir = 0; dir < 3; dir++) {
    Fab<double> dq_fab(cbox, QVAR);
    Arr<double> dq = dq_fab.arr();
    const int bdim[3] = {dir == 0, dir == 1, dir == 2};
    const int q_idx[3] = {bdim[0] * QU + bdim[1] * QV + bdim[2] * QW, bdim[0] * QV + bdim[1] * QU + bdim[2] * QU,
                          bdim[0] * QW + bdim[1] * QW + bdim[2] * QV};
    const int f_idx[3] = {bdim[0] * UMX + bdim[1] * UMY + bdim[2] * UMZ,
                          bdim[0] * UMY + bdim[1] * UMX + bdim[2] * UMX,
                          bdim[0] * UMZ + bdim[1] * UMZ + bdim[2] * UMY};
    if (mol_iorder != 1) {
      for_box(cbox, [&](int i, int j, int k) { mol_slope<NS>(i, j, k, dir, q_idx, q, qaux, dq); });
    }
    const Box tbox = grow_dir(cbox, dir, -1);
    const Box ebox = surrounding_nodes(tbox, dir);
    const Arr<double> f = flx[dir];
    const double a = area[dir];
    for_box(ebox, [&](int i, int j, int k) {
      const int im = i - (dir == 0), jm = j - (dir == 1), km = k - (dir == 2);
      enum { R_RHO = 0, R_UN = 1, R_UT1 = 2, R_UT2 = 3, R_P = 4, R_Y = 5 };
      double qtempl[5 + NS], qtempr[5 + NS];
      for (int n = 0; n < 5 + NS; ++n) qtempl[n] = qtempr[n] = 0.0;
      qtempl[R_UN] = q(im, jm, km, q_idx[0]) + 0.5 * ((dq(im, jm, km, 1) - dq(im, jm, km, 0)) / q(im, jm, km, QRHO));
      qtempl[R_P] = q(im, jm, km, QPRES) + 0.5 * (dq(im, jm, km, 0) + dq(im, jm, km, 1)) * qaux(im, jm, km, QC);
      qtempl[R_UT1] = q(im, jm, km, q_idx[1]) + 0.5 * dq(im, jm, km, 2);
      qtempl[R_UT2] = q(im, jm, km, q_idx[2]) + 0.5 * dq(im, jm, km, 3);
      qtempl[R_RHO] = 0.0;
      for (int n = 0; n < NS; n++) {
        qtempl[R_Y + n] = q(im, jm, km, QFS + n) * q(im, jm, km, QRHO) +
                          0.5 * (dq(im, jm, km, QFS + n) +
                                 q(im, jm, km, QFS + n) * (dq(im, jm, km, 0) + dq(im, jm, km, 1)) / qaux(im, jm, km, QC));
        qtempl[R_RHO] += qtempl[R_Y + n];
      }
      for (int n = 0; n < NS; n++) qtempl[R_Y + n] = qtempl[R_Y + n] / qtempl[R_RHO];
      qtempr[R_UN] = q(i, j, k, q_idx[0]) - 0.5 * ((dq(i, j, k, 1) - dq(i, j, k, 0)) / q(i, j, k, QRHO));
      qtempr[R_P] = q(i, j, k, QPRES) - 0.5 * (dq(i, j, k, 0) + dq(i, j, k, 1)) * qaux(i, j, k, QC);
      qtempr[R_UT1] = q(i, j, k, q_idx[1]) - 0.5 * dq(i, j, k, 2);
      qtempr[R_UT2] = q(i, j, k, q_idx[2]) - 0.5 * dq(i, j, k, 3);
      qtempr[R_RHO] = 0.0;
      for (int n = 0; n < NS; n++) {
        qtempr[R_Y + n] = q(i, j, k, QFS + n) * q(i, j, k, QRHO) -
                          0.5 * (dq(i, j, k, QFS + n) + q(i, j, k, QFS + n) * (dq(i, j, k, 0) + dq(i, j, k, 1)) / qaux(i, j, k, QC));
        qtempr[R_RHO] += qtempr[R_Y + n];
      }
      for (int n = 0; n < NS; n++) qtempr[R_Y + n] = qtempr[R_Y + n] / qtempr[R_RHO];
      const double cavg = 0.5 * (qaux(i, j, k, QC) + qaux(im, jm, km, QC));
      double spl[NS], spr[NS];
      for (int n = 0; n < NS; n++) { spl[n] = qtempl[R_Y + n]; spr[n] = qtempr[R_Y + n]; }
      double flux_tmp[7 + NS];
      for (int n = 0; n < NVAR; ++n) flux_tmp[n] = 0.0;
      double ustar = 0.0;
      if (!use_laxf_flux) {
        riemann<NS>(qtempl[R_RHO], qtempl[R_UN], qtempl[R_UT1], qtempl[R_UT2], qtempl[R_P], spl, qtempr[R_RHO],
                    qtempr[R_UN], qtempr[R_UT1], qtempr[R_UT2], qtempr[R_P], spr, cavg, ustar, flux_tmp[URHO],
                    &flux_tmp[UFS], flux_tmp[f_idx[0]], flux_tmp[f_idx[1]], flux_tmp[f_idx[2]], flux_tmp[UEDEN],
                    flux_tmp[UEINT], eos);
      } else {
        double maxeigval = 0.0;
        laxfriedrich_flux<NS>(qtempl[R_RHO], qtempl[R_UN], qtempl[R_UT1], qtempl[R_UT2], qtempl[R_P], spl,
                              qtempr[R_RHO], qtempr[R_UN], qtempr[R_UT1], qtempr[R_UT2], qtempr[R_P], spr, ustar,
                              maxeigval, flux_tmp[URHO], &flux_tmp[UFS], flux_tmp[f_idx[0]], flux_tmp[f_idx[1]],
                              flux_tmp[f_idx[2]], flux_tmp[UEDEN], flux_tmp[UEINT], eos);
      }
      flux_tmp[UTEMP] = 0.0;
      for (int ivar = 0; ivar < NVAR; ivar++) f(i, j, k, ivar) += flux_tmp[ivar] * a;
    });
  }
}

// The regular-box body of PeleC::getMOLSrcTerm for one box.
// S must cover grow(vbox, 4); rhs is written on vbox.
template <int NS, class EOS, class TRANS>
inline void mol_rhs_box(const pc_mol_config& cfg, const EOS& eos, const TRANS& trans, const Box& vbox,
                        const Arr<const double>& sar, const Arr<double>& rhs, const double dx[3],
                        long long& newton_fail, const Arr<double>* flux_out = nullptr) {
  const int NVAR = 7 + NS, QVAR = 8 + NS, nCompTr = NS + 3;
  if (!cfg.diffuse_temp && !cfg.diffuse_enth && !cfg.diffuse_spec && !cfg.diffuse_vel && !cfg.do_hydro) {
    for_box(vbox, [&](int i, int j, int k) {
      for (int n = 0; n < NVAR; ++n) rhs(i, j, k, n) = 0.0;
    });
    return;
  }
  const double dxinv[3] = {1.0 / dx[0], 1.0 / dx[1], 1.0 / dx[2]};
  // Cartesian metrics as AMReX Geometry::GetVolume / GetFaceArea.
  const double vol = dx[0] * dx[1] * dx[2];
  const double area[3] = {dx[1] * dx[2], dx[0] * dx[2], dx[0] * dx[1]};
  const int ng = 4;
  const Box gbox = grow(vbox, ng);
  const Box cbox = grow(vbox, ng - 1);
  Fab<double> qf(gbox, QVAR), qauxf(gbox, NQAUX), coeff_cc(gbox, nCompTr);
  Arr<double> qar = qf.arr(), qauxar = qauxf.arr(), coe = coeff_cc.arr();
  for_box(gbox, [&](int i, int j, int k) { ctoprim<NS>(i, j, k, sar, qar, qauxar, eos, newton_fail); });
  for_box(gbox, [&](int i, int j, int k) {
    double mu, xi, lam, Ddiag[NS], Y[NS];
    for (int n = 0; n < NS; ++n) Y[n] = qar(i, j, k, QFS + n);
    trans.transport(eos, qar(i, j, k, QTEMP), qar(i, j, k, QRHO), Y, Ddiag, mu, xi, lam);
    for (int n = 0; n < NS; ++n) coe(i, j, k, n) = Ddiag[n];
    coe(i, j, k, NS) = mu;
    coe(i, j, k, NS + 1) = xi;
    coe(i, j, k, NS + 2) = lam;
  });
  std::vector<Fab<double>> flux_ec;
  Box eboxes[3];
  Arr<double> flx[3];
  flux_ec.reserve(3);
  for (int dir = 0; dir < 3; ++dir) {
    eboxes[dir] = surrounding_nodes(cbox, dir);
    flux_ec.emplace_back(eboxes[dir], NVAR);
  }
  for (int dir = 0; dir < 3; ++dir) flx[dir] = flux_ec[dir].arr();
  Fab<double> Dfab(cbox, NVAR);
  Arr<double> Dterm = Dfab.arr();
  const bool harmonic = cfg.transport_harmonic_mean != 0;
  for (int dir = 0; dir < 3; dir++) {
    for_box(eboxes[dir], [&](int i, int j, int k) {
      double cf[PC_MAX_SPECIES + 3];
      const int im = i - (dir == 0), jm = j - (dir == 1), km = k - (dir == 2);
      for (int n = 0; n < nCompTr; n++) cf[n] = face_coef(coe(i, j, k, n), coe(im, jm, km, n), harmonic);
      diffusion_flux<NS>(i, j, k, dir, qar, cf, area[dir], flx[dir], dxinv, eos);
    });
  }
  for (int dir = 0; dir < 3; dir++) {
    for_box(eboxes[dir], [&](int i, int j, int k) {
      if (!cfg.diffuse_temp && !cfg.diffuse_enth) flx[dir](i, j, k, UEDEN) = 0.0;
      if (!cfg.diffuse_spec)
        for (int n = 0; n < NS; ++n) flx[dir](i, j, k, UFS + n) = 0.0;
      if (!cfg.diffuse_vel)
        for (int n = UMX; n <= UMZ; ++n) flx[dir](i, j, k, n) = 0.0;
    });
  }
  if (cfg.do_hydro) hyp_mol_flux<NS>(cbox, qar, qauxar, flx, area, cfg.plm_iorder, cfg.use_laxf_flux != 0, eos);
  // pc_flux_div (Diffterm.H:463-484): AMREX_D_TERM pastes the three
  // differences into one expression, -(fx1 - fx0 + fy1 - fy0 + fz1 - fz0) / V,
  // which C++ evaluates left to right.
  for_box(cbox, [&](int i, int j, int k) {
    for (int n = 0; n < NVAR; ++n)
      Dterm(i, j, k, n) = -(flx[0](i + 1, j, k, n) - flx[0](i, j, k, n) + flx[1](i, j + 1, k, n) - flx[1](i, j, k, n) +
                            flx[2](i, j, k + 1, n) - flx[2](i, j, k, n)) /
                          vol;
  });
  for_box(vbox, [&](int i, int j, int k) {
    for (int n = 0; n < NVAR; ++n) rhs(i, j, k, n) = Dterm(i, j, k, n);
  });
  // The fluxes getMOLSrcTerm hands to the flux registers for refluxing
  // (Diffusion.cpp:652-670), on surroundingNodes(vbox, dir).
  if (flux_out)
    for (int dir = 0; dir < 3; ++dir)
      for_box(surrounding_nodes(vbox, dir), [&](int i, int j, int k) {
        for (int n = 0; n < NVAR; ++n) flux_out[dir](i, j, k, n) = flx[dir](i, j, k, n);
      });
}

// ---------------------------------------------------------------------------
// Time-advance building blocks of the MOL step (do_mol_advance,
// Source/Advance.cpp:45-196).
// ---------------------------------------------------------------------------

// PeleC::computeTemp (PeleC.cpp:2254-2271) with the default
// allow_small_energy = allow_negative_energy = true: reset_internal_energy
// (pc_rst_int_e, Utilities.H:219-236) then pc_cmpTemp (Utilities.H:67-84).
template <int NS, class EOS>
inline void compute_temp(const Box& vbox, const Arr<double>& S, const EOS& eos, long long& fails) {
  for_box(vbox, [&](int i, int j, int k) {
    {
      const double rho = S(i, j, k, URHO);
      const double rhoInv = 1.0 / rho;
      const double Up = S(i, j, k, UMX) * rhoInv;
      const double Vp = S(i, j, k, UMY) * rhoInv;
      const double Wp = S(i, j, k, UMZ) * rhoInv;
      const double ke = 0.5 * (Up * Up + Vp * Vp + Wp * Wp) - 0.5 * 0.0 * 0.0 * 0.0 * 0.0;
      S(i, j, k, UEINT) = S(i, j, k, UEDEN) - rho * ke;
    }
    const double rhoInv = 1.0 / S(i, j, k, URHO);
    double T = S(i, j, k, UTEMP);
    const double e = S(i, j, k, UEINT) * rhoInv;
    double Y[NS];
    for (int n = 0; n < NS; ++n) Y[n] = S(i, j, k, UFS + n) * rhoInv;
    int iters = 0;
    bool ok = true;
    eos.REY2T(S(i, j, k, URHO), e, Y, T, iters, ok);
    if (!ok) {
#pragma omp atomic
      fails += 1;
    }
    S(i, j, k, UTEMP) = T;
  });
}

// MultiFab::LinComb: dst = a x + b y on vbox, NVAR components.
inline void lincomb(const Box& vbox, int nvar, const Arr<double>& dst, double a, const Arr<double>& x, double b,
                    const Arr<double>& y) {
  for_box(vbox, [&](int i, int j, int k) {
    for (int n = 0; n < nvar; ++n) dst(i, j, k, n) = a * x(i, j, k, n) + b * y(i, j, k, n);
  });
}

// Ghost fill of one level covering the domain: every ghost cell takes the
// value of the valid cell its index maps to (periodic wrap, foextrap clamp,
// mirror for reflecting faces with momentum sign flips).
struct FillBox {
  Box valid;
  Arr<double> S;
};
inline void fill_ghosts(const std::vector<FillBox>& boxes, const pc_geometry& g, int ng, int nvar) {
  int L[3];
  bool periodic[3];
  for (int d = 0; d < 3; ++d) {
    L[d] = g.domain_hi[d] - g.domain_lo[d] + 1;
    periodic[d] = g.bc_lo[d] == PC_BC_INTERIOR && g.bc_hi[d] == PC_BC_INTERIOR;
  }
  for (const FillBox& b : boxes) {
    const Box gb = grow(b.valid, ng);
    for_box(gb, [&](int i, int j, int k) {
      const int idx[3] = {i, j, k};
      bool inside = true;
      for (int d = 0; d < 3; ++d) inside = inside && idx[d] >= b.valid.lo[d] && idx[d] <= b.valid.hi[d];
      if (inside) return;
      int src[3];
      double sign[3] = {1.0, 1.0, 1.0};  // momentum x, y, z
      for (int d = 0; d < 3; ++d) {
        int x = idx[d];
        const int lo = g.domain_lo[d], hi = g.domain_hi[d];
        if (x < lo || x > hi) {
          const int bc = x < lo ? g.bc_lo[d] : g.bc_hi[d];
          if (periodic[d]) {
            x = x < lo ? x + L[d] : x - L[d];
          } else if (bc == PC_BC_OUTFLOW) {
            x = x < lo ? lo : hi;
          } else {
            x = x < lo ? 2 * lo - 1 - x : 2 * hi + 1 - x;
            if (bc == PC_BC_NOSLIPWALL) {
              for (int c = 0; c < 3; ++c) sign[c] = -sign[c];
            } else {
              sign[d] = -sign[d];
            }
          }
        }
        src[d] = x;
      }
      for (const FillBox& o : boxes) {
        bool in = true;
        for (int d = 0; d < 3; ++d) in = in && src[d] >= o.valid.lo[d] && src[d] <= o.valid.hi[d];
        if (!in) continue;
        for (int n = 0; n < nvar; ++n) {
          double v = o.S(src[0], src[1], src[2], n);
          if (n >= UMX && n <= UMZ) v = v * sign[n - UMX];
          b.S(i, j, k, n) = v;
        }
        break;
      }
    });
  }
}

// PeleC::estTimeStep (PeleC.cpp:839-972): pc_estdt_hydro / veldif / tempdif /
// enthdif (Timestep.H:51-237) over vbox; returns the four minima.
template <int NS, class EOS, class TRANS>
inline void est_dt(const Box& vbox, const Arr<double>& u, const EOS& eos, const TRANS& tr, const double dx[3],
                   double out[4]) {
  const double big = std::numeric_limits<double>::max();
  double dth = big, dtv = big, dtt = big, dte = big;
  for (int k = vbox.lo[2]; k <= vbox.hi[2]; ++k)
    for (int j = vbox.lo[1]; j <= vbox.hi[1]; ++j)
      for (int i = vbox.lo[0]; i <= vbox.hi[0]; ++i) {
        const double rho = u(i, j, k, URHO);
        const double rhoInv = 1.0 / rho;
        double Y[NS];
        for (int n = 0; n < NS; ++n) Y[n] = u(i, j, k, UFS + n) * rhoInv;
        const double T = u(i, j, k, UTEMP);
        double c;
        eos.RTY2Cs(rho, T, Y, c);
        for (int d = 0; d < 3; ++d) {
          const double ud = u(i, j, k, UMX + d) * rhoInv;
          dth = std::min(dth, dx[d] / (c + std::fabs(ud)));
        }
        double Dd[NS], mu, xi, lam;
        tr.transport(eos, T, rho, Y, Dd, mu, xi, lam);
        double cp, cv;
        eos.TY2CpCv(T, Y, cp, cv);
        double Dv = mu * rhoInv;
        if (Dv == 0.0) Dv = small_num();
        double Dt = lam * (rhoInv / cv);
        if (Dt == 0.0) Dt = small_num();
        const double De = lam * (rhoInv / cp);
        for (int d = 0; d < 3; ++d) {
          dtv = std::min(dtv, 0.5 * dx[d] * dx[d] / (3 * Dv));
          dtt = std::min(dtt, 0.5 * dx[d] * dx[d] / (3 * Dt));
          dte = std::min(dte, 0.5 * dx[d] * dx[d] / (3 * De));
        }
      }
  out[0] = dth;
  out[1] = dtv;
  out[2] = dtt;
  out[3] = dte;
}

}  // namespace orc
