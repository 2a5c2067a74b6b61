// ref_physics.cpp — ORACLE test infrastructure (oracle/ref_build.py): the
// bodies of the PelePhysics stand-in (ref_shim/PelePhysics.H).  PelePhysics
// is absent from the reference tree, so the equation of state and the
// transport that the compiled reference sources call are the oracle's
// restatements (pc_oracle.hpp), selected per call by pc_ref_select.  This
// is the one part of the reference-source build that stays unpinned.
#include "PelePhysics.H"

#include <stdexcept>

#include "pc_oracle.hpp"

namespace {

const pc_mol_config* g_cfg = nullptr;

int maxit() { return g_cfg->newton_max_iter > 0 ? g_cfg->newton_max_iter : 50; }
bool ideal() { return g_cfg->eos == PC_EOS_IDEAL_MIX; }

template <class F>
void with_eos(F&& f) {
  if (!g_cfg) throw std::runtime_error("pc_ref_select was not called");
  if (ideal())
    f(orc::IdealMix<PC_REF_NS>{&g_cfg->mech, maxit()});
  else
    f(orc::GammaLaw<PC_REF_NS>{&g_cfg->mech});
}

}  // namespace

void pc_ref_select(const pc_mol_config* cfg) { g_cfg = cfg; }

namespace pele {
namespace physics {
namespace eos {

using R = amrex::Real;

void RefEos::Y2WBAR(const R* Y, R& wbar) const {
  with_eos([&](const auto& e) { e.Y2WBAR(Y, wbar); });
}
// PelePhysics' REY2T takes T as the Newton guess and returns the solution;
// the oracle's iteration count and convergence flag are dropped here.
void RefEos::REY2T(R rho, R ein, const R* Y, R& T) const {
  with_eos([&](const auto& e) {
    int it = 0;
    bool ok = true;
    e.REY2T(rho, ein, Y, T, it, ok);
  });
}
void RefEos::RTY2P(R rho, R T, const R* Y, R& p) const {
  with_eos([&](const auto& e) { e.RTY2P(rho, T, Y, p); });
}
void RefEos::RTY2Cs(R rho, R T, const R* Y, R& cs) const {
  with_eos([&](const auto& e) { e.RTY2Cs(rho, T, Y, cs); });
}
void RefEos::RTY2G(R rho, R T, const R* Y, R& g) const {
  with_eos([&](const auto& e) { e.RTY2G(rho, T, Y, g); });
}
void RefEos::RTY2Cv(R, R T, const R* Y, R& cv) const {
  with_eos([&](const auto& e) {
    R cp;
    e.TY2CpCv(T, Y, cp, cv);
  });
}
void RefEos::RTY2Cp(R, R T, const R* Y, R& cp) const {
  with_eos([&](const auto& e) {
    R cv;
    e.TY2CpCv(T, Y, cp, cv);
  });
}
void RefEos::RTY2dpde_dpdre(R rho, R T, const R* Y, R& dpde, R& dpdr_e) const {
  with_eos([&](const auto& e) { e.RTY2dpde_dpdre(rho, T, Y, dpde, dpdr_e); });
}
void RefEos::RPY2Cs(R rho, R p, const R* Y, R& cs) const {
  with_eos([&](const auto& e) { e.RPY2Cs(rho, p, Y, cs); });
}
void RefEos::RYP2E(R rho, const R* Y, R p, R& ein) const {
  with_eos([&](const auto& e) { e.RYP2E(rho, Y, p, ein); });
}
// The three below serve only the EB and isothermal-wall paths, which the
// harness never takes; they are the ideal-gas relations p = rho (R/Wbar) T.
void RefEos::RYP2T(R rho, const R* Y, R p, R& T) const {
  with_eos([&](const auto& e) {
    R wbar;
    e.Y2WBAR(Y, wbar);
    T = p * wbar / (rho * orc::RU);
  });
}
void RefEos::RTY2E(R rho, R T, const R* Y, R& ein) const {
  R p;
  RTY2P(rho, T, Y, p);
  RYP2E(rho, Y, p, ein);
}
void RefEos::PYT2R(R p, const R* Y, R T, R& rho) const {
  with_eos([&](const auto& e) {
    R wbar;
    e.Y2WBAR(Y, wbar);
    rho = p * wbar / (orc::RU * T);
  });
}
void RefEos::Y2X(const R* Y, R* X) const {
  with_eos([&](const auto& e) { e.Y2X(Y, X); });
}
void RefEos::T2Hi(R T, R* h) const {
  with_eos([&](const auto& e) { e.T2Hi(T, h); });
}
void RefEos::T2Ei(R, R*) const { throw std::runtime_error("T2Ei is not used on the regular MOL path"); }

}  // namespace eos

namespace transport {

void RefTransport::transport(bool, bool, bool, bool, bool, amrex::Real T, amrex::Real rho, amrex::Real* Y,
                             amrex::Real* Ddiag, amrex::Real*, amrex::Real& mu, amrex::Real& xi,
                             amrex::Real& lam, const void*) const {
  amrex::Real scratch[PC_REF_NS];
  if (!Ddiag) Ddiag = scratch;  // a caller that wants no species coefficients
  with_eos([&](const auto& e) {
    using E = std::decay_t<decltype(e)>;
    if (g_cfg->transport == PC_TRANSPORT_SIMPLE)
      orc::SimpleTransport<PC_REF_NS, E>{&g_cfg->mech}.transport(e, T, rho, Y, Ddiag, mu, xi, lam);
    else
      orc::ConstantTransport<PC_REF_NS, E>{&g_cfg->mech}.transport(e, T, rho, Y, Ddiag, mu, xi, lam);
  });
}

}  // namespace transport
}  // namespace physics
}  // namespace pele
