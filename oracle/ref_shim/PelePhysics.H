// PelePhysics.H — ORACLE test infrastructure: the PelePhysics interface that
// PeleC's hot-path headers call (the EOS functor, the transport functor and
// their parameter types), for compiling those reference sources unchanged
// (oracle/ref_build.py).  PelePhysics is absent from the reference tree, so
// every method forwards to the oracle's own restatement of the equation of
// state and the transport (oracle/pc_oracle.hpp, through ref_physics.cpp)
// under the configuration that the harness selects before each call.  The
// call sites this interface serves: Source/Utilities.H:67-84, 239-320;
// Source/Riemann.H:44-178, 237-255; Source/Diffterm.H:32-52;
// Source/TransCoeff.H:29-33; Source/MOL.cpp:259-273; Source/Timestep.H:17-239.
#pragma once

#include "amrex_shim.H"
#include "mechanism.H"

namespace pele {
namespace physics {

namespace Constants {
// Universal gas constant, erg/(mol K); the oracle uses the same value.
constexpr amrex::Real RU = 8.31446261815324e7;
}  // namespace Constants

namespace eos {

// The EOS of the configuration selected by pc_ref_select (GammaLaw or the
// NASA-7 ideal mixture, as pc_mol_config.eos says).
struct RefEos {
  void Y2WBAR(const amrex::Real* Y, amrex::Real& wbar) const;
  void REY2T(amrex::Real rho, amrex::Real e, const amrex::Real* Y, amrex::Real& T) const;
  void RTY2P(amrex::Real rho, amrex::Real T, const amrex::Real* Y, amrex::Real& p) const;
  void RTY2Cs(amrex::Real rho, amrex::Real T, const amrex::Real* Y, amrex::Real& cs) const;
  void RTY2G(amrex::Real rho, amrex::Real T, const amrex::Real* Y, amrex::Real& g) const;
  void RTY2Cv(amrex::Real rho, amrex::Real T, const amrex::Real* Y, amrex::Real& cv) const;
  void RTY2Cp(amrex::Real rho, amrex::Real T, const amrex::Real* Y, amrex::Real& cp) const;
  void RTY2dpde_dpdre(amrex::Real rho, amrex::Real T, const amrex::Real* Y, amrex::Real& dpde,
                      amrex::Real& dpdr_e) const;
  void RPY2Cs(amrex::Real rho, amrex::Real p, const amrex::Real* Y, amrex::Real& cs) const;
  void RYP2E(amrex::Real rho, const amrex::Real* Y, amrex::Real p, amrex::Real& e) const;
  void RYP2T(amrex::Real rho, const amrex::Real* Y, amrex::Real p, amrex::Real& T) const;
  void RTY2E(amrex::Real rho, amrex::Real T, const amrex::Real* Y, amrex::Real& e) const;
  void PYT2R(amrex::Real p, const amrex::Real* Y, amrex::Real T, amrex::Real& rho) const;
  void Y2X(const amrex::Real* Y, amrex::Real* X) const;
  void T2Hi(amrex::Real T, amrex::Real* h) const;
  void T2Ei(amrex::Real T, amrex::Real* e) const;
};

// Soave-Redlich-Kwong: only named by the reference's explicit
// specialisation SpeciesEnergyFlux<SRK> (Diffterm.H:77-154), never used.
struct SRK {
  void Y2X(const amrex::Real* Y, amrex::Real* X) const;
  void RTY2transport(amrex::Real rho, amrex::Real T, const amrex::Real* Y, amrex::Real* diP,
                     amrex::Real (*dijY)[NUM_SPECIES]) const;
  void RTY2Hi(amrex::Real rho, amrex::Real T, const amrex::Real* Y, amrex::Real* h) const;
};

}  // namespace eos

using EosType = eos::RefEos;

namespace transport {

template <class EOS, class TRANSPORT>
struct TransParm {};

// The transport of the selected configuration (constant or mixture-averaged,
// as pc_mol_config.transport says).  The get_* switches are always all on in
// getMOLSrcTerm's call (Diffusion.cpp:190-191); estTimeStep's
// (Timestep.H:17-46) asks for one coefficient and passes no Ddiag array.
struct RefTransport {
  void transport(bool get_xi, bool get_mu, bool get_lam, bool get_Ddiag, bool get_chi, amrex::Real T,
                 amrex::Real rho, amrex::Real* Y, amrex::Real* Ddiag, amrex::Real* chi_mix, amrex::Real& mu,
                 amrex::Real& xi, amrex::Real& lam, const void* tparm) const;
};

}  // namespace transport

struct PhysicsType {
  using eos_type = eos::RefEos;
  using transport_type = transport::RefTransport;
  static eos_type eos() { return {}; }
  static transport_type transport() { return {}; }
};

}  // namespace physics
}  // namespace pele
