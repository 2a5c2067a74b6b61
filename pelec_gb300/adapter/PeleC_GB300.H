// PeleC_GB300.H — the reference-side adapter: what a PeleC maintainer adds to
// Source/Diffusion.cpp so that PeleC::getMOLSrcTerm (Source/PeleC.H:523-528,
// Source/Diffusion.cpp:4-681) runs its regular (non-EB) levels through the
// GB300 library (include/pelec_mol.h), with the signature and every caller
// (Source/Advance.cpp:100, :134, :180, :298, :336) unchanged.
//
// Usage inside Diffusion.cpp (a level whose boxes are all regular):
//
//   #include "PeleC_GB300.H"
//   void PeleC::getMOLSrcTerm(const amrex::MultiFab& S, amrex::MultiFab& MOLSrcTerm,
//                             amrex::Real /*time*/, amrex::Real dt, amrex::Real reflux_factor)
//   {
//     if (!diffuse_temp && !diffuse_enth && !diffuse_spec && !diffuse_vel && !do_hydro) {
//       MOLSrcTerm.setVal(0, 0, NVAR, MOLSrcTerm.nGrow());      // Diffusion.cpp:13-18
//       return;
//     }
//     static pc_mol_handle* h = pc_gb300::handle(pc_gb300::flags_config(
//         do_hydro, diffuse_vel, diffuse_temp, diffuse_spec, diffuse_enth, plm_iorder,
//         use_laxf_flux, transport_harmonic_mean));
//     const bool reflux = do_reflux && reflux_factor != 0;     // Diffusion.cpp:653
//     amrex::FArrayBox dm_as_fine;                              // unused on regular boxes
//     pc_gb300::mol_src_term(h, S, MOLSrcTerm, geom, reflux,
//         [&](const amrex::MFIter& mfi, const std::array<amrex::FArrayBox const*, 3>& flux) {
//           update_flux_registers(reflux_factor * dt, mfi, amrex::FabType::regular, flux, dm_as_fine);
//         });
//   }
//
// The EOS and transport models are chosen when PeleC is compiled
// (Exec/Make.PeleC:74-115); set PC_GB300_EOS / PC_GB300_TRANSPORT to the
// pc_eos_kind / pc_transport_kind that match them (defaults: the ideal-gas
// mixture and mixture-averaged "Simple" transport).
#pragma once

#include <array>
#include <cmath>
#include <vector>

#include <AMReX_FArrayBox.H>
#include <AMReX_Geometry.H>
#include <AMReX_MultiFab.H>

#include "PelePhysics.H"
#include "mechanism.H"
#include "pelec_mol.h"

#ifndef PC_GB300_EOS
#define PC_GB300_EOS PC_EOS_IDEAL_MIX
#endif
#ifndef PC_GB300_TRANSPORT
#define PC_GB300_TRANSPORT PC_TRANSPORT_SIMPLE
#endif

namespace pc_gb300 {

// ---------------------------------------------------------------------------
// Mechanism data: the compiled PelePhysics mechanism restated as
// pc_mechanism.  PelePhysics' generated mechanism.H exposes its NASA-7
// thermodynamics only through evaluation functions, so the coefficients are
// recovered from them exactly: cp/R is a quartic in T on each range, so five
// samples per range (Chebyshev nodes, T scaled by 1000 K) determine a0..a4,
// and h/(RT) - (a0 + a1 T/2 + ... + a4 T^4/5) = a5 / T gives a5.  Entry
// points used (Fuego-generated mechanism.H): get_mw(mw) in g/mol;
// cp_R(cp, tc) and speciesEnthalpy(hRT, tc) with tc = {ln T, T, T^2, T^3,
// T^4}.  The range split is the CHEMKIN common temperature, 1000 K, for every
// species; recover_range checks the recovered polynomials against fresh
// samples and fails if a species uses another split.
//
// Transport ("Simple" mixture-averaged, called from Source/TransCoeff.H:29-33
// as trans.transport(..., tparm)): the pure-species fits of TransParm,
// ln(q) = sum_{n<4} c_n (ln T)^n, for the viscosity (g/cm/s, fitmu), the
// conductivity (erg/cm/s/K, fitlam) and the binary diffusion coefficients
// (cm^2/s at 1 atm, fitdbin, symmetric); four coefficients per fit
// (TransParm's NUM_FIT), T in K.  The bulk viscosity is taken as zero
// (bulk_ratio = 0) unless the caller sets it.
// ---------------------------------------------------------------------------
constexpr double kTmid = 1000.0;
constexpr double kTlo = 300.0, kThi = 3500.0;

inline void tc_of(double T, double tc[5]) {
  tc[0] = std::log(T);
  tc[1] = T;
  tc[2] = T * T;
  tc[3] = T * T * T;
  tc[4] = T * T * T * T;
}

// a[0..4] from cp/R at 5 points of [t0, t1] (Gaussian elimination with
// partial pivoting on the scaled Vandermonde system), a[5] from h/RT.
template <int NS>
bool recover_range(double t0, double t1, int k, double a[7]) {
  double T[5], A[5][6];
  for (int i = 0; i < 5; ++i) {
    T[i] = 0.5 * (t0 + t1) + 0.5 * (t1 - t0) * std::cos(3.14159265358979323846 * (2 * i + 1) / 10.0);
    double tc[5], cp[NS];
    tc_of(T[i], tc);
    cp_R(cp, tc);
    const double x = T[i] / 1000.0;
    double p = 1.0;
    for (int n = 0; n < 5; ++n, p *= x) A[i][n] = p;
    A[i][5] = cp[k];
  }
  for (int c = 0; c < 5; ++c) {
    int piv = c;
    for (int r = c + 1; r < 5; ++r)
      if (std::fabs(A[r][c]) > std::fabs(A[piv][c])) piv = r;
    for (int n = 0; n < 6; ++n) std::swap(A[c][n], A[piv][n]);
    for (int r = 0; r < 5; ++r) {
      if (r == c) continue;
      const double f = A[r][c] / A[c][c];
      for (int n = c; n < 6; ++n) A[r][n] -= f * A[c][n];
    }
  }
  double s = 1.0;
  for (int n = 0; n < 5; ++n, s *= 1000.0) a[n] = A[n][5] / A[n][n] / s;
  double a5 = 0.0;
  for (int i = 0; i < 5; ++i) {
    double tc[5], h[NS];
    tc_of(T[i], tc);
    speciesEnthalpy(h, tc);
    const double t = T[i];
    const double poly = a[0] + t * (a[1] / 2 + t * (a[2] / 3 + t * (a[3] / 4 + t * a[4] / 5)));
    a5 += (h[k] - poly) * t;
  }
  a[5] = a5 / 5.0;
  a[6] = 0.0;  // the entropy constant: not used by the MOL right-hand side
  // the quartic must reproduce cp/R at points between the nodes
  for (double u : {0.13, 0.51, 0.87}) {
    const double t = t0 + u * (t1 - t0);
    double tc[5], cp[NS];
    tc_of(t, tc);
    cp_R(cp, tc);
    const double q = a[0] + t * (a[1] + t * (a[2] + t * (a[3] + t * a[4])));
    if (!(std::fabs(q - cp[k]) <= 1e-9 * std::fabs(cp[k]))) return false;
  }
  return true;
}

// Fills m's species thermodynamics from the compiled mechanism
// (NUM_SPECIES <= PC_MAX_SPECIES).  Returns PC_OK, or PC_ERR_UNSUPPORTED for
// a mechanism this library has no kernels for.
// With the GammaLaw EOS only the molecular weights are read: the caller sets
// m.gamma (eos.gamma) and, for constant transport, m.const_mu, const_xi,
// const_lambda and const_rhoD (the transport.const_* parameters).
inline int fill_mechanism(pc_mechanism& m) {
  constexpr int NS = NUM_SPECIES;
  if (NS > PC_MAX_SPECIES) return PC_ERR_UNSUPPORTED;
  m = pc_mechanism{};
  m.nspec = NS;
  double mw[NS];
  get_mw(mw);
  for (int k = 0; k < NS; ++k) {
    m.mw[k] = mw[k];
    if (PC_GB300_EOS == PC_EOS_GAMMA_LAW) continue;
    m.nasa_tmid[k] = kTmid;
    if (!recover_range<NS>(kTlo, kTmid, k, m.nasa_lo[k]) || !recover_range<NS>(kTmid, kThi, k, m.nasa_hi[k]))
      return PC_ERR_UNSUPPORTED;
  }
  m.diff_pref = 1013250.0;  // the binary fits are at 1 atm
  return PC_OK;
}

// ... and the Simple transport's fits from a TransParm (host copy).
template <class TransParmT>
int fill_mechanism(pc_mechanism& m, const TransParmT& tp) {
  const int rc = fill_mechanism(m);
  if (rc != PC_OK) return rc;
  constexpr int NS = NUM_SPECIES, NF = 4;
  for (int k = 0; k < NS; ++k)
    for (int n = 0; n < NF; ++n) {
      m.visc_fit[k][n] = tp.fitmu[k * NF + n];
      m.cond_fit[k][n] = tp.fitlam[k * NF + n];
      for (int j = 0; j < NS; ++j) m.diff_fit[k][j][n] = tp.fitdbin[(k * NS + j) * NF + n];
    }
  return PC_OK;
}

inline pc_mol_config flags_config(int do_hydro, int diffuse_vel, int diffuse_temp, int diffuse_spec,
                                  int diffuse_enth, int plm_iorder, int use_laxf_flux, int harmonic_mean) {
  pc_mol_config c{};
  c.nspec = NUM_SPECIES;
  c.eos = PC_GB300_EOS;
  c.transport = PC_GB300_TRANSPORT;
  c.precision = PC_PRECISION_FP64;
  c.do_hydro = do_hydro;
  c.diffuse_vel = diffuse_vel;
  c.diffuse_temp = diffuse_temp;
  c.diffuse_spec = diffuse_spec;
  c.diffuse_enth = diffuse_enth;
  c.plm_iorder = plm_iorder;
  c.use_laxf_flux = use_laxf_flux;
  c.transport_harmonic_mean = harmonic_mean;
  c.check_output = 1;
  return c;
}

// A handle for cfg with the compiled mechanism's data (and the Simple
// transport parameters, from PeleC's trans_parms host copy, when given).
// Aborts as getMOLSrcTerm does on an unsupported case (Diffusion.cpp:272).
inline pc_mol_handle* create_or_abort(pc_mol_config& cfg, int rc) {
  pc_mol_handle* h = nullptr;
  if (rc == PC_OK) rc = pc_mol_create(&h, &cfg);
  if (rc != PC_OK) amrex::Abort(pc_mol_error_string(rc));
  return h;
}
inline pc_mol_handle* handle(pc_mol_config cfg) { return create_or_abort(cfg, fill_mechanism(cfg.mech)); }
template <class TransParmT>
pc_mol_handle* handle(pc_mol_config cfg, const TransParmT& tp) {
  return create_or_abort(cfg, fill_mechanism(cfg.mech, tp));
}

// An amrex::Array4 as the ABI's pc_array4 (AMReX_Array4.H: p, jstride,
// kstride, nstride, begin, end, ncomp).
template <class T>
pc_array4 to_pc(const amrex::Array4<T>& a) {
  pc_array4 r{};
  r.p = const_cast<double*>(a.p);
  r.jstride = a.jstride;
  r.kstride = a.kstride;
  r.nstride = a.nstride;
  r.begin[0] = a.begin.x;
  r.begin[1] = a.begin.y;
  r.begin[2] = a.begin.z;
  r.end[0] = a.end.x;
  r.end[1] = a.end.y;
  r.end[2] = a.end.z;
  r.ncomp = a.ncomp;
  return r;
}

// The MFIter loop of getMOLSrcTerm (Diffusion.cpp:85-679) on regular boxes:
// one library call per level.  With want_fluxes, the face fluxes of every
// box (flux_ec of Diffusion.cpp:222-232, times the face areas, on
// surroundingNodes of the box) are computed in the same call and handed to
// sink(mfi, {fx, fy, fz}) box by box, as update_flux_registers receives them
// (Diffusion.cpp:667-670).
template <class Sink>
void mol_src_term(pc_mol_handle* h, const amrex::MultiFab& S, amrex::MultiFab& MOLSrcTerm,
                  const amrex::Geometry& geom, bool want_fluxes, Sink&& sink) {
  std::vector<pc_box_desc> boxes;
  std::vector<pc_array4> fx;
  std::vector<std::array<amrex::FArrayBox, 3>> flux;
  if (want_fluxes) flux.resize(MOLSrcTerm.local_size());
  for (amrex::MFIter mfi(MOLSrcTerm, false); mfi.isValid(); ++mfi) {
    const amrex::Box vbox = mfi.validbox();
    pc_box_desc b{};
    for (int d = 0; d < 3; ++d) {
      b.lo[d] = vbox.smallEnd(d);
      b.hi[d] = vbox.bigEnd(d);
    }
    b.state = to_pc(S.const_array(mfi));
    b.rhs = to_pc(MOLSrcTerm.array(mfi));
    boxes.push_back(b);
    if (want_fluxes)
      for (int d = 0; d < 3; ++d) {
        amrex::FArrayBox& f = flux[mfi.LocalIndex()][d];
        f.resize(amrex::surroundingNodes(vbox, d), MOLSrcTerm.nComp(), amrex::The_Async_Arena());
        fx.push_back(to_pc(f.array()));
      }
  }
  const auto dx = geom.CellSizeArray();
  const double dxv[3] = {dx[0], dx[1], dx[2]};
  void* stream = static_cast<void*>(amrex::Gpu::gpuStream());
  const int rc = want_fluxes ? pc_mol_rhs_level_fluxes(h, boxes.data(), (int)boxes.size(), dxv, fx.data(), stream)
                             : pc_mol_rhs_level(h, boxes.data(), (int)boxes.size(), dxv, stream);
  if (rc != PC_OK) amrex::Abort(pc_mol_error_string(rc));
  if (want_fluxes)
    for (amrex::MFIter mfi(MOLSrcTerm, false); mfi.isValid(); ++mfi) {
      auto& f = flux[mfi.LocalIndex()];
      sink(mfi, std::array<amrex::FArrayBox const*, 3>{&f[0], &f[1], &f[2]});
    }
}

}  // namespace pc_gb300
