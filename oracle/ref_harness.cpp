// ref_harness.cpp — ORACLE test infrastructure (oracle/ref_build.py): runs
// PeleC's OWN hot-path source code, compiled where it lies in the reference
// tree, on one regular box at a time, so that the tests can pin the oracle's
// restatement (pc_oracle.hpp) to it bit for bit.
//
// Compiled from the reference (unchanged, by #include through the include
// path; ref_shim/ stands in for AMReX and PelePhysics, which are absent):
//   Source/MOL.cpp        pc_compute_hyp_mol_flux (:5-204), with mol_slope
//                         (MOL.H:28-113), riemann (Riemann.H:6-200) and
//                         laxfriedrich_flux (Riemann.H:202-307)
//   Source/Diffterm.H     pc_diffusion_flux (:344-461), SpeciesEnergyFlux
//                         (:20-75), pc_flux_div (:463-484)
//   Source/Utilities.H    pc_ctoprim (:239-320), pc_move_transcoefs_to_ec
//                         (:322-342), setV / setC / copy_array4
//   Source/TransCoeff.H   pc_transcoeff (:7-37)
//   Source/Timestep.H     pc_estdt_hydro / veldif / tempdif / enthdif
//                         (:48-237), the cell limits of estTimeStep
//   Source/Utilities.H    pc_rst_int_e (:86-237) and pc_cmpTemp (:67-84),
//                         the cell updates of computeTemp
// Written here (the driver): the regular-box body of getMOLSrcTerm
// (Diffusion.cpp:85-145, 180-369, 530-541, 672) with its MFIter, MultiFab
// and EB-factory plumbing replaced by plain arrays — the same calls in the
// same order.  The EOS and transport behind the reference's calls are the
// oracle's (ref_physics.cpp): PelePhysics stays unpinned.
#include "pelec_mol.h"

#include "MOL.cpp"
#include "Diffterm.H"
#include "Timestep.H"

ProbParmDevice* PeleC::d_prob_parm_device = nullptr;

void pc_ref_select(const pc_mol_config* cfg);

namespace {

template <class T>
amrex::Array4<T> view(const pc_array4& a) {
  amrex::Array4<T> v;
  v.p = reinterpret_cast<decltype(v.p)>(a.p);  // the counting build's Real is one double wide
  v.jstride = a.jstride;
  v.kstride = a.kstride;
  v.nstride = a.nstride;
  v.begin = amrex::Dim3{a.begin[0], a.begin[1], a.begin[2]};
  v.end = amrex::Dim3{a.end[0], a.end[1], a.end[2]};
  v.ncomp = a.ncomp;
  return v;
}

bool covers(const pc_array4& a, const amrex::Box& b) {
  for (int d = 0; d < 3; ++d)
    if (a.begin[d] > b.lo[d] || a.end[d] - 1 < b.hi[d]) return false;
  return true;
}

// One box of getMOLSrcTerm's MFIter loop, regular cells, no rotating frame,
// no isothermal walls, no LES filter.  fluxes (optional) receives flx on
// surroundingNodes(vbox, dir): the flux_ec data update_flux_registers gets.
int mol_rhs_box(const pc_mol_config& cfg, const pc_box_desc& bd, const double dx[3], const pc_array4* fluxes) {
  const amrex::Box vbox(amrex::IntVect(bd.lo[0], bd.lo[1], bd.lo[2]), amrex::IntVect(bd.hi[0], bd.hi[1], bd.hi[2]));
  const int ng = 4;  // PeleC::numGrow() without EB (PeleC.H:877-900)
  const amrex::Box gbox = amrex::grow(vbox, ng);
  const amrex::Box cbox = amrex::grow(vbox, ng - 1);
  if (!covers(bd.state, gbox) || !covers(bd.rhs, vbox)) return PC_ERR_INVALID_ARGUMENT;
  if (bd.state.ncomp < NVAR || bd.rhs.ncomp < NVAR) return PC_ERR_INVALID_ARGUMENT;
  auto const MOLSrc = view<amrex::Real>(bd.rhs);
  if (!cfg.diffuse_temp && !cfg.diffuse_enth && !cfg.diffuse_spec && !cfg.diffuse_vel && !cfg.do_hydro) {
    setV(vbox, NVAR, MOLSrc, 0.0);  // Diffusion.cpp:13-18
    return PC_OK;
  }
  amrex::Geometry geom;
  for (int d = 0; d < 3; ++d) geom.gd.dx[d] = dx[d];
  const amrex::GpuArray<amrex::Real, AMREX_SPACEDIM> dxinv = geom.InvCellSizeArray();
  const int nCompTr = dComp_lambda + 1;

  amrex::FArrayBox q(gbox, QVAR), qaux(gbox, NQAUX), coeff_cc(gbox, nCompTr);
  auto const sar = view<const amrex::Real>(bd.state);
  auto const qar = q.array();
  auto const qauxar = qaux.array();
  amrex::ParallelFor(gbox, [=](int i, int j, int k) { pc_ctoprim(i, j, k, sar, qar, qauxar); });

  // Transport coefficients on gbox (Diffusion.cpp:180-220).
  auto const coe_cc = coeff_cc.array();
  {
    auto const qar_yin = q.array(QFS);
    auto const qar_Tin = q.array(QTEMP);
    auto const qar_rhoin = q.array(QRHO);
    auto const coe_rhoD = coeff_cc.array(dComp_rhoD);
    auto const coe_mu = coeff_cc.array(dComp_mu);
    auto const coe_xi = coeff_cc.array(dComp_xi);
    auto const coe_lambda = coeff_cc.array(dComp_lambda);
    const pele::physics::transport::TransParm<pele::physics::PhysicsType::eos_type,
                                              pele::physics::PhysicsType::transport_type>* ltransparm = nullptr;
    const auto geomdata = geom.data();
    const ProbParmDevice lprobparm{};
    const bool get_xi = true, get_mu = true, get_lam = true, get_Ddiag = true, get_chi = false;
    amrex::ParallelFor(gbox, [=](int i, int j, int k) {
      amrex::Real muloc, xiloc, lamloc;
      amrex::Real Ddiag[NUM_SPECIES], Y[NUM_SPECIES] = {0.0};
      amrex::Real* chi_mix = nullptr;
      amrex::Real T = qar_Tin(i, j, k);
      amrex::Real rho = qar_rhoin(i, j, k);
      for (int n = 0; n < NUM_SPECIES; ++n) Y[n] = qar_yin(i, j, k, n);
      const amrex::RealVect x = pc_cmp_loc({i, j, k}, geomdata);
      pc_transcoeff(get_xi, get_mu, get_lam, get_Ddiag, get_chi, T, rho, Y, Ddiag, chi_mix, muloc, xiloc, lamloc,
                    ltransparm, lprobparm, x);
      for (int n = 0; n < NUM_SPECIES; ++n) coe_rhoD(i, j, k, n) = Ddiag[n];
      coe_mu(i, j, k) = muloc;
      coe_xi(i, j, k) = xiloc;
      coe_lambda(i, j, k) = lamloc;
    });
  }

  // Face-area and volume arrays: Cartesian metrics (PeleC.cpp:593-604).
  amrex::FArrayBox flux_ec[AMREX_SPACEDIM], area_fab[AMREX_SPACEDIM];
  const amrex::Box eboxes[AMREX_SPACEDIM] = {amrex::surroundingNodes(cbox, 0), amrex::surroundingNodes(cbox, 1),
                                             amrex::surroundingNodes(cbox, 2)};
  const amrex::Real face_area[3] = {dx[1] * dx[2], dx[0] * dx[2], dx[0] * dx[1]};
  amrex::GpuArray<amrex::Array4<amrex::Real>, AMREX_SPACEDIM> flx;
  for (int dir = 0; dir < AMREX_SPACEDIM; dir++) {
    flux_ec[dir].resize(eboxes[dir], NVAR);
    flx[dir] = flux_ec[dir].array();
    setV(eboxes[dir], NVAR, flx[dir], 0);
    area_fab[dir].resize(eboxes[dir], 1);
    setV(eboxes[dir], 1, area_fab[dir].array(), face_area[dir]);
  }
  const amrex::GpuArray<const amrex::Array4<const amrex::Real>, AMREX_SPACEDIM> area_arr{
      {area_fab[0].array(), area_fab[1].array(), area_fab[2].array()}};
  amrex::FArrayBox vol_fab(cbox, 1);
  setV(cbox, 1, vol_fab.array(), dx[0] * dx[1] * dx[2]);

  amrex::FArrayBox Dfab(cbox, NVAR);
  auto const Dterm = Dfab.array();
  setV(cbox, NVAR, Dterm, 0.0);
  const amrex::Array4<amrex::EBCellFlag const> flag_arr{};

  // Diffusion fluxes (Diffusion.cpp:222-252, regular boxes).
  {
    const bool l_transport_harmonic_mean = cfg.transport_harmonic_mean != 0;
    for (int dir = 0; dir < AMREX_SPACEDIM; dir++) {
      amrex::ParallelFor(eboxes[dir], [=](int i, int j, int k) {
        amrex::GpuArray<amrex::Real, dComp_lambda + 1> cf = {0.0};
        if (flag_arr(i, j, k).isRegular() || flag_arr(i, j, k).isSingleValued()) {
          for (int n = 0; n < static_cast<int>(cf.size()); n++)
            pc_move_transcoefs_to_ec(i, j, k, n, coe_cc, cf.data(), dir, l_transport_harmonic_mean);
        }
        pc_diffusion_flux(i, j, k, qar, cf, area_arr[dir], flx[dir], dxinv, dir);
      });
    }
  }
  // Switched-off diffusion (Diffusion.cpp:321-341).
  if (!cfg.diffuse_temp && !cfg.diffuse_enth)
    for (int dir = 0; dir < AMREX_SPACEDIM; dir++) setC(eboxes[dir], UEDEN, UEINT, flx[dir], 0.0);
  if (!cfg.diffuse_spec)
    for (int dir = 0; dir < AMREX_SPACEDIM; dir++) setC(eboxes[dir], UFS, UFS + NUM_SPECIES, flx[dir], 0.0);
  if (!cfg.diffuse_vel)
    for (int dir = 0; dir < AMREX_SPACEDIM; dir++) setC(eboxes[dir], UMX, UMX + 3, flx[dir], 0.0);

  // Hyperbolic MOL fluxes (Diffusion.cpp:344-369).
  if (cfg.do_hydro) {
    const amrex::GpuArray<amrex::Real, AMREX_SPACEDIM> axis_loc = {{0.0, 0.0, 0.0}};
    pc_compute_hyp_mol_flux(cbox, qar, qauxar, flx, area_arr, cfg.plm_iorder, cfg.use_laxf_flux != 0, flag_arr,
                            geom, axis_loc, 0.0, 0, false);
  }

  // Divergence on cbox (Diffusion.cpp:530-541), copy on vbox (:672).
  {
    auto const vol = vol_fab.array();
    amrex::ParallelFor(cbox, NVAR, [=](int i, int j, int k, int n) {
      pc_flux_div(i, j, k, n, flx[0], flx[1], flx[2], vol, Dterm);
    });
  }
  if (fluxes) {
    for (int dir = 0; dir < 3; ++dir) {
      if (!covers(fluxes[dir], amrex::surroundingNodes(vbox, dir)) || fluxes[dir].ncomp < NVAR)
        return PC_ERR_INVALID_ARGUMENT;
      copy_array4(amrex::surroundingNodes(vbox, dir), NVAR, flx[dir], view<amrex::Real>(fluxes[dir]));
    }
  }
  copy_array4(vbox, NVAR, Dterm, MOLSrc);
  return PC_OK;
}

}  // namespace

extern "C" {

// NUM_SPECIES of this build.
int ref_nspec(void) { return NUM_SPECIES; }

// The regular-box body of getMOLSrcTerm for each box (host arrays);
// fluxes, when not NULL, holds 3 arrays per box (surroundingNodes(valid, d)).
int ref_mol_rhs(const pc_mol_config* cfg, const pc_box_desc* boxes, int nboxes, const double dx[3],
                const pc_array4* fluxes) {
  if (!cfg || !boxes || nboxes < 0 || !dx) return PC_ERR_INVALID_ARGUMENT;
  if (cfg->nspec != NUM_SPECIES) return PC_ERR_UNSUPPORTED;
  pc_ref_select(cfg);
  for (int b = 0; b < nboxes; ++b) {
    const int rc = mol_rhs_box(*cfg, boxes[b], dx, fluxes ? fluxes + 3 * b : nullptr);
    if (rc != PC_OK) return rc;
  }
  return PC_OK;
}

#ifdef PC_COUNT_FLOPS
// The arithmetic of ref_mol_rhs on the boxes, counted by class
// (flop_count.hpp): out = [add, mul, div, fma, sqrt, exp, log, pow, cmp].
int ref_count_mol_rhs(const pc_mol_config* cfg, const pc_box_desc* boxes, int nboxes, const double dx[3],
                      unsigned long long* out) {
  pcc::tally() = pcc::Tally{};
  const int rc = ref_mol_rhs(cfg, boxes, nboxes, dx, nullptr);
  const pcc::Tally& t = pcc::tally();
  const unsigned long long v[9] = {t.add, t.mul, t.div, t.fma, t.sqrt, t.exp, t.log, t.pow, t.cmp};
  for (int q = 0; q < 9; ++q) out[q] = v[q];
  return rc;
}
#else
// pc_ctoprim on one cell: U[NVAR] -> q[QVAR], qaux[NQAUX].
int ref_ctoprim_cell(const pc_mol_config* cfg, const double* U, double* qv, double* qa) {
  if (cfg->nspec != NUM_SPECIES) return PC_ERR_UNSUPPORTED;
  pc_ref_select(cfg);
  const amrex::Array4<const amrex::Real> u(U, amrex::Dim3{0, 0, 0}, amrex::Dim3{1, 1, 1}, NVAR);
  const amrex::Array4<amrex::Real> q(qv, amrex::Dim3{0, 0, 0}, amrex::Dim3{1, 1, 1}, QVAR);
  const amrex::Array4<amrex::Real> x(qa, amrex::Dim3{0, 0, 0}, amrex::Dim3{1, 1, 1}, NQAUX);
  pc_ctoprim(0, 0, 0, u, q, x);
  return PC_OK;
}

// riemann() (laxf = 0) or laxfriedrich_flux() (laxf = 1) on one face:
// left/right = [rho, un, ut1, ut2, p, Y(NUM_SPECIES)] -> flux[NVAR] in the x
// direction's component order (UTEMP slot 0), ustar.
int ref_riemann_face(const pc_mol_config* cfg, int laxf, const double* l, const double* r, double cav, double* flux,
                     double* ustar) {
  if (cfg->nspec != NUM_SPECIES) return PC_ERR_UNSUPPORTED;
  pc_ref_select(cfg);
  for (int n = 0; n < NVAR; ++n) flux[n] = 0.0;
  *ustar = 0.0;
  if (!laxf) {
    amrex::Real qint_iu = 0.0, tmp1 = 0.0, tmp2 = 0.0, tmp3 = 0.0, tmp4 = 0.0;
    riemann(l[0], l[1], l[2], l[3], l[4], l + 5, r[0], r[1], r[2], r[3], r[4], r + 5, 1, cav, *ustar, flux[URHO],
            &flux[UFS], flux[UMX], flux[UMY], flux[UMZ], flux[UEDEN], flux[UEINT], qint_iu, tmp1, tmp2, tmp3, tmp4);
  } else {
    amrex::Real maxeigval = 0.0;
    laxfriedrich_flux(l[0], l[1], l[2], l[3], l[4], l + 5, r[0], r[1], r[2], r[3], r[4], r + 5, 1, cav, *ustar,
                      maxeigval, flux[URHO], &flux[UFS], flux[UMX], flux[UMY], flux[UMZ], flux[UEDEN],
                      flux[UEINT]);
  }
  return PC_OK;
}

// PeleC::computeTemp on each box's valid cells (PeleC.cpp:2187-2271):
// reset_internal_energy with the default flags (pelec_defaults.H:36-39), then
// pc_cmpTemp.  lohi: 6 ints per box.
int ref_compute_temp(const pc_mol_config* cfg, int nboxes, const int* lohi, const pc_array4* st) {
  if (cfg->nspec != NUM_SPECIES) return PC_ERR_UNSUPPORTED;
  pc_ref_select(cfg);
  const bool allow_small_energy = true, allow_negative_energy = true, dual_energy_update_E_from_e = true;
  const amrex::Real dual_energy_eta2 = 1.0e-4;
  for (int b = 0; b < nboxes; ++b) {
    const amrex::Box vbox(amrex::IntVect(lohi[6 * b], lohi[6 * b + 1], lohi[6 * b + 2]),
                          amrex::IntVect(lohi[6 * b + 3], lohi[6 * b + 4], lohi[6 * b + 5]));
    auto const S = view<amrex::Real>(st[b]);
    amrex::ParallelFor(vbox, [=](int i, int j, int k) {
      pc_rst_int_e(i, j, k, S, allow_small_energy, allow_negative_energy, dual_energy_update_E_from_e,
                   dual_energy_eta2);
    });
    amrex::ParallelFor(vbox, [=](int i, int j, int k) { pc_cmpTemp(i, j, k, S); });
  }
  return PC_OK;
}

// The four cell-limit minima of PeleC::estTimeStep over the boxes' valid
// cells (PeleC.cpp:839-972 calls these per box): parts = [hydro, veldif,
// tempdif, enthdif].
int ref_est_dt_parts(const pc_mol_config* cfg, const pc_box_desc* boxes, int nboxes, const double dx[3],
                     double* parts) {
  if (cfg->nspec != NUM_SPECIES) return PC_ERR_UNSUPPORTED;
  pc_ref_select(cfg);
  amrex::GeometryData gd;
  for (int d = 0; d < 3; ++d) gd.dx[d] = dx[d];
  const ProbParmDevice prob_parm{};
  const pele::physics::transport::TransParm<pele::physics::PhysicsType::eos_type,
                                            pele::physics::PhysicsType::transport_type>* tp = nullptr;
  const amrex::Array4<const amrex::EBCellFlag> flags{};
  for (int q = 0; q < 4; ++q) parts[q] = std::numeric_limits<amrex::Real>::max();
  for (int b = 0; b < nboxes; ++b) {
    const amrex::Box vbox(amrex::IntVect(boxes[b].lo[0], boxes[b].lo[1], boxes[b].lo[2]),
                          amrex::IntVect(boxes[b].hi[0], boxes[b].hi[1], boxes[b].hi[2]));
    auto const u = view<const amrex::Real>(boxes[b].state);
    parts[0] = amrex::min(parts[0], pc_estdt_hydro(vbox, u, flags, dx[0], dx[1], dx[2]));
    parts[1] = amrex::min(parts[1], pc_estdt_veldif(vbox, u, flags, gd, tp, prob_parm));
    parts[2] = amrex::min(parts[2], pc_estdt_tempdif(vbox, u, flags, gd, tp, prob_parm));
    parts[3] = amrex::min(parts[3], pc_estdt_enthdif(vbox, u, flags, gd, tp, prob_parm));
  }
  return PC_OK;
}
#endif  // PC_COUNT_FLOPS

}  // extern "C"
