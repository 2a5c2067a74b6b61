// adapter_driver.cpp — test program of tests/test_adapter.py: compiles the
// PeleC adapter (pelec_gb300/adapter/PeleC_GB300.H) against the stand-ins in
// this directory, links libpelec_mol.so, and prints what the test checks:
// the mechanism recovered by fill_mechanism against the table it came from,
// the Array4 -> pc_array4 mapping, and the status of pc_mol_create reached
// through the C ABI (no device here: the adapter aborts with the library's
// message, as getMOLSrcTerm aborts).
#include <cmath>
#include <cstdio>

#include "PeleC_GB300.H"

static double rel(double a, double b) { return b == 0.0 ? std::fabs(a) : std::fabs(a - b) / std::fabs(b); }

int main() {
  constexpr int NS = NUM_SPECIES, NVARS = 7 + NUM_SPECIES;
  TestTransParm tp{};
  for (int k = 0; k < NS; ++k)
    for (int n = 0; n < 4; ++n) {
      tp.fitmu[k * 4 + n] = kVISC[k][n];
      tp.fitlam[k * 4 + n] = kCOND[k][n];
      for (int j = 0; j < NS; ++j) tp.fitdbin[(k * NS + j) * 4 + n] = kDIFF[k][j][n];
    }
  pc_mechanism m;
  const int rc = pc_gb300::fill_mechanism(m, tp);
  double enasa = 0.0, efit = 0.0, emw = 0.0;
  for (int k = 0; k < NS; ++k) {
    emw = std::fmax(emw, rel(m.mw[k], kMW[k]));
    for (int n = 0; n < 6; ++n) {
      // compare each coefficient's contribution at T = 1000 K (cp/R units)
      const double scale = n < 5 ? std::pow(1000.0, n) : 1.0 / 1000.0;
      enasa = std::fmax(enasa, std::fabs(m.nasa_lo[k][n] - kLO[k][n]) * scale);
      enasa = std::fmax(enasa, std::fabs(m.nasa_hi[k][n] - kHI[k][n]) * scale);
    }
    for (int n = 0; n < 4; ++n) {
      efit = std::fmax(efit, rel(m.visc_fit[k][n], kVISC[k][n]));
      efit = std::fmax(efit, rel(m.cond_fit[k][n], kCOND[k][n]));
      for (int j = 0; j < NS; ++j) efit = std::fmax(efit, rel(m.diff_fit[k][j][n], kDIFF[k][j][n]));
    }
  }
  std::printf("fill_mechanism rc %d mw_err %.3e nasa_err %.3e fit_err %.3e tmid %.1f\n", rc, emw, enasa, efit,
              m.nasa_tmid[0]);

  const amrex::Box vb(amrex::IntVect(2, 3, 4), amrex::IntVect(9, 7, 13));
  amrex::MultiFab S({vb}, NVARS, 4), R({vb}, NVARS, 0);
  amrex::MFIter mfi(S, false);
  const pc_array4 a = pc_gb300::to_pc(S.const_array(mfi));
  const pc_array4 r = pc_gb300::to_pc(R.array(mfi));
  std::printf("array4 begin %d %d %d end %d %d %d jstride %lld kstride %lld nstride %lld ncomp %d rhs_begin %d %d %d\n",
              a.begin[0], a.begin[1], a.begin[2], a.end[0], a.end[1], a.end[2], a.jstride, a.kstride, a.nstride,
              a.ncomp, r.begin[0], r.begin[1], r.begin[2]);

  try {
    pc_mol_handle* h = pc_gb300::handle(pc_gb300::flags_config(1, 1, 1, 1, 1, 2, 0, 1), tp);
    amrex::Geometry geom;
    for (int d = 0; d < 3; ++d) geom.gd.dx[d] = 1e-3;
    pc_gb300::mol_src_term(h, S, R, geom, false, [](const amrex::MFIter&, const std::array<amrex::FArrayBox const*, 3>&) {});
    std::printf("create ok\n");
  } catch (const std::exception& e) {
    std::printf("abort %s\n", e.what());
  }
  return 0;
}
