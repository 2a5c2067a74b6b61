// pc_oracle.cpp — ORACLE (test infrastructure): extern "C" entry points of the
// CPU restatement in pc_oracle.hpp, loaded by oracle/pyoracle.py through
// ctypes.  Only tests/, the smoke check and bench.py's CPU-baseline leg call
// these.  Parity status: see pc_oracle.hpp (pinned to the reference's own
// hot-path code; the PelePhysics parts unpinned).
#include "pc_oracle.hpp"

#include <omp.h>

using namespace orc;

namespace {

Arr<double> view(const pc_array4& a) {
  Arr<double> v;
  v.p = a.p;
  v.js = a.jstride;
  v.ks = a.kstride;
  v.ns = a.nstride;
  for (int d = 0; d < 3; ++d) v.b[d] = a.begin[d];
  return v;
}

bool covers(const pc_array4& a, const Box& b) {
  for (int d = 0; d < 3; ++d)
    if (a.begin[d] > b.lo[d] || a.end[d] - 1 < b.hi[d]) return false;
  return true;
}

template <int NS, class EOS, class TR>
int run_box(const pc_mol_config& cfg, const EOS& eos, const TR& tr, const pc_box_desc& bd, const double dx[3],
            long long& fails, const pc_array4* fluxes) {
  Box vbox;
  for (int d = 0; d < 3; ++d) { vbox.lo[d] = bd.lo[d]; vbox.hi[d] = bd.hi[d]; }
  // The reference computes primitives on grow(vbox, 4); the state FAB must
  // cover it (PeleC::numGrow() = 4 without EB).
  if (!covers(bd.state, grow(vbox, 4)) || !covers(bd.rhs, vbox)) return PC_ERR_INVALID_ARGUMENT;
  if (bd.state.ncomp < 7 + NS || bd.rhs.ncomp < 7 + NS) return PC_ERR_INVALID_ARGUMENT;
  Arr<double> s = view(bd.state);
  Arr<const double> sc;
  sc.p = s.p;
  sc.js = s.js;
  sc.ks = s.ks;
  sc.ns = s.ns;
  for (int d = 0; d < 3; ++d) sc.b[d] = s.b[d];
  if (fluxes) {
    Arr<double> fo[3];
    for (int d = 0; d < 3; ++d) {
      if (!covers(fluxes[d], surrounding_nodes(vbox, d)) || fluxes[d].ncomp < 7 + NS) return PC_ERR_INVALID_ARGUMENT;
      fo[d] = view(fluxes[d]);
    }
    mol_rhs_box<NS>(cfg, eos, tr, vbox, sc, view(bd.rhs), dx, fails, fo);
  } else {
    mol_rhs_box<NS>(cfg, eos, tr, vbox, sc, view(bd.rhs), dx, fails);
  }
  return PC_OK;
}

template <int NS>
int dispatch(const pc_mol_config& cfg, const pc_box_desc& bd, const double dx[3], long long& fails,
             const pc_array4* fluxes = nullptr) {
  const int maxit = cfg.newton_max_iter > 0 ? cfg.newton_max_iter : 50;
  if (cfg.eos == PC_EOS_GAMMA_LAW) {
    GammaLaw<NS> eos{&cfg.mech};
    if (cfg.transport == PC_TRANSPORT_CONSTANT)
      return run_box<NS>(cfg, eos, ConstantTransport<NS, GammaLaw<NS>>{&cfg.mech}, bd, dx, fails, fluxes);
    return run_box<NS>(cfg, eos, SimpleTransport<NS, GammaLaw<NS>>{&cfg.mech}, bd, dx, fails, fluxes);
  }
  IdealMix<NS> eos{&cfg.mech, maxit};
  if (cfg.transport == PC_TRANSPORT_CONSTANT)
    return run_box<NS>(cfg, eos, ConstantTransport<NS, IdealMix<NS>>{&cfg.mech}, bd, dx, fails, fluxes);
  return run_box<NS>(cfg, eos, SimpleTransport<NS, IdealMix<NS>>{&cfg.mech}, bd, dx, fails, fluxes);
}

template <int NS, class EOS>
void ct_boxes(int nboxes, const int* lohi, const pc_array4* st, const EOS& eos, long long& fails) {
  for (int i = 0; i < nboxes; ++i) {
    Box v;
    for (int d = 0; d < 3; ++d) {
      v.lo[d] = lohi[6 * i + d];
      v.hi[d] = lohi[6 * i + 3 + d];
    }
    compute_temp<NS>(v, view(st[i]), eos, fails);
  }
}

}  // namespace

extern "C" {

// RHS of each box, as getMOLSrcTerm's MFIter loop.  Host pointers.
int oracle_mol_rhs(const pc_mol_config* cfg, const pc_box_desc* boxes, int nboxes, const double dx[3], int nthreads,
                   long long* newton_fail) {
  if (!cfg || !boxes || nboxes < 0 || !dx) return PC_ERR_INVALID_ARGUMENT;
  if (nthreads > 0) omp_set_num_threads(nthreads);
  long long fails = 0;
  for (int b = 0; b < nboxes; ++b) {
    int rc;
    if (cfg->nspec == 1)
      rc = dispatch<1>(*cfg, boxes[b], dx, fails);
    else if (cfg->nspec == 9)
      rc = dispatch<9>(*cfg, boxes[b], dx, fails);
    else if (cfg->nspec == 21)
      rc = dispatch<21>(*cfg, boxes[b], dx, fails);
    else
      return PC_ERR_UNSUPPORTED;
    if (rc != PC_OK) return rc;
  }
  if (newton_fail) *newton_fail = fails;
  return PC_OK;
}

// RHS of each box plus its face fluxes (fluxes[3 b + dir] on
// surroundingNodes(valid, dir)).
int oracle_mol_rhs_fluxes(const pc_mol_config* cfg, const pc_box_desc* boxes, int nboxes, const double dx[3],
                          const pc_array4* fluxes, int nthreads) {
  if (!cfg || !boxes || nboxes < 0 || !dx || !fluxes) return PC_ERR_INVALID_ARGUMENT;
  if (nthreads > 0) omp_set_num_threads(nthreads);
  long long fails = 0;
  for (int b = 0; b < nboxes; ++b) {
    int rc;
    if (cfg->nspec == 1)
      rc = dispatch<1>(*cfg, boxes[b], dx, fails, fluxes + 3 * b);
    else if (cfg->nspec == 9)
      rc = dispatch<9>(*cfg, boxes[b], dx, fails, fluxes + 3 * b);
    else if (cfg->nspec == 21)
      rc = dispatch<21>(*cfg, boxes[b], dx, fails, fluxes + 3 * b);
    else
      return PC_ERR_UNSUPPORTED;
    if (rc != PC_OK) return rc;
  }
  return PC_OK;
}

// pc_ctoprim on one cell: U[NVAR] -> q[QVAR], qaux[6].
int oracle_ctoprim_cell(const pc_mol_config* cfg, const double* U, double* q, double* qaux, int* newton_ok) {
  const int ns = cfg->nspec;
  Arr<const double> u;
  u.p = U; u.js = 1; u.ks = 1; u.ns = 1;
  Arr<double> qa, qx;
  qa.p = q; qa.js = 1; qa.ks = 1; qa.ns = 1;
  qx.p = qaux; qx.js = 1; qx.ks = 1; qx.ns = 1;
  long long fails = 0;
  const int maxit = cfg->newton_max_iter > 0 ? cfg->newton_max_iter : 50;
  if (ns == 1 && cfg->eos == PC_EOS_GAMMA_LAW) {
    ctoprim<1>(0, 0, 0, u, qa, qx, GammaLaw<1>{&cfg->mech}, fails);
  } else if (ns == 9 && cfg->eos == PC_EOS_IDEAL_MIX) {
    ctoprim<9>(0, 0, 0, u, qa, qx, IdealMix<9>{&cfg->mech, maxit}, fails);
  } else if (ns == 1 && cfg->eos == PC_EOS_IDEAL_MIX) {
    ctoprim<1>(0, 0, 0, u, qa, qx, IdealMix<1>{&cfg->mech, maxit}, fails);
  } else if (ns == 9 && cfg->eos == PC_EOS_GAMMA_LAW) {
    ctoprim<9>(0, 0, 0, u, qa, qx, GammaLaw<9>{&cfg->mech}, fails);
  } else if (ns == 21 && cfg->eos == PC_EOS_IDEAL_MIX) {
    ctoprim<21>(0, 0, 0, u, qa, qx, IdealMix<21>{&cfg->mech, maxit}, fails);
  } else {
    return PC_ERR_UNSUPPORTED;
  }
  if (newton_ok) *newton_ok = fails == 0;
  return PC_OK;
}

// Mixture-averaged or constant transport on one cell: out = [rhoD(ns), mu, xi, lambda].
int oracle_transport_cell(const pc_mol_config* cfg, double T, double rho, const double* Y, double* out) {
  double mu, xi, lam;
  if (cfg->nspec == 9 && cfg->eos == PC_EOS_IDEAL_MIX) {
    IdealMix<9> eos{&cfg->mech, 50};
    if (cfg->transport == PC_TRANSPORT_SIMPLE)
      SimpleTransport<9, IdealMix<9>>{&cfg->mech}.transport(eos, T, rho, Y, out, mu, xi, lam);
    else
      ConstantTransport<9, IdealMix<9>>{&cfg->mech}.transport(eos, T, rho, Y, out, mu, xi, lam);
    out[9] = mu; out[10] = xi; out[11] = lam;
    return PC_OK;
  }
  if (cfg->nspec == 1 && cfg->eos == PC_EOS_GAMMA_LAW) {
    GammaLaw<1> eos{&cfg->mech};
    ConstantTransport<1, GammaLaw<1>>{&cfg->mech}.transport(eos, T, rho, Y, out, mu, xi, lam);
    out[1] = mu; out[2] = xi; out[3] = lam;
    return PC_OK;
  }
  return PC_ERR_UNSUPPORTED;
}

// Mixture thermodynamics at (T, Y): out = [e, cv, cp, Wbar] (IdealMix only).
int oracle_thermo(const pc_mol_config* cfg, double T, const double* Y, double* out) {
  if (cfg->nspec != 9 || cfg->eos != PC_EOS_IDEAL_MIX) return PC_ERR_UNSUPPORTED;
  IdealMix<9> eos{&cfg->mech, 50};
  double e, cv, cp, cv2, wbar;
  eos.TY2E_Cv(T, Y, e, cv);
  eos.TY2CpCv(T, Y, cp, cv2);
  eos.Y2WBAR(Y, wbar);
  out[0] = e; out[1] = cv; out[2] = cp; out[3] = wbar;
  return PC_OK;
}

// riemann() on one face: returns flux[NVAR] (UTEMP slot 0) and ustar.
int oracle_riemann_face(const pc_mol_config* cfg, const double* left, const double* right, double cav, double* flux,
                        double* ustar) {
  // left/right = [rho, un, ut1, ut2, p, Y(ns)]
  if (cfg->nspec == 9 && cfg->eos == PC_EOS_IDEAL_MIX) {
    IdealMix<9> eos{&cfg->mech, 50};
    for (int n = 0; n < 16; ++n) flux[n] = 0.0;
    riemann<9>(left[0], left[1], left[2], left[3], left[4], left + 5, right[0], right[1], right[2], right[3], right[4],
               right + 5, cav, *ustar, flux[URHO], flux + UFS, flux[UMX], flux[UMY], flux[UMZ], flux[UEDEN],
               flux[UEINT], eos);
    return PC_OK;
  }
  if (cfg->nspec == 1 && cfg->eos == PC_EOS_GAMMA_LAW) {
    GammaLaw<1> eos{&cfg->mech};
    for (int n = 0; n < 8; ++n) flux[n] = 0.0;
    riemann<1>(left[0], left[1], left[2], left[3], left[4], left + 5, right[0], right[1], right[2], right[3], right[4],
               right + 5, cav, *ustar, flux[URHO], flux + UFS, flux[UMX], flux[UMY], flux[UMZ], flux[UEDEN],
               flux[UEINT], eos);
    return PC_OK;
  }
  return PC_ERR_UNSUPPORTED;
}

int oracle_max_threads(void) { return omp_get_max_threads(); }

// Ghost fill of a level covering the domain (host arrays).
int oracle_fill_ghosts(const pc_box_desc* boxes, int nboxes, const pc_geometry* geom, int ngrow, int nvar) {
  std::vector<FillBox> fb;
  for (int b = 0; b < nboxes; ++b) {
    FillBox f;
    for (int d = 0; d < 3; ++d) {
      f.valid.lo[d] = boxes[b].lo[d];
      f.valid.hi[d] = boxes[b].hi[d];
    }
    if (!covers(boxes[b].state, grow(f.valid, ngrow))) return PC_ERR_INVALID_ARGUMENT;
    f.S = view(boxes[b].state);
    fb.push_back(f);
  }
  fill_ghosts(fb, *geom, ngrow, nvar);
  return PC_OK;
}

// dst = a x + b y on each box's valid cells (lohi: 6 ints per box).
int oracle_lincomb(int nboxes, const int* lohi, const pc_array4* dst, double a, const pc_array4* x, double b,
                   const pc_array4* y, int nvar) {
  for (int i = 0; i < nboxes; ++i) {
    Box v;
    for (int d = 0; d < 3; ++d) {
      v.lo[d] = lohi[6 * i + d];
      v.hi[d] = lohi[6 * i + 3 + d];
    }
    lincomb(v, nvar, view(dst[i]), a, view(x[i]), b, view(y[i]));
  }
  return PC_OK;
}

int oracle_compute_temp(const pc_mol_config* cfg, int nboxes, const int* lohi, const pc_array4* st,
                        long long* newton_fail) {
  long long fails = 0;
  const int maxit = cfg->newton_max_iter > 0 ? cfg->newton_max_iter : 50;
  if (cfg->nspec == 1 && cfg->eos == PC_EOS_GAMMA_LAW)
    ct_boxes<1>(nboxes, lohi, st, GammaLaw<1>{&cfg->mech}, fails);
  else if (cfg->nspec == 9 && cfg->eos == PC_EOS_IDEAL_MIX)
    ct_boxes<9>(nboxes, lohi, st, IdealMix<9>{&cfg->mech, maxit}, fails);
  else if (cfg->nspec == 21 && cfg->eos == PC_EOS_IDEAL_MIX)
    ct_boxes<21>(nboxes, lohi, st, IdealMix<21>{&cfg->mech, maxit}, fails);
  else
    return PC_ERR_UNSUPPORTED;
  if (newton_fail) *newton_fail = fails;
  return PC_OK;
}

// estTimeStep: dt = cfl * min(hydro, vdif, tdif, edif) capped by max_dt
// (the limits that the configuration's flags switch on); parts[4] returns
// the four minima.
int oracle_est_dt(const pc_mol_config* cfg, const pc_box_desc* boxes, int nboxes, const double dx[3], double cfl,
                  double max_dt, double* dt, double* parts) {
  const double big = std::numeric_limits<double>::max();
  double m4[4] = {big, big, big, big};
  for (int b = 0; b < nboxes; ++b) {
    Box v;
    for (int d = 0; d < 3; ++d) {
      v.lo[d] = boxes[b].lo[d];
      v.hi[d] = boxes[b].hi[d];
    }
    double o[4];
    if (cfg->nspec == 1 && cfg->eos == PC_EOS_GAMMA_LAW) {
      GammaLaw<1> eos{&cfg->mech};
      est_dt<1>(v, view(boxes[b].state), eos, ConstantTransport<1, GammaLaw<1>>{&cfg->mech}, dx, o);
    } else if (cfg->nspec == 9 && cfg->eos == PC_EOS_IDEAL_MIX) {
      IdealMix<9> eos{&cfg->mech, 50};
      est_dt<9>(v, view(boxes[b].state), eos, SimpleTransport<9, IdealMix<9>>{&cfg->mech}, dx, o);
    } else if (cfg->nspec == 21 && cfg->eos == PC_EOS_IDEAL_MIX) {
      IdealMix<21> eos{&cfg->mech, 50};
      est_dt<21>(v, view(boxes[b].state), eos, SimpleTransport<21, IdealMix<21>>{&cfg->mech}, dx, o);
    } else {
      return PC_ERR_UNSUPPORTED;
    }
    for (int q = 0; q < 4; ++q) m4[q] = std::min(m4[q], o[q]);
  }
  const double mdc = max_dt / cfl;
  double eh = mdc, ev = mdc, et = mdc, ee = mdc;
  if (cfg->do_hydro) eh = std::min(eh, m4[0]);
  if (cfg->diffuse_vel) ev = std::min(ev, m4[1]);
  if (cfg->diffuse_temp) et = std::min(et, m4[2]);
  if (cfg->diffuse_enth) ee = std::min(ee, m4[3]);
  eh = std::min(eh, std::min(ev, std::min(et, ee)));
  eh *= cfl;
  *dt = std::min(max_dt, eh);
  if (parts)
    for (int q = 0; q < 4; ++q) parts[q] = m4[q];
  return PC_OK;
}

// The transport's exp and log (pc_exp.h) over an array, for their accuracy
// tests.  which = 0: exp, 1: log.
void oracle_exp_log(int which, const double* x, double* y, long long n) {
  for (long long i = 0; i < n; ++i) y[i] = which == 0 ? pc_math::exp(x[i]) : pc_math::log(x[i]);
}

}  // extern "C"
