// pc_kernels.cuh — the two passes of the MOL right-hand side on one level.
//
// Pass 1 (cell_kernel): one thread per cell of grow(valid, 2) of every box.
//   Conserved -> primitive conversion with the EOS temperature solve
//   (pc_ctoprim, Source/Utilities.H:239-320) and, on grow(valid, 1), the
//   per-cell diffusion data: transport coefficients (pc_transcoeff,
//   Source/TransCoeff.H:7-37), mole fractions (Y2X) and species enthalpies
//   (T2Hi) used by SpeciesEnergyFlux (Source/Diffterm.H:20-75).  The record is
//   written once per cell, structure-of-arrays, into the handle's scratch.
//
// Pass 2 (flux_kernel): one CTA per 8x8x4 tile of valid cells.  For each
//   direction the CTA evaluates every face of the tile exactly once — MOL
//   slopes (mol_slope, MOL.H:28-113), face states (MOL.cpp:69-123), the
//   approximate Riemann solver (riemann, Riemann.H:6-200) or Lax-Friedrichs
//   (Riemann.H:202-307), and the viscous/thermal/species diffusion flux
//   (pc_diffusion_flux, Diffterm.H:344-461) — stages the NVAR face fluxes in
//   shared memory and accumulates the divergence (pc_flux_div,
//   Diffterm.H:463-484) in registers; the RHS is written once.
//
// The expensive per-cell work (Newton solve, ~55 exponentials of the
// mixture-averaged transport) is done once per cell and each face flux once
// per face: on GB300 the FP64 pipe, not HBM, bounds this computation.
#pragma once

#include <atomic>

#include "pc_device.cuh"

namespace PCG_NAMESPACE {

struct DevBox {
  int lo[3], hi[3];
  const double* S;
  long long sj, sk, sn;
  int sb[3];
  int pad0;
  double* R;
  long long rj, rk, rn;
  int rb[3];
  int pad1;
  double* rec;       // scratch records of this box: field f of cell c at rec[f*ncell + c]
  long long ncell;   // cells of grow(valid, 2)
  int g2lo[3];       // smallEnd of grow(valid, 2)
  int n2[3];         // extents of grow(valid, 2)
};

struct Geo {
  double dxs[3];  // cell sizes
  double dxinv[3];
  double area[3];
  double vol;
  double ivol;   // 1 / vol rounded toward zero (rcp_q), the divergence's shared divisor
  double p_ref;  // mixed precision: pressure offset of the FP32 records
};

// Record fields (pass 1 -> pass 2).  IRHO, IC, IC2 are the reciprocals
// rcp_q of rho, c and c c of every cell, the divisors' reciprocals of the
// slopes' and face states' quotients (div_fast), evaluated once per cell.
template <int NS>
struct Rec {
  static constexpr int RHO = 0, U = 1, V = 2, W = 3, P = 4, C = 5, Y = 6;
  static constexpr int T = 6 + NS, X = 7 + NS, H = 7 + 2 * NS, D = 7 + 3 * NS;
  static constexpr int MU = 7 + 4 * NS, XI = 8 + 4 * NS, LAM = 9 + 4 * NS;
  static constexpr int IRHO = 10 + 4 * NS, IC = 11 + 4 * NS, IC2 = 12 + 4 * NS;
  static constexpr int N = 13 + 4 * NS;
};

// Loads of record fields in the flux pass (a Dual specialisation reads
// value and tangent records).
template <class R>
struct RecAcc;
template <>
struct RecAcc<double> {
  const double* p;
  long long N;
  __device__ __forceinline__ double ld(int fld, long long c) const { return __ldg(p + (long long)fld * N + c); }
};

// Tangent arrays of one box for the Jacobian-vector product: the state
// direction Sd (covering grow(valid, 2)), the RHS tangent Rd (valid box) and
// the tangent records trec (same layout as rec).
struct TanBox {
  const double* Sd;
  long long sj, sk, sn;
  int sb[3];
  int pad0;
  double* Rd;
  long long rj, rk, rn;
  int rb[3];
  int pad1;
  double* trec;
};

// Face-flux outputs of one box (refluxing): direction d's fluxes, times the
// face area, on surroundingNodes(valid, d): face (i,j,k), component n at
// p[d][(i-b[d][0]) + (j-b[d][1]) js[d] + (k-b[d][2]) ks[d] + n ns[d]].
struct FluxBox {
  double* p[3];
  long long js[3], ks[3], ns[3];
  int b[3][3];
  int pad;
};

// kCounterSlowCell / kCounterSlowFlux: lanes of the fast cell / flux pass
// with an operand that div_fast leaves to a real division; nonzero makes the
// exact twin of that pass evaluate it again.
enum {
  kCounterCells = 0,
  kCounterNewton = 1,
  kCounterNonpos = 2,
  kCounterNonfinite = 3,
  kCounterSlowCell = 4,
  kCounterSlowFlux = 5,
  kCounterSlowAdj = 6,  // the same for the face adjoint of the VJP
  kNumCounters = 7
};

__device__ __forceinline__ void warp_count(unsigned long long* ctr, bool pred) {
  const unsigned m = __ballot_sync(0xffffffffu, pred);
  if ((threadIdx.x & 31) == 0 && m) atomicAdd(ctr, (unsigned long long)__popc(m));
}

constexpr int kCellThreads = 256;

// ---------------------------------------------------------------------------
// Pass 1.
// items[b] = (box index, first cell of the 256-cell chunk in grow(valid,2)).
// ---------------------------------------------------------------------------
// The EOS temperature solve of the cell pass (a Dual overload differentiates
// it by the implicit-function theorem).
template <class EOS, int NS>
__device__ __forceinline__ double rey2t_of(const DevMech<NS>& m, const double* Y, double rw, double e, double Tguess,
                                           int maxit, bool& ok) {
  return EOS::rey2t(m, Y, rw, e, Tguess, maxit, ok);
}

// pc_ctoprim and the per-cell diffusion data of one cell, generic in the
// scalar type: U holds the conserved components, Tguess the Newton guess
// U(UTEMP); st(field, value) writes a record field.  inner: the cell lies in
// grow(valid, 1), where the diffusion fluxes need T, X, h and the transport
// coefficients.
template <int NS, class EOS, class TR, class R, class Store, class Q = QuotSelf>
__device__ __forceinline__ void cell_record(const DevMech<NS>& m, const DevFlags& f, const R* U, double Tguess,
                                            bool inner, Store st, bool& newton_fail, bool& nonpos, Q&& q = Q()) {
  using RC = Rec<NS>;
  const R rho = U[URHO];
  const R rhoinv = 1.0 / rho;
  const R vx = U[UMX] * rhoinv;
  const R vy = U[UMY] * rhoinv;
  const R vz = U[UMZ] * rhoinv;
  const R kineng = 0.5 * rho * (vx * vx + vy * vy + vz * vz);
  const R e = (U[UEDEN] - kineng) * rhoinv;
  const R rhoinv_q = rcp_q_from_rn(rho, rhoinv);  // the quotients' reciprocal (rounded toward zero)
  R Y[NS];
#pragma unroll
  for (int n = 0; n < NS; ++n) {
    const R y = q(U[UFS + n], rho, rhoinv_q);  // = rho Y_n / rho, correctly rounded
    Y[n] = zero_below(y, 1e-4 * 2.220446049250313e-16);  // |Y| < 1e-4 eps -> 0 (Utilities.H:288-294)
  }
  const R rw = mix_rw<NS>(m, Y);
  bool ok = true;
  const R T = rey2t_of<EOS>(m, Y, rw, e, Tguess, f.newton_maxit, ok);
  const R p = rho * rw * T;                      // RTY2P
  const R cs = EOS::cs_T(m, Y, rw, rho, T, p);  // RTY2Cs
  newton_fail = !ok;
  nonpos = !(rho > 0.0) || !(p > 0.0) || !(T > 0.0);
  st(RC::RHO, rho);
  st(RC::U, vx);
  st(RC::V, vy);
  st(RC::W, vz);
  st(RC::P, p);
  st(RC::C, cs);
  st(RC::IRHO, rhoinv_q);
  st(RC::IC, rcp_q(cs));
  st(RC::IC2, rcp_q(cs * cs));
#pragma unroll
  for (int n = 0; n < NS; ++n) st(RC::Y + n, Y[n]);
  if (inner) {
    // Mole fractions (Y2X) and enthalpies (T2Hi) of the cell.
    R X[NS];
    y2x(m, Y, rw, X, q);
    R out[NS + 3];
    TR::eval(m, T, rho, p, Y, X, out, q);
    st(RC::T, T);
#pragma unroll
    for (int n = 0; n < NS; ++n) st(RC::X + n, X[n]);
    R h[NS];
    EOS::hi(m, T, h);
#pragma unroll
    for (int n = 0; n < NS; ++n) st(RC::H + n, h[n]);
#pragma unroll
    for (int n = 0; n < NS + 3; ++n) st(RC::D + n, out[n]);
  }
}

// Cell (i, j, k) of record index c in grow(valid, 2) of box b.
__device__ __forceinline__ void cell_index(const DevBox& b, long long c, int& i, int& j, int& k) {
  const int nx = b.n2[0], ny = b.n2[1];
  i = b.g2lo[0] + (int)(c % nx);
  j = b.g2lo[1] + (int)((c / nx) % ny);
  k = b.g2lo[2] + (int)(c / ((long long)nx * ny));
}

__device__ __forceinline__ bool in_grow1(const DevBox& b, int i, int j, int k) {
  return i >= b.lo[0] - 1 && i <= b.hi[0] + 1 && j >= b.lo[1] - 1 && j <= b.hi[1] + 1 && k >= b.lo[2] - 1 &&
         k <= b.hi[2] + 1;
}

// Bit pattern the fast cell pass leaves in the RHO field of a record whose
// quotients need an IEEE division (a NaN no arithmetic produces), so that
// the exact twin evaluates only those cells again.
constexpr long long kSlowRecord = 0x7ff8dead5107beefLL;

// kExact = false: the fast pass (quotients by div_fast); kExact = true: its
// exact twin, which returns at once unless the fast pass counted a lane that
// needs a real division, and then writes again, with IEEE quotients, the
// records the fast pass marked (kSlowRecord).
template <int NS, class EOS, class TR, bool kExact = false>
__global__ void __launch_bounds__(kCellThreads)
    cell_kernel(const DevBox* __restrict__ boxes, const int2* __restrict__ items, const __grid_constant__ DevMech<NS> m,
                const DevFlags f, unsigned long long* __restrict__ counters) {
  constexpr int NVAR = 7 + NS;
  if (kExact && __ldcg(&counters[kCounterSlowCell]) == 0ull) return;
  const int2 it = items[blockIdx.x];
  const DevBox& b = boxes[it.x];
  const long long c = (long long)it.y + threadIdx.x;
  bool newton_fail = false, nonpos = false;
  Quot<kExact> quo;
  if (c < b.ncell) {
    int i, j, k;
    cell_index(b, c, i, j, k);
    const double* s = b.S + (i - b.sb[0]) + (long long)(j - b.sb[1]) * b.sj + (long long)(k - b.sb[2]) * b.sk;
    const long long sn = b.sn;
    double U[NVAR];
#pragma unroll
    for (int n = 0; n < NVAR; ++n) U[n] = (n == UEINT || n == UTEMP) ? 0.0 : __ldg(s + n * sn);
    double* r = b.rec + c;
    const long long N = b.ncell;
    const bool todo = !kExact || __double_as_longlong(r[Rec<NS>::RHO * N]) == kSlowRecord;
    if (todo) {
      cell_record<NS, EOS, TR>(m, f, U, __ldg(s + UTEMP * sn), in_grow1(b, i, j, k),
                               [&](int fld, double v) { r[fld * N] = v; }, newton_fail, nonpos, quo);
      if (!kExact && quo.slow) r[Rec<NS>::RHO * N] = __longlong_as_double(kSlowRecord);
    }
  }
  if (!kExact) {  // the exact twin re-evaluates cells the fast pass has counted already
    warp_count(&counters[kCounterNewton], newton_fail);
    warp_count(&counters[kCounterNonpos], nonpos);
    warp_count(&counters[kCounterSlowCell], quo.slow);
  }
}

// Host: the cell pass over nitems chunks: the fast kernel, then its exact
// twin (which returns at once unless the fast kernel counted a lane that
// needs a real division).  The PC_PRECISION_FP64_RCP compilation has no
// such lanes and launches the fast kernel only.
template <int NS, class EOS, class TR>
inline cudaError_t launch_cell_fp64(const DevBox* boxes, const int2* items, unsigned nitems, const DevMech<NS>& m,
                                    const DevFlags& f, unsigned long long* counters, cudaStream_t s) {
  if (nitems == 0) return cudaSuccess;
  cell_kernel<NS, EOS, TR, false><<<nitems, kCellThreads, 0, s>>>(boxes, items, m, f, counters);
#ifndef PCG_RECIPROCAL_QUOTIENTS
  cell_kernel<NS, EOS, TR, true><<<nitems, kCellThreads, 0, s>>>(boxes, items, m, f, counters);
#endif
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Hyperbolic flux on the low face of the cell at record index cR in
// direction d, times the face area: F[n] = flux_n * A (Riemann.H, MOL.cpp).
// Divisions that share a divisor use div_by (exact, see pc_device.cuh).
// ---------------------------------------------------------------------------
// MOL slopes of the cell at record index c in direction d (mol_slope,
// MOL.H:53-112): the characteristic slopes dq[0..3] and the species slopes
// ds[NS].  A function of the cells c - st, c and c + st only, so one
// evaluation serves both faces of the cell.
template <int NS, int d, class R, class Q = QuotSelf>
__device__ __forceinline__ void cell_slopes(const RecAcc<R>& ra, long long c, long long st, R* dq, R* ds,
                                            Q&& q = Q()) {
  using RC = Rec<NS>;
  auto ld = [&](int fld, long long cc) { return ra.ld(fld, cc); };
  const long long cm = c - st, cp = c + st;
  const int fun = RC::U + d;
  const int fut1 = (d == 0) ? RC::V : RC::U;
  const int fut2 = (d == 2) ? RC::V : RC::W;
  const R r0 = ld(RC::RHO, c), rm = ld(RC::RHO, cm), rp = ld(RC::RHO, cp);
  const R p0 = ld(RC::P, c), pm = ld(RC::P, cm), pp = ld(RC::P, cp);
  const R u0 = ld(fun, c), um = ld(fun, cm), up = ld(fun, cp);
  const R c0 = ld(RC::C, c);
  const R yc = ld(RC::IC, c);  // 1 / c0
  const R dpl = p0 - pm, dpr = pp - p0;
  {
    const R a = q(halve(dpl), c0, yc), bb = halve(r0) * (u0 - um);
    const R a2 = q(halve(dpr), c0, yc), b2 = halve(r0) * (up - u0);
    dq[0] = mc_limit(a - bb, a2 - b2);
    dq[1] = mc_limit(a + bb, a2 + b2);
  }
  {
    const R t0 = ld(fut1, c);
    dq[2] = mc_limit(t0 - ld(fut1, cm), ld(fut1, cp) - t0);
    const R w0 = ld(fut2, c);
    dq[3] = mc_limit(w0 - ld(fut2, cm), ld(fut2, cp) - w0);
  }
  const R c2 = c0 * c0;
  const R yc2 = ld(RC::IC2, c);  // 1 / c2
#pragma unroll
  for (int n = 0; n < NS; ++n) {
    const R y0 = ld(RC::Y + n, c);
    const R ry0 = r0 * y0;
    ds[n] = mc_limit(ry0 - rm * ld(RC::Y + n, cm) - q(y0 * dpl, c2, yc2),
                     rp * ld(RC::Y + n, cp) - ry0 - q(y0 * dpr, c2, yc2));
  }
}

// Hyperbolic flux on the low face of the cell at record index cR in
// direction d, times the face area, given the slopes of its two cells.
template <int NS, class EOS, int d, class R, class Q = QuotSelf>
__device__ __forceinline__ void hydro_face_sl(const RecAcc<R>& ra, const DevMech<NS>& m, const DevFlags& f,
                                              long long cR, long long st, double A, const R* dqL, const R* dsL,
                                              const R* dqR, const R* dsR, R* F, Q&& q = Q()) {
  using RC = Rec<NS>;
  const long long cL = cR - st;
  auto ld = [&](int fld, long long c) { return ra.ld(fld, c); };
  const int fun = RC::U + d;
  const int fut1 = (d == 0) ? RC::V : RC::U;
  const int fut2 = (d == 2) ? RC::V : RC::W;
  const R rL = ld(RC::RHO, cL), rR = ld(RC::RHO, cR);
  const R pL = ld(RC::P, cL), pR = ld(RC::P, cR);
  const R uL = ld(fun, cL), uR = ld(fun, cR);
  const R cLc = ld(RC::C, cL), cRc = ld(RC::C, cR);
  const R t1L = ld(fut1, cL), t1R = ld(fut1, cR), t2L = ld(fut2, cL), t2R = ld(fut2, cR);
  const R ycL = ld(RC::IC, cL), ycR = ld(RC::IC, cR);  // 1 / c of both cells
  // Face states (MOL.cpp:69-123).
  const R unl = uL + halve(q(dqL[1] - dqL[0], rL, ld(RC::IRHO, cL)));
  const R pl = pL + halve(dqL[0] + dqL[1]) * cLc;
  const R ut1l = t1L + halve(dqL[2]);
  const R ut2l = t2L + halve(dqL[3]);
  const R unr = uR - halve(q(dqR[1] - dqR[0], rR, ld(RC::IRHO, cR)));
  const R pr = pR - halve(dqR[0] + dqR[1]) * cRc;
  const R ut1r = t1R - halve(dqR[2]);
  const R ut2r = t2R - halve(dqR[3]);
  R spl[NS], spr[NS];
  R rl = 0.0, rr = 0.0;
  {
    const R sL = dqL[0] + dqL[1], sR = dqR[0] + dqR[1];
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      const R yL = ld(RC::Y + n, cL), yR = ld(RC::Y + n, cR);
      spl[n] = yL * rL + halve(dsL[n] + q(yL * sL, cLc, ycL));
      spr[n] = yR * rR - halve(dsR[n] + q(yR * sR, cRc, ycR));
      rl += spl[n];
      rr += spr[n];
    }
    const R yrl = rcp_q(rl), yrr = rcp_q(rr);
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      spl[n] = q(spl[n], rl, yrl);
      spr[n] = q(spr[n], rr, yrr);
    }
  }
  const R cavg = halve(cRc + cLc);
  R fl_rho, fl_un, fl_ut1, fl_ut2, fl_E, fl_ei;
  R flY[NS];
  const R rwl = mix_rw<NS>(m, spl), rwr = mix_rw<NS>(m, spr);
  const R cl = EOS::cs_rp(m, spl, rwl, rl, pl);
  const R cr = EOS::cs_rp(m, spr, rwr, rr, pr);
  if (!f.laxf) {
    // riemann(), Source/Riemann.H:42-199.
    const double wsmall = 2.2250738585072014e-308;
    const R wl = fmax_pos(cl * rl, wsmall);  // max(wsmall, c rho), on the bit patterns for double
    const R wr = fmax_pos(cr * rr, wsmall);
    const R ww = wl + wr, yww = rcp_q(ww);
    const R pstar = fmax_pos(q((wr * pl + wl * pr) + wl * wr * (unl - unr), ww, yww), wsmall);
    R ustar = q((wl * unl + wr * unr) + (pl - pr), ww, yww);
    bool mask = ustar > 0.0;
    R rspo[NS];
    R uo = mask ? unl : unr;
    R po = mask ? pl : pr;
    const bool m0 = fabs(ustar) < kSmallU * 0.5 * (fabs(unl) + fabs(unr)) || ustar == 0.0;
    ustar = m0 ? 0.0 : ustar;
    {
      const R ro_ = mask ? rl : rr;
#pragma unroll
      for (int n = 0; n < NS; ++n) rspo[n] = ro_ * (mask ? spl[n] : spr[n]);
    }
    R iv1 = mask ? ut1l : ut1r;
    R iv2 = mask ? ut2l : ut2r;
    // u* = 0 (Riemann.H:79-85, 131-133): the average of both sides.  Rare, so
    // evaluated only in warps where some face needs it.
    rare_for_warp(m0, [&] {
#pragma unroll
      for (int n = 0; n < NS; ++n) rspo[n] = halve(rl * spl[n] + rr * spr[n]);
      uo = halve(unl + unr);
      po = halve(pl + pr);
      iv1 = halve(ut1l + ut1r);
      iv2 = halve(ut2l + ut2r);
    });
    R ro = 0.0;
#pragma unroll
    for (int n = 0; n < NS; ++n) ro += rspo[n];
    R Yt[NS];
    {
      const R y = rcp_q(ro);
#pragma unroll
      for (int n = 0; n < NS; ++n) Yt[n] = q(rspo[n], ro, y);
    }
    const R co = EOS::cs_rp(m, Yt, mix_rw<NS>(m, Yt), ro, po);
    const R drho = (pstar - po) / (co * co);
    R rspstar[NS];
    R rstar = 0.0;
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      rspstar[n] = fmax_pos(rspo[n] + drho * Yt[n], 0.0);  // max(0, .)
      rstar += rspstar[n];
    }
    {
      const R y = rcp_q(rstar);
#pragma unroll
      for (int n = 0; n < NS; ++n) Yt[n] = q(rspstar[n], rstar, y);
    }
    const R cstar = EOS::cs_rp(m, Yt, mix_rw<NS>(m, Yt), rstar, pstar);
    R spout = co - signed_by(uo, ustar);     // co - copysign(1, u*) uo
    R spin = cstar - signed_by(ustar, ustar);
    const R ushock = halve(spin + spout);
    mask = pstar < po;
    spout = mask ? spout : ushock;
    spin = mask ? spin : ushock;
    // Godunov state (Riemann.H:123-162): the star state where spin >= 0, else
    // the upwind state where spout < 0, else the rarefaction-fan blend.  The
    // blend and its fraction are evaluated only in warps where some face lies
    // in a fan (transonic rarefactions; none in subsonic flow).
    const bool mout = spout < 0.0, min_ = spin >= 0.0;
    R iu = min_ ? ustar : uo;
    R gdp = min_ ? pstar : po;
#pragma unroll
    for (int n = 0; n < NS; ++n) flY[n] = min_ ? rspstar[n] : rspo[n];
    const bool fan = !min_ && !mout;
    rare_for_warp(fan, [&] {
      const R scr = (fabs(spout - spin) < PCG_VERY_SMALL_NUM) ? kSmallNum * cavg : spout - spin;
      const R frac = fmax(0.0, fmin(1.0, (1.0 + (spout + spin) / scr) * 0.5));
      const R omf = 1.0 - frac;
      iu = frac * ustar + omf * uo;
      gdp = frac * pstar + omf * po;
#pragma unroll
      for (int n = 0; n < NS; ++n) flY[n] = frac * rspstar[n] + omf * rspo[n];
    });
    R rgd = 0.0;
#pragma unroll
    for (int n = 0; n < NS; ++n) rgd += flY[n];
    {
      const R y = rcp_q(rgd);
#pragma unroll
      for (int n = 0; n < NS; ++n) Yt[n] = q(flY[n], rgd, y);
    }
    const R regd = rgd * EOS::e_rp(m, Yt, mix_rw<NS>(m, Yt), rgd, gdp);
    fl_rho = rgd * iu;
#pragma unroll
    for (int n = 0; n < NS; ++n) flY[n] *= iu;
    fl_un = fl_rho * iu + gdp;
    fl_ut1 = fl_rho * iv1;
    fl_ut2 = fl_rho * iv2;
    const R rhoetot = regd + halve(rgd) * (iu * iu + iv1 * iv1 + iv2 * iv2);
    fl_E = iu * (rhoetot + gdp);
    fl_ei = iu * regd;
  } else {
    // laxfriedrich_flux(), Source/Riemann.H:202-307.
    const R el = EOS::e_rp(m, spl, rwl, rl, pl);
    const R er = EOS::e_rp(m, spr, rwr, rr, pr);
    const R r_elt = rl * (el + 0.5 * (unl * unl + ut1l * ut1l + ut2l * ut2l));
    const R r_ert = rr * (er + 0.5 * (unr * unr + ut1r * ut1r + ut2r * ut2r));
    const double wsmall = 2.2250738585072014e-308;
    const R wl = fmax_pos(cl * rl, wsmall);
    const R wr = fmax_pos(cr * rr, wsmall);
    R ustar = ((wl * unl + wr * unr) + (pl - pr)) / (wl + wr);
    const bool m0 = fabs(ustar) < kSmallU * 0.5 * (fabs(unl) + fabs(unr)) || ustar == 0.0;
    ustar = m0 ? 0.0 : ustar;
    const R mw = fabs(ustar) + 0.5 * (cr + cl);
    fl_rho = 0.0;
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      flY[n] = 0.5 * ((rl * unl * spl[n] + rr * unr * spr[n]) - mw * (rr * spr[n] - rl * spl[n]));
      fl_rho += flY[n];
    }
    fl_un = 0.5 * ((rl * unl * unl + pl + rr * unr * unr + pr) - mw * (rr * unr - rl * unl));
    fl_ut1 = 0.5 * ((rl * ut1l * unl + rr * ut1r * unr) - mw * (rr * ut1r - rl * ut1l));
    fl_ut2 = 0.5 * ((rl * ut2l * unl + rr * ut2r * unr) - mw * (rr * ut2r - rl * ut2l));
    fl_E = 0.5 * (((r_elt + pl) * unl + (r_ert + pr) * unr) - mw * (r_ert - r_elt));
    fl_ei = 0.5 * ((rl * el * unl + rr * er * unr) - mw * (rr * er - rl * el));
  }
  F[URHO] = fl_rho * A;
  F[UMX + d] = fl_un * A;
  F[(d == 0) ? UMY : UMX] = fl_ut1 * A;
  F[(d == 2) ? UMY : UMZ] = fl_ut2 * A;
  F[UEDEN] = fl_E * A;
  F[UEINT] = fl_ei * A;
  F[UTEMP] = 0.0;
#pragma unroll
  for (int n = 0; n < NS; ++n) F[UFS + n] = flY[n] * A;
}

// Hyperbolic flux on the low face of the cell at record index cR in
// direction d, times the face area: F[n] = flux_n * A (Riemann.H, MOL.cpp),
// with the slopes of both cells evaluated here.
template <int NS, class EOS, int d, class R, class Q = QuotSelf>
__device__ __forceinline__ void hydro_face(const RecAcc<R>& ra, const DevMech<NS>& m, const DevFlags& f, long long cR,
                                           long long st, double A, R* F, Q&& q = Q()) {
  R dqL[4] = {0.0, 0.0, 0.0, 0.0}, dqR[4] = {0.0, 0.0, 0.0, 0.0};
  R dsL[NS], dsR[NS];
#pragma unroll
  for (int n = 0; n < NS; ++n) dsL[n] = dsR[n] = 0.0;
  if (f.slopes) {
    cell_slopes<NS, d>(ra, cR - st, st, dqL, dsL, q);
    cell_slopes<NS, d>(ra, cR, st, dqR, dsR, q);
  }
  hydro_face_sl<NS, EOS, d>(ra, m, f, cR, st, A, dqL, dsL, dqR, dsR, F, q);
}

// pc_diffusion_flux + SpeciesEnergyFlux (Diffterm.H:20-75, 344-461), times
// the area, added to the hyperbolic flux already in F (the reference stores
// the diffusion flux and adds the hyperbolic one, MOL.cpp:199-201; the sum of
// two rounded terms does not depend on their order).  Components switched off
// by the diffuse_* flags get no diffusion term (Diffusion.cpp:321-341).
template <int NS, class EOS, int d, class R>
__device__ __forceinline__ void diffusion_face(const RecAcc<R>& ra, const DevFlags& f, const Geo& g, long long cR,
                                               const long long stv[3], R* F) {
  using RC = Rec<NS>;
  auto ld = [&](int fld, long long c) { return ra.ld(fld, c); };
  const long long cL = cR - stv[d];
  const bool harm = f.harmonic != 0;
  const R mu = face_coef(ld(RC::MU, cR), ld(RC::MU, cL), harm);
  const R xi = face_coef(ld(RC::XI, cR), ld(RC::XI, cL), harm);
  const R lam = face_coef(ld(RC::LAM, cR), ld(RC::LAM, cL), harm);
  // Velocity gradients at the face.
  R grad[3][3];  // grad[c][a] = d u_c / d x_a (only the entries used)
  const R uR[3] = {ld(RC::U, cR), ld(RC::V, cR), ld(RC::W, cR)};
  const R uL[3] = {ld(RC::U, cL), ld(RC::V, cL), ld(RC::W, cL)};
#pragma unroll
  for (int c = 0; c < 3; ++c) grad[c][d] = g.dxinv[d] * (uR[c] - uL[c]);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (a == d) continue;
    const long long sa = stv[a];
    const double q4 = 0.25 * g.dxinv[a];
    // components a (for div u) and d (for tau_da)
    const int ca = RC::U + a, cd = RC::U + d;
    grad[a][a] = (ld(ca, cR + sa) + ld(ca, cL + sa) - ld(ca, cR - sa) - ld(ca, cL - sa)) * q4;
    grad[d][a] = (ld(cd, cR + sa) + ld(cd, cL + sa) - ld(cd, cR - sa) - ld(cd, cL - sa)) * q4;
  }
  const R divu = grad[0][0] + grad[1][1] + grad[2][2];
  R tau[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (a == d)
      tau[a] = mu * (2.0 * grad[d][d] - 2.0 / 3.0 * divu) + xi * divu;
    else
      tau[a] = mu * (grad[d][a] + grad[a][d]);
  }
  const R TR = ld(RC::T, cR), TL = ld(RC::T, cL);
  const R dTdd = g.dxinv[d] * (TR - TL);
  R fE = halve(-tau[0] * (uR[0] + uL[0]) - tau[1] * (uR[1] + uL[1]) - tau[2] * (uR[2] + uL[2])) - lam * dTdd;
  const double A = g.area[d];
  const bool spec = f.diffuse_spec != 0;
  const bool ener = (f.diffuse_temp != 0) || (f.diffuse_enth != 0);
  if (NS > 1 || spec || ener) {
    const R pR = ld(RC::P, cR), pL = ld(RC::P, cL);
    const R dpdx = g.dxinv[d] * (pR - pL);
    const R dlnp = dpdx / halve(pR + pL);
    R Vd[NS], Yf[NS], hf[NS];
    R Vc = 0.0;
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      const R x1 = ld(RC::X + n, cR), x2 = ld(RC::X + n, cL);
      const R y1 = ld(RC::Y + n, cR), y2 = ld(RC::Y + n, cL);
      const R Xface = halve(x1 + x2);
      Yf[n] = halve(y1 + y2);
      hf[n] = halve(ld(RC::H + n, cR) + ld(RC::H + n, cL));
      const R dXdx = g.dxinv[d] * (x1 - x2);
      const R D = face_coef(ld(RC::D + n, cR), ld(RC::D + n, cL), harm);
      Vd[n] = -D * (dXdx + (Xface - Yf[n]) * dlnp);
      Vc += Vd[n];
      fE += Vd[n] * hf[n];
    }
#pragma unroll
    for (int n = 0; n < NS; ++n) {
      const R v = Vd[n] - Yf[n] * Vc;
      fE -= Yf[n] * hf[n] * Vc;
      if (spec) F[UFS + n] += v * A;
    }
  }
  if (f.diffuse_vel) {
#pragma unroll
    for (int a = 0; a < 3; ++a) F[UMX + a] += -tau[a] * A;
  }
  if (ener) F[UEDEN] += fE * A;
}

// ---------------------------------------------------------------------------
// Pass 2.  tiles[b] = (box index, tile origin i, j, k).
// ---------------------------------------------------------------------------
// Tile of the flux pass: TX x TY x TZ cells, one thread per cell, MINB CTAs
// per SM requested from the register allocator.  MAXF and MAXC are the
// largest face and slope-cell counts of one direction (the shared-memory
// staging of the FP64 pass).
template <int TX_, int TY_, int TZ_, int MINB_>
struct Tile {
  static constexpr int TX = TX_, TY = TY_, TZ = TZ_, MINB = MINB_, NT = TX_ * TY_ * TZ_;
  static constexpr int F0 = (TX_ + 1) * TY_ * TZ_, F1 = TX_ * (TY_ + 1) * TZ_, F2 = TX_ * TY_ * (TZ_ + 1);
  static constexpr int MAXF = F0 > F1 ? (F0 > F2 ? F0 : F2) : (F1 > F2 ? F1 : F2);
  // cells whose slopes a direction pass needs: the tile plus one layer on
  // each side in that direction
  static constexpr int C0 = (TX_ + 2) * TY_ * TZ_, C1 = TX_ * (TY_ + 2) * TZ_, C2 = TX_ * TY_ * (TZ_ + 2);
  static constexpr int MAXC = C0 > C1 ? (C0 > C2 ? C0 : C2) : (C1 > C2 ? C1 : C2);
};
// The tile shapes the level autotuner chooses from (index = PC_TILE_* order).
using TileDefault = Tile<8, 8, 4, 2>;
using TileCube = Tile<8, 8, 8, 1>;
using TileLong = Tile<16, 8, 4, 1>;
using TileSmall = Tile<8, 4, 4, 4>;
constexpr int kNumTiles = 4;
// Launch configurations of the flux pass: tile shape t (one CTA per tile) and
// t + kNumTiles (the same shape, persistent grid).
constexpr int kNumLaunchConfigs = 2 * kNumTiles;
__host__ __device__ constexpr int tile_extent(int t, int d) {
  return t == 1 ? 8 : t == 2 ? (d == 0 ? 16 : d == 1 ? 8 : 4) : t == 3 ? (d == 0 ? 8 : 4) : (d == 2 ? 4 : 8);
}
constexpr int kTX = TileDefault::TX, kTY = TileDefault::TY, kTZ = TileDefault::TZ, kFluxThreads = TileDefault::NT;
constexpr int kMaxFaces = TileDefault::MAXF;

// What a CTA hands from one tile to the next tile up the same column (z
// pass only): the fluxes of the shared face layer and the slopes of the cell
// layer above it, which the next tile would otherwise evaluate again.
//   carry: this tile continues the column of the CTA's previous tile: take
//          face layer 0 and slope layer 1 from cflux / cslope;
//   save:  the CTA's next tile continues this one: leave the top face layer
//          and the top slope layer there.
struct ZCarry {
  bool carry, save;
  double* cflux;   // NVAR x (TX TY)
  double* cslope;  // (4 + NS) x (TX TY)
};

// One direction of pass 2: every face of the tile with normal d, staged in
// shared memory, then differenced into the cell accumulators.
template <int NS, class EOS, int d, class TL, class Q>
__device__ __forceinline__ void dir_pass(const DevBox& b, const DevMech<NS>& m, const DevFlags& f, const Geo& g,
                                         const int o[3], const int ext[3], const long long stv[3], bool mine, int tx,
                                         int ty, int tz, double* fbuf, double* acc, const FluxBox* fxb,
                                         const ZCarry& zc, Q& quo) {
  constexpr int LAYER = TL::TX * TL::TY;  // carry buffer stride
  constexpr int NVAR = 7 + NS;
  constexpr int NSL = 4 + NS;  // slope fields of a cell
  const RecAcc<double> ra{b.rec, b.ncell};
  const bool diff = f.diffuse_vel || f.diffuse_temp || f.diffuse_spec || f.diffuse_enth;
  const bool slopes = f.do_hydro && f.slopes;
  // Slopes of every cell of the tile and of its two neighbour layers in d,
  // each evaluated once: field q of cell ci at sbuf[q MAXC + ci].
  double* sbuf = fbuf + NVAR * TL::MAXF;
  const int ne0 = ext[0] + 2 * (d == 0), ne1 = ext[1] + 2 * (d == 1), ne2 = ext[2] + 2 * (d == 2);
  const bool carry = d == 2 && zc.carry;
  if (slopes) {
    const int ncells = ne0 * ne1 * ne2;
    for (int ci = threadIdx.x; ci < ncells; ci += TL::NT) {
      const int ex = ci % ne0, ey = (ci / ne0) % ne1, ez = ci / (ne0 * ne1);
      if (carry && ez < 2) {  // layer 0 feeds only face layer 0 (carried); layer 1 is the carried top layer
        if (ez == 1) {
#pragma unroll
          for (int q = 0; q < NSL; ++q) sbuf[q * TL::MAXC + ci] = zc.cslope[q * LAYER + ex + ne0 * ey];
        }
        continue;
      }
      const int i = o[0] + ex - (d == 0), j = o[1] + ey - (d == 1), k = o[2] + ez - (d == 2);
      const long long c = (i - b.g2lo[0]) + (j - b.g2lo[1]) * stv[1] + (k - b.g2lo[2]) * stv[2];
      double sl[NSL];
      cell_slopes<NS, d>(ra, c, stv[d], sl, sl + 4, quo);
#pragma unroll
      for (int q = 0; q < NSL; ++q) sbuf[q * TL::MAXC + ci] = sl[q];
    }
    __syncthreads();
  }
  const int nf0 = ext[0] + (d == 0), nf1 = ext[1] + (d == 1), nf2 = ext[2] + (d == 2);
  const int nfaces = nf0 * nf1 * nf2;
  const int cstep = (d == 0) ? 1 : (d == 1) ? ne0 : ne0 * ne1;
  for (int fi = threadIdx.x; fi < nfaces; fi += TL::NT) {
    const int fx = fi % nf0, fy = (fi / nf0) % nf1, fz = fi / (nf0 * nf1);
    const int i = o[0] + fx, j = o[1] + fy, k = o[2] + fz;
    if (carry && fz == 0) {  // the face layer the previous tile of the column evaluated (and exported)
#pragma unroll
      for (int n = 0; n < NVAR; ++n) fbuf[n * TL::MAXF + fi] = zc.cflux[n * LAYER + fx + nf0 * fy];
      continue;
    }
    const long long cR = (i - b.g2lo[0]) + (j - b.g2lo[1]) * stv[1] + (k - b.g2lo[2]) * stv[2];
    double F[NVAR];
    if (f.do_hydro) {
      double sL[NSL], sR[NSL];
      if (slopes) {
        const int ciL = fx + ne0 * (fy + ne1 * fz);  // the low cell's slot; the high cell is one step on
#pragma unroll
        for (int q = 0; q < NSL; ++q) {
          sL[q] = sbuf[q * TL::MAXC + ciL];
          sR[q] = sbuf[q * TL::MAXC + ciL + cstep];
        }
      } else {
#pragma unroll
        for (int q = 0; q < NSL; ++q) sL[q] = sR[q] = 0.0;
      }
      hydro_face_sl<NS, EOS, d>(ra, m, f, cR, stv[d], g.area[d], sL, sL + 4, sR, sR + 4, F, quo);
    } else {
#pragma unroll
      for (int n = 0; n < NVAR; ++n) F[n] = 0.0;
    }
    if (diff) diffusion_face<NS, EOS, d>(ra, f, g, cR, stv, F);
#pragma unroll
    for (int n = 0; n < NVAR; ++n) fbuf[n * TL::MAXF + fi] = F[n];
    if (fxb) {  // export (a face shared by two tiles is written twice, with the same value)
      double* q = fxb->p[d] + (i - fxb->b[d][0]) + (long long)(j - fxb->b[d][1]) * fxb->js[d] +
                  (long long)(k - fxb->b[d][2]) * fxb->ks[d];
#pragma unroll
      for (int n = 0; n < NVAR; ++n) q[n * fxb->ns[d]] = F[n];
    }
  }
  __syncthreads();
  if (d == 2 && zc.save) {  // top face layer and top slope layer, for the next tile of the column
    const int nl = nf0 * nf1;
    for (int l = threadIdx.x; l < nl; l += TL::NT) {
#pragma unroll
      for (int n = 0; n < NVAR; ++n) zc.cflux[n * LAYER + l] = fbuf[n * TL::MAXF + (nf2 - 1) * nl + l];
      if (slopes) {
#pragma unroll
        for (int q = 0; q < NSL; ++q) zc.cslope[q * LAYER + l] = sbuf[q * TL::MAXC + (ne2 - 1) * nl + l];
      }
    }
  }
  if (mine) {
    // pc_flux_div (Diffterm.H:475-481) sums fx1 - fx0 + fy1 - fy0 + fz1 - fz0
    // left to right (AMREX_D_TERM pastes the three differences into one
    // expression); acc holds that running sum, negated and divided at the end.
    const int flo = tx + nf0 * (ty + nf1 * tz);
    const int fhi = flo + ((d == 0) ? 1 : (d == 1) ? nf0 : nf0 * nf1);
#pragma unroll
    for (int n = 0; n < NVAR; ++n)
      acc[n] = d == 0 ? fbuf[n * TL::MAXF + fhi] - fbuf[n * TL::MAXF + flo]
                      : acc[n] + fbuf[n * TL::MAXF + fhi] - fbuf[n * TL::MAXF + flo];
  }
  __syncthreads();
}

// Dynamic shared memory of the FP64 flux pass: face fluxes, cell slopes and
// the z carry (one face layer, one slope layer).
template <int NS, class TL>
constexpr size_t flux_smem_bytes() {
  return sizeof(double) * ((size_t)(7 + NS) * TL::MAXF + (size_t)(4 + NS) * TL::MAXC +
                           (size_t)(7 + NS + 4 + NS) * TL::TX * TL::TY);
}

// Pass 2 over the tile list.  CTA b takes the contiguous share
// [b n / G, (b + 1) n / G) of the n tiles (G = gridDim.x): one tile each when
// G = n; in a persistent launch (as many CTAs as fit on the GPU at once) a
// run of tiles.  The list holds each column of a box's tiles bottom to top,
// so consecutive tiles of a run are mostly z neighbours, and the z pass hands
// its top face and slope layers on (ZCarry) instead of having them evaluated
// again: a tile of 8x8x4 cells then evaluates 4 z face layers and 4 z slope
// layers instead of 5 and 6.
//
// kExact = false: the fast pass (quotients by div_fast); kExact = true: its
// exact twin, which returns at once unless the fast pass counted a lane that
// needs a real division, and then evaluates again, with IEEE quotients, the
// tiles the fast pass marked (bit for bit what the fast pass gives where it
// needs none).
template <int NS, class EOS, class TL = TileDefault, bool kExact = false>
__global__ void __launch_bounds__(TL::NT, TL::MINB)
    flux_kernel(const DevBox* __restrict__ boxes, const int4* __restrict__ tiles, int ntiles,
                const __grid_constant__ DevMech<NS> m, const DevFlags f, const Geo g,
                unsigned long long* __restrict__ counters, const FluxBox* __restrict__ fluxes) {
  constexpr int NVAR = 7 + NS;
  if (kExact && __ldcg(&counters[kCounterSlowFlux]) == 0ull) return;
  Quot<kExact> quo;
  extern __shared__ double flux_dyn_smem[];
  double* fbuf = flux_dyn_smem;
  const int tx = threadIdx.x % TL::TX, ty = (threadIdx.x / TL::TX) % TL::TY, tz = threadIdx.x / (TL::TX * TL::TY);
  ZCarry zc;
  zc.cflux = fbuf + (size_t)NVAR * TL::MAXF + (size_t)(4 + NS) * TL::MAXC;
  zc.cslope = zc.cflux + (size_t)NVAR * TL::TX * TL::TY;
  const int t0 = (int)((long long)blockIdx.x * ntiles / gridDim.x);
  const int t1 = (int)((long long)(blockIdx.x + 1) * ntiles / gridDim.x);
  // the next tile continues tile a's column: same box and x/y origin, z origin one tile up
  auto continues = [&](int a) {
    const int4 p = tiles[a], q = tiles[a + 1];
    return q.x == p.x && q.y == p.y && q.z == p.z && q.w == p.w + TL::TZ;
  };
  bool any_slow = false;     // a lane of this CTA met operands div_fast does not cover
  bool carried_slow = false;  // ... in the tile whose z face and slope layers this one takes over
  for (int tb = t0; tb < t1; ++tb) {
    const int4 t = tiles[tb];
    const DevBox& b = boxes[t.x];
    const int o[3] = {t.y, t.z, t.w};
    // The RHS of the tile's first cell, component 0: the fast pass leaves
    // kSlowRecord there in a tile whose quotients need an IEEE division, and
    // the exact twin evaluates only those tiles again (without the z carry).
    double* r0 = b.R + (o[0] - b.rb[0]) + (long long)(o[1] - b.rb[1]) * b.rj + (long long)(o[2] - b.rb[2]) * b.rk;
    if (kExact && __double_as_longlong(*(volatile double*)r0) != kSlowRecord) continue;
    const int ext[3] = {min(TL::TX, b.hi[0] - o[0] + 1), min(TL::TY, b.hi[1] - o[1] + 1),
                        min(TL::TZ, b.hi[2] - o[2] + 1)};
    const bool mine = tx < ext[0] && ty < ext[1] && tz < ext[2];
    const long long stv[3] = {1, b.n2[0], (long long)b.n2[0] * b.n2[1]};
    double acc[NVAR];
#pragma unroll
    for (int n = 0; n < NVAR; ++n) acc[n] = 0.0;
    const FluxBox* fxb = fluxes ? fluxes + t.x : nullptr;
    zc.carry = !kExact && tb > t0 && continues(tb - 1);
    zc.save = !kExact && tb + 1 < t1 && continues(tb);
    quo.slow = false;
    dir_pass<NS, EOS, 0, TL>(b, m, f, g, o, ext, stv, mine, tx, ty, tz, fbuf, acc, fxb, zc, quo);
    dir_pass<NS, EOS, 1, TL>(b, m, f, g, o, ext, stv, mine, tx, ty, tz, fbuf, acc, fxb, zc, quo);
    dir_pass<NS, EOS, 2, TL>(b, m, f, g, o, ext, stv, mine, tx, ty, tz, fbuf, acc, fxb, zc, quo);
    bool bad = false;
    if (mine) {
      const int i = o[0] + tx, j = o[1] + ty, k = o[2] + tz;
      double* r = b.R + (i - b.rb[0]) + (long long)(j - b.rb[1]) * b.rj + (long long)(k - b.rb[2]) * b.rk;
#pragma unroll
      for (int n = 0; n < NVAR; ++n) {
        const double v = quo(-acc[n], g.vol, g.ivol);  // = -acc[n] / vol, correctly rounded
        bad |= !isfinite(v);
        r[n * b.rn] = v;
      }
    }
    if (!kExact) {  // the exact twin re-evaluates tiles the fast pass has counted already
      // a tile is marked when one of its own lanes, or the tile it carried
      // from, met an operand that needs an IEEE division
      const bool tile_slow = __syncthreads_or(quo.slow) != 0 || carried_slow;
      if (tile_slow && threadIdx.x == 0) *r0 = __longlong_as_double(kSlowRecord);  // after the cell's own write
      any_slow |= quo.slow;
      carried_slow = tile_slow && zc.save;
      if (f.check_output) warp_count(&counters[kCounterNonfinite], bad);
      if (threadIdx.x == 0) atomicAdd(&counters[kCounterCells], (unsigned long long)(ext[0] * ext[1] * ext[2]));
    }
  }
  if (!kExact) warp_count(&counters[kCounterSlowFlux], any_slow);
}

// Host: CTAs of a kernel that are resident on the current device at once
// (the grid of a persistent launch); cached per device by the caller.
template <class K>
inline int resident_ctas(K kernel, int threads, size_t smem) {
  int dev = 0, nsm = 0, nb = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, threads, smem) != cudaSuccess) return 0;
  return nb > 0 ? nb * nsm : nsm;
}

// Host: opt the flux kernel into its dynamic shared memory (more than the
// default 48 KB) on the current device, once per device; then launch it, one
// CTA per tile or (persistent) as many CTAs as are resident at once.
template <int NS, class EOS, class TL = TileDefault>
inline cudaError_t launch_flux_fp64(const DevBox* boxes, const int4* tiles, int ntiles, const DevMech<NS>& m,
                                    const DevFlags& f, const Geo& g, unsigned long long* counters, cudaStream_t s,
                                    const FluxBox* fluxes = nullptr, bool persistent = false) {
  static std::atomic<unsigned long long> opted{0};  // bit per device
  static std::atomic<int> resident[64];             // persistent grid per device (0: not known yet)
  constexpr size_t smem = flux_smem_bytes<NS, TL>();
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = (dev >= 0 && dev < 64) ? (1ull << dev) : 0ull;
  if (!bit || !(opted.load() & bit)) {
    e = cudaFuncSetAttribute(flux_kernel<NS, EOS, TL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    opted.fetch_or(bit);
  }
  if (ntiles <= 0) return cudaSuccess;
  int grid = ntiles;
  if (persistent) {
    int r = bit ? resident[dev].load() : 0;
    if (r <= 0) {
      r = resident_ctas(flux_kernel<NS, EOS, TL>, TL::NT, smem);
      if (bit && r > 0) resident[dev].store(r);
    }
    if (r > 0 && r < grid) grid = r;
  }
  flux_kernel<NS, EOS, TL><<<grid, TL::NT, smem, s>>>(boxes, tiles, ntiles, m, f, g, counters, fluxes);
  return cudaGetLastError();
}

// Host: the exact twin of the flux pass (flux_kernel with kExact), launched
// after the fast pass of any tile shape; persistent, at the default tile
// shape (every shape gives the same result).  Its CTAs return at once unless
// the fast pass counted a lane that needs a real division.  Not needed in the
// PC_PRECISION_FP64_RCP compilation.
template <int NS, class EOS>
inline cudaError_t launch_flux_exact(const DevBox* boxes, const int4* tiles, int ntiles, const DevMech<NS>& m,
                                     const DevFlags& f, const Geo& g, unsigned long long* counters, cudaStream_t s,
                                     const FluxBox* fluxes = nullptr) {
#ifdef PCG_RECIPROCAL_QUOTIENTS
  (void)boxes, (void)tiles, (void)ntiles, (void)m, (void)f, (void)g, (void)counters, (void)s, (void)fluxes;
  return cudaSuccess;
#else
  using TL = TileDefault;
  static std::atomic<unsigned long long> opted{0};
  static std::atomic<int> resident[64];
  constexpr size_t smem = flux_smem_bytes<NS, TL>();
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = (dev >= 0 && dev < 64) ? (1ull << dev) : 0ull;
  if (!bit || !(opted.load() & bit)) {
    e = cudaFuncSetAttribute(flux_kernel<NS, EOS, TL, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    opted.fetch_or(bit);
  }
  if (ntiles <= 0) return cudaSuccess;
  int r = bit ? resident[dev].load() : 0;
  if (r <= 0) {
    r = resident_ctas(flux_kernel<NS, EOS, TL, true>, TL::NT, smem);
    if (bit && r > 0) resident[dev].store(r);
  }
  const int grid = (r > 0 && r < ntiles) ? r : ntiles;
  flux_kernel<NS, EOS, TL, true><<<grid, TL::NT, smem, s>>>(boxes, tiles, ntiles, m, f, g, counters, fluxes);
  return cudaGetLastError();
#endif
}

}  // namespace PCG_NAMESPACE
