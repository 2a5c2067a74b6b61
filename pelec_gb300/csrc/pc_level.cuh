// pc_level.cuh — level operations of the MOL time advance around the RHS:
// ghost fill, LinComb, computeTemp and the time-step estimate
// (do_mol_advance, Source/Advance.cpp:45-196; estTimeStep, PeleC.cpp:839-972).
// Same FP64 arithmetic rules as the RHS kernels (this header is compiled in
// the translation unit without multiply-add contraction), so computeTemp and
// the time step reproduce the CPU restatement's values.
#pragma once

#include "pc_adjoint.cuh"
#include "pc_kernels.cuh"
#include "pelec_mol.h"

namespace pcg {

// A writable Array4 plus its valid box.
struct LevelBox {
  int lo[3], hi[3];
  double* S;
  long long sj, sk, sn;
  int sb[3];
  int pad;
};

__device__ __forceinline__ double* at(const LevelBox& b, int i, int j, int k) {
  return b.S + (i - b.sb[0]) + (long long)(j - b.sb[1]) * b.sj + (long long)(k - b.sb[2]) * b.sk;
}

struct FillGeom {
  int dlo[3], dhi[3], len[3];
  int bclo[3], bchi[3];
  int periodic[3];
  int ng;
  int nvar;
};

// One thread per cell of grow(valid, ng) of a box; valid cells return.  The
// ghost cell takes the value of the valid cell its index maps to.  items[b]
// = (box, first cell of the 256-cell chunk in the grown box).  ADJ: the
// transpose — the ghost cell's value (a cotangent) is added, with the same
// sign flips, to the valid cell it maps to, and the ghost is zeroed (FP64
// atomics: several ghosts map to one cell).
template <bool ADJ>
__global__ void __launch_bounds__(256) fill_ghosts_kernel(const LevelBox* __restrict__ boxes,
                                                          const int2* __restrict__ items,
                                                          const int* __restrict__ owner, const FillGeom g) {
  const int2 it = items[blockIdx.x];
  const LevelBox& b = boxes[it.x];
  const int gx = b.hi[0] - b.lo[0] + 1 + 2 * g.ng, gy = b.hi[1] - b.lo[1] + 1 + 2 * g.ng;
  const long long gz = b.hi[2] - b.lo[2] + 1 + 2 * g.ng;
  const long long c = (long long)it.y + threadIdx.x;
  if (c >= (long long)gx * gy * gz) return;
  const int idx[3] = {b.lo[0] - g.ng + (int)(c % gx), b.lo[1] - g.ng + (int)((c / gx) % gy),
                      b.lo[2] - g.ng + (int)(c / ((long long)gx * gy))};
  if (idx[0] >= b.lo[0] && idx[0] <= b.hi[0] && idx[1] >= b.lo[1] && idx[1] <= b.hi[1] && idx[2] >= b.lo[2] &&
      idx[2] <= b.hi[2])
    return;
  int src[3];
  double sign[3] = {1.0, 1.0, 1.0};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    int x = idx[d];
    const int lo = g.dlo[d], hi = g.dhi[d];
    if (x < lo || x > hi) {
      const int bc = x < lo ? g.bclo[d] : g.bchi[d];
      if (g.periodic[d]) {
        x = x < lo ? x + g.len[d] : x - g.len[d];
      } else if (bc == PC_BC_OUTFLOW) {
        x = x < lo ? lo : hi;
      } else {
        x = x < lo ? 2 * lo - 1 - x : 2 * hi + 1 - x;
        if (bc == PC_BC_NOSLIPWALL) {
          sign[0] = -sign[0];
          sign[1] = -sign[1];
          sign[2] = -sign[2];
        } else {
          sign[d] = -sign[d];
        }
      }
    }
    src[d] = x;
  }
  int ob = it.x;
  if (owner) {
    const long long o = (src[0] - g.dlo[0]) + (long long)(src[1] - g.dlo[1]) * g.len[0] +
                        (long long)(src[2] - g.dlo[2]) * g.len[0] * g.len[1];
    ob = owner[o];
  }
  const LevelBox& sb = boxes[ob];
  double* s = at(sb, src[0], src[1], src[2]);
  double* dst = at(b, idx[0], idx[1], idx[2]);
  for (int n = 0; n < g.nvar; ++n) {
    if constexpr (ADJ) {
      double v = dst[n * b.sn];
      dst[n * b.sn] = 0.0;
      if (n >= UMX && n <= UMZ) v = v * sign[n - UMX];
      if (v != 0.0) atomicAdd(s + n * sb.sn, v);
    } else {
      double v = s[n * sb.sn];
      if (n >= UMX && n <= UMZ) v = v * sign[n - UMX];
      dst[n * b.sn] = v;
    }
  }
}

// dst = a x + b y on valid cells.  items over valid cells of each box.
struct LinCombArgs {
  const LevelBox* dst;
  const LevelBox* x;
  const LevelBox* y;
  double a, b;
  int nvar;
};

__device__ __forceinline__ bool valid_cell(const LevelBox& b, long long c, int& i, int& j, int& k) {
  const int nx = b.hi[0] - b.lo[0] + 1, ny = b.hi[1] - b.lo[1] + 1;
  const long long nz = b.hi[2] - b.lo[2] + 1;
  if (c >= (long long)nx * ny * nz) return false;
  i = b.lo[0] + (int)(c % nx);
  j = b.lo[1] + (int)((c / nx) % ny);
  k = b.lo[2] + (int)(c / ((long long)nx * ny));
  return true;
}

__global__ void __launch_bounds__(256) lincomb_kernel(const int2* __restrict__ items, const LinCombArgs A) {
  const int2 it = items[blockIdx.x];
  int i, j, k;
  if (!valid_cell(A.dst[it.x], (long long)it.y + threadIdx.x, i, j, k)) return;
  const LevelBox &D = A.dst[it.x], &X = A.x[it.x], &Y = A.y[it.x];
  const double* xp = at(X, i, j, k);
  const double* yp = at(Y, i, j, k);
  double* dp = at(D, i, j, k);
  for (int n = 0; n < A.nvar; ++n) dp[n * D.sn] = A.a * xp[n * X.sn] + A.b * yp[n * Y.sn];
}

// LinComb whose second coefficient is A.b times a scalar read on the device
// (the time step of a captured SSP-RK2 step, written before each replay).
// A.b is 1 or 0.5 there, so the product is exact: the same bits as the
// host-side coefficient of lincomb_kernel.
__global__ void __launch_bounds__(256) lincomb_dt_kernel(const int2* __restrict__ items, const LinCombArgs A,
                                                         const double* __restrict__ dt) {
  const int2 it = items[blockIdx.x];
  int i, j, k;
  if (!valid_cell(A.dst[it.x], (long long)it.y + threadIdx.x, i, j, k)) return;
  const double b = A.b * __ldg(dt);
  const LevelBox &D = A.dst[it.x], &X = A.x[it.x], &Y = A.y[it.x];
  const double* xp = at(X, i, j, k);
  const double* yp = at(Y, i, j, k);
  double* dp = at(D, i, j, k);
  for (int n = 0; n < A.nvar; ++n) dp[n * D.sn] = A.a * xp[n * X.sn] + b * yp[n * Y.sn];
}

__global__ void set_scalar_kernel(double* p, double v) { *p = v; }

// computeTemp: rho e = rho E - rho |u|^2 / 2, then T from e (guess U(UTEMP)).
template <int NS, class EOS>
__global__ void __launch_bounds__(256) compute_temp_kernel(const LevelBox* __restrict__ boxes,
                                                           const int2* __restrict__ items,
                                                           const __grid_constant__ DevMech<NS> m, int maxit,
                                                           unsigned long long* __restrict__ counters) {
  const int2 it = items[blockIdx.x];
  const LevelBox& b = boxes[it.x];
  int i, j, k;
  bool fail = false;
  if (valid_cell(b, (long long)it.y + threadIdx.x, i, j, k)) {
    double* s = at(b, i, j, k);
    const long long sn = b.sn;
    {
      const double rho = s[URHO * sn];
      const double rhoInv = 1.0 / rho;
      const double Up = s[UMX * sn] * rhoInv;
      const double Vp = s[UMY * sn] * rhoInv;
      const double Wp = s[UMZ * sn] * rhoInv;
      const double ke = 0.5 * (Up * Up + Vp * Vp + Wp * Wp);
      s[UEINT * sn] = s[UEDEN * sn] - rho * ke;
    }
    const double rhoInv = 1.0 / s[URHO * sn];
    const double e = s[UEINT * sn] * rhoInv;
    double Y[NS];
#pragma unroll
    for (int n = 0; n < NS; ++n) Y[n] = s[(UFS + n) * sn] * rhoInv;
    bool ok = true;
    const double T = EOS::rey2t(m, Y, mix_rw<NS>(m, Y), e, s[UTEMP * sn], maxit, ok);
    fail = !ok;
    s[UTEMP * sn] = T;
  }
  warp_count(&counters[kCounterNewton], fail);
}

// Transpose of computeTemp on the valid cells.  state holds the state after
// computeTemp (its UTEMP is the converged T); bar holds the cotangent of that
// state and is overwritten with the cotangent of the state before it:
// UEINT and UTEMP were overwritten (cotangent 0), their cotangents flow to
// rho, momentum, rho E and rho Y through rho e = rho E - |m|^2 / (2 rho) and
// the implicit-function theorem on e(T, Y) = e.
template <int NS, class EOS>
__global__ void __launch_bounds__(256) compute_temp_adjoint_kernel(const LevelBox* __restrict__ boxes,
                                                                   const LevelBox* __restrict__ bars,
                                                                   const int2* __restrict__ items,
                                                                   const __grid_constant__ DevMech<NS> m) {
  const int2 it = items[blockIdx.x];
  const LevelBox& b = boxes[it.x];
  const LevelBox& q = bars[it.x];
  int i, j, k;
  if (!valid_cell(b, (long long)it.y + threadIdx.x, i, j, k)) return;
  const double* s = at(b, i, j, k);
  double* o = at(q, i, j, k);
  const long long sn = b.sn, qn = q.sn;
  const double rho = s[URHO * sn];
  const double rhoInv = 1.0 / rho;
  const double mm[3] = {s[UMX * sn], s[UMY * sn], s[UMZ * sn]};
  const double u[3] = {mm[0] * rhoInv, mm[1] * rhoInv, mm[2] * rhoInv};
  const double ke = 0.5 * (u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
  const double rhoe = s[UEDEN * sn] - rho * ke;
  double Y[NS];
#pragma unroll
  for (int n = 0; n < NS; ++n) Y[n] = s[(UFS + n) * sn] * rhoInv;
  const double rw = mix_rw<NS>(m, Y);
  const double T = s[UTEMP * sn];
  // reverse
  double Yb[NS];
#pragma unroll
  for (int n = 0; n < NS; ++n) Yb[n] = 0.0;
  double eb = 0.0, rwb = 0.0;
  EosAdj<NS, EOS>::rey2t(m, Y, rw, T, o[UTEMP * qn], eb, Yb, rwb);
#pragma unroll
  for (int n = 0; n < NS; ++n) Yb[n] += rwb * m.rW[n];
  const double rhoeb = o[UEINT * qn] + eb * rhoInv;  // e = rho e / rho
  double rinvb = eb * rhoe;
#pragma unroll
  for (int n = 0; n < NS; ++n) {
    o[(UFS + n) * qn] += Yb[n] * rhoInv;
    rinvb += Yb[n] * s[(UFS + n) * sn];
  }
  o[UEDEN * qn] += rhoeb;  // rho e = rho E - rho ke
  double rhob = -rhoeb * ke;
  const double keb = -rhoeb * rho;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const double ub = keb * u[c];
    o[(UMX + c) * qn] += ub * rhoInv;
    rinvb += ub * mm[c];
  }
  rhob -= rinvb * rhoInv * rhoInv;
  o[URHO * qn] += rhob;
  o[UEINT * qn] = 0.0;
  o[UTEMP * qn] = 0.0;
}

// Positive doubles order as their bit patterns: atomic minimum on the bits.
__device__ __forceinline__ void atomic_min_pos(unsigned long long* a, double v) {
  atomicMin(a, (unsigned long long)__double_as_longlong(v));
}

// Time-step limits: out[0..3] = min over valid cells of the hydro, viscous,
// thermal and enthalpy limits (pc_estdt_*, Timestep.H:51-237).
template <int NS, class EOS, class TR>
__global__ void __launch_bounds__(256) est_dt_kernel(const LevelBox* __restrict__ boxes,
                                                     const int2* __restrict__ items,
                                                     const __grid_constant__ DevMech<NS> m, const Geo g,
                                                     unsigned long long* __restrict__ out) {
  const int2 it = items[blockIdx.x];
  const LevelBox& b = boxes[it.x];
  const double big = 1.7976931348623157e308;
  double dth = big, dtv = big, dtt = big, dte = big;
  int i, j, k;
  if (valid_cell(b, (long long)it.y + threadIdx.x, i, j, k)) {
    const double* s = at(b, i, j, k);
    const long long sn = b.sn;
    const double rho = s[URHO * sn];
    const double rhoInv = 1.0 / rho;
    double Y[NS];
#pragma unroll
    for (int n = 0; n < NS; ++n) Y[n] = s[(UFS + n) * sn] * rhoInv;
    const double T = s[UTEMP * sn];
    const double rw = mix_rw<NS>(m, Y);
    const double c = EOS::cs_T(m, Y, rw, rho, T, rho * rw * T);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double ud = s[(UMX + d) * sn] * rhoInv;
      dth = fmin(dth, g.dxs[d] / (c + fabs(ud)));
    }
    double X[NS];
    y2x(m, Y, rw, X);
    double tr[NS + 3];
    TR::eval(m, T, rho, rho * rw * T, Y, X, tr);
    double cv;
    if constexpr (EOS::kIdealMix) {
      double C[6];
      IdealMixEos<NS>::coefs(m, Y, IdealMixEos<NS>::range(m, T), C);
      cv = IdealMixEos<NS>::cv_of(C, rw, T);
    } else {
      cv = rw / m.gm1;
    }
    const double cp = cv + rw;
    double Dv = tr[NS] * rhoInv;
    if (Dv == 0.0) Dv = kSmallNum;
    double Dt = tr[NS + 2] * (rhoInv / cv);
    if (Dt == 0.0) Dt = kSmallNum;
    const double De = tr[NS + 2] * (rhoInv / cp);
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double dd = g.dxs[d];
      dtv = fmin(dtv, 0.5 * dd * dd / (3 * Dv));
      dtt = fmin(dtt, 0.5 * dd * dd / (3 * Dt));
      dte = fmin(dte, 0.5 * dd * dd / (3 * De));
    }
  }
  // block reduction then one atomic per block and limit
  __shared__ double red[4][8];
  double v[4] = {dth, dtv, dtt, dte};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    for (int o = 16; o > 0; o >>= 1) v[q] = fmin(v[q], __shfl_down_sync(0xffffffffu, v[q], o));
    if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = v[q];
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double r = red[threadIdx.x][0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) r = fmin(r, red[threadIdx.x][w]);
    atomic_min_pos(&out[threadIdx.x], r);
  }
}

}  // namespace pcg
