// pc_tangent.cuh — forward-mode tangent (Jacobian-vector product) of the
// FP64 RHS: the passes of pc_kernels.cuh instantiated with Dual numbers
// (pc_dual.cuh).  Values follow the forward's own operation sequence, so the
// tangent kernels also return the RHS itself, bit for bit, and take every
// branch the forward takes; the EOS temperature solve runs the FP64 Newton
// iteration on the values and differentiates the converged T by the
// implicit-function theorem.
#pragma once

#include "pc_dual.cuh"
#include "pc_kernels.cuh"

namespace pcg {

// Value and tangent records: field f of cell c at p[f N + c] and t[f N + c].
template <>
struct RecAcc<Dual> {
  const double* p;
  const double* t;
  long long N;
  __device__ __forceinline__ Dual ld(int fld, long long c) const {
    const long long o = (long long)fld * N + c;
    return Dual(__ldg(p + o), __ldg(t + o));
  }
};

// a / b for a shared divisor: the forward's quotient for the value (div_by,
// div_fast or exact_quotient, as the policy of the pass chooses), and
// (a' - q b') / b for the tangent.
__device__ __forceinline__ Dual div_by(const Dual& a, const Dual& b, const Dual& y) {
  const double q = div_by(a.v, b.v, y.v);
  return Dual(q, (a.d - q * b.d) * y.v);
}
// rcp_q of a dual number: the value rounded as div_fast expects, the
// tangent -b' / b^2.
__device__ __forceinline__ Dual rcp_q(const Dual& b) {
  const double y = rcp_q(b.v);
  return Dual(y, -b.d * y * y);
}
__device__ __forceinline__ Dual rcp_q_from_rn(const Dual& b, const Dual& r) {
  return Dual(rcp_q_from_rn(b.v, r.v), r.d);
}
__device__ __forceinline__ Dual div_fast(const Dual& a, const Dual& b, const Dual& y, bool& slow) {
  const double q = div_fast(a.v, b.v, y.v, slow);
  return Dual(q, (a.d - q * b.d) * y.v);
}
__device__ __forceinline__ Dual exact_quotient(const Dual& a, const Dual& b, const Dual& y) {
  const double q = exact_quotient(a.v, b.v, y.v);
  return Dual(q, (a.d - q * b.d) * y.v);
}

template <class EOS, int NS>
__device__ __forceinline__ Dual rey2t_of(const DevMech<NS>& m, const Dual* Y, Dual rw, Dual e, double Tguess,
                                         int maxit, bool& ok) {
  if constexpr (EOS::kIdealMix) {
    double Yv[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) Yv[k] = Y[k].v;
    const double T = EOS::rey2t(m, Yv, rw.v, e.v, Tguess, maxit, ok);
    // e(T; C(Y), rw(Y)) = e:  cv dT = de - sum_n de/dC_n dC_n + T drw
    const int r = EOS::range(m, T);
    double C[6];
    EOS::coefs(m, Yv, r, C);
    const double cv = EOS::cv_of(C, rw.v, T);
    double s = e.d + T * rw.d;
    double tp = T;
#pragma unroll
    for (int n = 0; n < 6; ++n) {
      double dC = 0.0;
#pragma unroll
      for (int k = 0; k < NS; ++k) dC = fma(Y[k].d, m.cpc[r][n][k], dC);
      const double w = (n < 5) ? tp / (double)(n + 1) : 1.0;
      s -= w * dC;
      tp *= T;
    }
    return Dual(T, s / cv);
  } else {
    return EOS::rey2t(m, Y, rw, e, Tguess, maxit, ok);
  }
}

// kExact as for cell_kernel: the fast pass counts lanes whose quotients need
// an IEEE division; the exact twin returns at once unless there were some.
template <int NS, class EOS, class TR, bool kExact = false>
__global__ void __launch_bounds__(kCellThreads)
    cell_tangent_kernel(const DevBox* __restrict__ boxes, const TanBox* __restrict__ tans,
                        const int2* __restrict__ items, const __grid_constant__ DevMech<NS> m, const DevFlags f,
                        unsigned long long* __restrict__ counters) {
  constexpr int NVAR = 7 + NS;
  if (kExact && __ldcg(&counters[kCounterSlowCell]) == 0ull) return;
  Quot<kExact> quo;
  const int2 it = items[blockIdx.x];
  const DevBox& b = boxes[it.x];
  const TanBox& tb = tans[it.x];
  const long long c = (long long)it.y + threadIdx.x;
  bool newton_fail = false, nonpos = false;
  if (c < b.ncell) {
    int i, j, k;
    cell_index(b, c, i, j, k);
    const double* s = b.S + (i - b.sb[0]) + (long long)(j - b.sb[1]) * b.sj + (long long)(k - b.sb[2]) * b.sk;
    const double* sd = tb.Sd + (i - tb.sb[0]) + (long long)(j - tb.sb[1]) * tb.sj + (long long)(k - tb.sb[2]) * tb.sk;
    Dual U[NVAR];
#pragma unroll
    for (int n = 0; n < NVAR; ++n)
      U[n] = (n == UEINT || n == UTEMP) ? Dual(0.0) : Dual(__ldg(s + n * b.sn), __ldg(sd + n * tb.sn));
    double* r = b.rec + c;
    double* rt = tb.trec + c;
    const long long N = b.ncell;
    // the twin writes again only the records the fast pass marked (kSlowRecord)
    const bool todo = !kExact || __double_as_longlong(r[Rec<NS>::RHO * N]) == kSlowRecord;
    if (todo) {
      cell_record<NS, EOS, TR>(m, f, U, __ldg(s + UTEMP * b.sn), in_grow1(b, i, j, k),
                               [&](int fld, const Dual& v) {
                                 r[fld * N] = v.v;
                                 rt[fld * N] = v.d;
                               },
                               newton_fail, nonpos, quo);
      if (!kExact && quo.slow) r[Rec<NS>::RHO * N] = __longlong_as_double(kSlowRecord);
    }
  }
  if (!kExact) {
    warp_count(&counters[kCounterNewton], newton_fail);
    warp_count(&counters[kCounterNonpos], nonpos);
    warp_count(&counters[kCounterSlowCell], quo.slow);
  }
}

// Flux pass of the tangent on 8x4x4 tiles (the layout's tile list must use
// that shape): per direction, the slopes of the tile's cells and of one
// neighbour layer on each side evaluated once each and staged in shared
// memory, then each face once, staged as Dual, differenced into the cell
// accumulators.
using TileTangent = TileSmall;

// Dynamic shared memory of the tangent flux pass: Dual face fluxes
// (NVAR x MAXF) and Dual cell slopes ((4 + NS) x MAXC).
template <int NS>
constexpr size_t tangent_smem_bytes() {
  return sizeof(double2) * ((size_t)(7 + NS) * TileTangent::MAXF + (size_t)(4 + NS) * TileTangent::MAXC);
}

template <int NS, class EOS, int d, class Q>
__device__ __forceinline__ void dir_pass_tangent(const DevBox& b, const RecAcc<Dual>& ra, const DevMech<NS>& m,
                                                 const DevFlags& f, const Geo& g, const int o[3], const int ext[3],
                                                 const long long stv[3], bool mine, int tx, int ty, int tz,
                                                 Dual* fbuf, Dual* sbuf, Dual* acc, Q& quo) {
  using TL = TileTangent;
  constexpr int NVAR = 7 + NS;
  constexpr int NSL = 4 + NS;
  const bool diff = f.diffuse_vel || f.diffuse_temp || f.diffuse_spec || f.diffuse_enth;
  const bool slopes = f.do_hydro && f.slopes;
  // field q of the slopes of cell ci (tile plus one layer each side in d)
  // at sbuf[q MAXC + ci]
  const int ne0 = ext[0] + 2 * (d == 0), ne1 = ext[1] + 2 * (d == 1), ne2 = ext[2] + 2 * (d == 2);
  if (slopes) {
    const int ncells = ne0 * ne1 * ne2;
    for (int ci = threadIdx.x; ci < ncells; ci += TL::NT) {
      const int ex = ci % ne0, ey = (ci / ne0) % ne1, ez = ci / (ne0 * ne1);
      const int i = o[0] + ex - (d == 0), j = o[1] + ey - (d == 1), k = o[2] + ez - (d == 2);
      const long long c = (i - b.g2lo[0]) + (j - b.g2lo[1]) * stv[1] + (k - b.g2lo[2]) * stv[2];
      Dual sl[NSL];
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
    const long long cR = (i - b.g2lo[0]) + (j - b.g2lo[1]) * stv[1] + (k - b.g2lo[2]) * stv[2];
    Dual F[NVAR];
    if (f.do_hydro) {
      Dual sL[NSL], sR[NSL];
      if (slopes) {
        const int ciL = fx + ne0 * (fy + ne1 * fz);  // the low cell's slot; the high cell is one step on
#pragma unroll
        for (int q = 0; q < NSL; ++q) {
          sL[q] = sbuf[q * TL::MAXC + ciL];
          sR[q] = sbuf[q * TL::MAXC + ciL + cstep];
        }
      } else {
#pragma unroll
        for (int q = 0; q < NSL; ++q) sL[q] = sR[q] = Dual(0.0);
      }
      hydro_face_sl<NS, EOS, d>(ra, m, f, cR, stv[d], g.area[d], sL, sL + 4, sR, sR + 4, F, quo);
    } else {
#pragma unroll
      for (int n = 0; n < NVAR; ++n) F[n] = Dual(0.0);
    }
    if (diff) diffusion_face<NS, EOS, d>(ra, f, g, cR, stv, F);
#pragma unroll
    for (int n = 0; n < NVAR; ++n) fbuf[n * TL::MAXF + fi] = F[n];
  }
  __syncthreads();
  if (mine) {
    const int flo = tx + nf0 * (ty + nf1 * tz);
    const int fhi = flo + ((d == 0) ? 1 : (d == 1) ? nf0 : nf0 * nf1);
#pragma unroll
    for (int n = 0; n < NVAR; ++n)  // the forward's summation order (pc_kernels.cuh dir_pass)
      acc[n] = d == 0 ? fbuf[n * TL::MAXF + fhi] - fbuf[n * TL::MAXF + flo]
                      : acc[n] + fbuf[n * TL::MAXF + fhi] - fbuf[n * TL::MAXF + flo];
  }
  __syncthreads();
}

template <int NS, class EOS, bool kExact = false>
__global__ void __launch_bounds__(TileTangent::NT)
    flux_tangent_kernel(const DevBox* __restrict__ boxes, const TanBox* __restrict__ tans,
                        const int4* __restrict__ tiles, const __grid_constant__ DevMech<NS> m, const DevFlags f,
                        const Geo g, unsigned long long* __restrict__ counters) {
  using TL = TileTangent;
  constexpr int NVAR = 7 + NS;
  if (kExact && __ldcg(&counters[kCounterSlowFlux]) == 0ull) return;
  Quot<kExact> quo;
  extern __shared__ double2 tan_smem_raw[];  // Dual has a constructor: raw storage
  Dual* fbuf = reinterpret_cast<Dual*>(tan_smem_raw);
  Dual* sbuf = fbuf + NVAR * TL::MAXF;
  const int4 t = tiles[blockIdx.x];
  const DevBox& b = boxes[t.x];
  const TanBox& tb = tans[t.x];
  const RecAcc<Dual> ra{b.rec, tb.trec, b.ncell};
  const int o[3] = {t.y, t.z, t.w};
  const int ext[3] = {min(TL::TX, b.hi[0] - o[0] + 1), min(TL::TY, b.hi[1] - o[1] + 1), min(TL::TZ, b.hi[2] - o[2] + 1)};
  const int tx = threadIdx.x % TL::TX, ty = (threadIdx.x / TL::TX) % TL::TY, tz = threadIdx.x / (TL::TX * TL::TY);
  const bool mine = tx < ext[0] && ty < ext[1] && tz < ext[2];
  const long long stv[3] = {1, b.n2[0], (long long)b.n2[0] * b.n2[1]};
  Dual acc[NVAR];
#pragma unroll
  for (int n = 0; n < NVAR; ++n) acc[n] = Dual(0.0);
  dir_pass_tangent<NS, EOS, 0>(b, ra, m, f, g, o, ext, stv, mine, tx, ty, tz, fbuf, sbuf, acc, quo);
  dir_pass_tangent<NS, EOS, 1>(b, ra, m, f, g, o, ext, stv, mine, tx, ty, tz, fbuf, sbuf, acc, quo);
  dir_pass_tangent<NS, EOS, 2>(b, ra, m, f, g, o, ext, stv, mine, tx, ty, tz, fbuf, sbuf, acc, quo);
  if (mine) {
    const int i = o[0] + tx, j = o[1] + ty, k = o[2] + tz;
    double* r = b.R + (i - b.rb[0]) + (long long)(j - b.rb[1]) * b.rj + (long long)(k - b.rb[2]) * b.rk;
    double* rd = tb.Rd + (i - tb.rb[0]) + (long long)(j - tb.rb[1]) * tb.rj + (long long)(k - tb.rb[2]) * tb.rk;
#pragma unroll
    for (int n = 0; n < NVAR; ++n) {
      const Dual v = -acc[n] / g.vol;
      r[n * b.rn] = v.v;
      rd[n * tb.rn] = v.d;
    }
  }
  if (!kExact) warp_count(&counters[kCounterSlowFlux], quo.slow);
}

}  // namespace pcg
