// pc_rhs_rcp.cu — the FP64 right-hand side (both passes, every flux-pass
// launch configuration) compiled with PCG_RECIPROCAL_QUOTIENTS: a quotient by
// a divisor shared by several numerators (mass fractions Y_k = rhoY_k / rho,
// the characteristic slopes' 1/c and 1/c^2, the face states' renormalisation,
// the Riemann weights 1/(w_L + w_R), the divergence's 1/V) is the product with
// the correctly rounded reciprocal, within one ulp of the correctly rounded
// quotient that the default FP64 form (and the CPU restatement) computes.
// Every other operation is the default form's, in the same order, compiled
// like it without multiply-add contraction.
#define PCG_NAMESPACE pcg_rcp
#define PCG_RECIPROCAL_QUOTIENTS 1
#include <cstring>

#include "pc_kernels.cuh"
#include "pc_rcp.h"

namespace pcg_rcp {

namespace {

template <int NS, class EOS, class TR>
cudaError_t launch_passes(const pcg::RcpLaunch& a) {
  DevMech<NS> m;
  DevFlags f;
  Geo g;
  std::memcpy(&m, a.mech, sizeof m);
  std::memcpy(&f, a.flags, sizeof f);
  std::memcpy(&g, a.geo, sizeof g);
  const DevBox* boxes = static_cast<const DevBox*>(a.boxes);
  const int4* tiles = static_cast<const int4*>(a.tiles);
  const FluxBox* fx = static_cast<const FluxBox*>(a.fluxes);
  cudaStream_t s = a.stream;
  if (a.ev[0]) cudaEventRecord(a.ev[0], s);
  if (a.nitems > 0)
    cell_kernel<NS, EOS, TR><<<a.nitems, kCellThreads, 0, s>>>(boxes, static_cast<const int2*>(a.items), m, f,
                                                                 a.counters);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (a.ev[1]) cudaEventRecord(a.ev[1], s);
  const bool p = a.persistent;
  switch (a.tile) {
    case 0: e = launch_flux_fp64<NS, EOS, TileDefault>(boxes, tiles, a.ntiles, m, f, g, a.counters, s, fx, p); break;
    case 1: e = launch_flux_fp64<NS, EOS, TileCube>(boxes, tiles, a.ntiles, m, f, g, a.counters, s, fx, p); break;
    case 2: e = launch_flux_fp64<NS, EOS, TileLong>(boxes, tiles, a.ntiles, m, f, g, a.counters, s, fx, p); break;
    case 3: e = launch_flux_fp64<NS, EOS, TileSmall>(boxes, tiles, a.ntiles, m, f, g, a.counters, s, fx, p); break;
    default: e = cudaErrorInvalidValue;
  }
  if (a.ev[2]) cudaEventRecord(a.ev[2], s);
  return e;
}

}  // namespace

}  // namespace pcg_rcp

namespace pcg {

cudaError_t launch_rhs_rcp(const RcpLaunch& a) {
  if (a.flags_size != sizeof(pcg_rcp::DevFlags) || a.geo_size != sizeof(pcg_rcp::Geo) ||
      a.devbox_size != sizeof(pcg_rcp::DevBox) || a.fluxbox_size != sizeof(pcg_rcp::FluxBox))
    return cudaErrorInvalidValue;
  return pcg_rcp::with_species(a.variant, [&](auto ns) {
    constexpr int NS = decltype(ns)::value;
    using P = pcg_rcp::Physics<NS>;
    if (a.mech_size != sizeof(pcg_rcp::DevMech<NS>)) return cudaErrorInvalidValue;
    return pcg_rcp::launch_passes<NS, typename P::EOS, typename P::TR>(a);
  });
}

}  // namespace pcg
