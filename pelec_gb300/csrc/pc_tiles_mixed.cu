// pc_tiles_mixed.cu — the mixed-precision flux pass at the tile shapes other
// than the default 8x8x4 (which pc_mol_mixed.cu launches itself), for both
// mixed forms.  Compiled like pc_mol_mixed.cu, once per species count
// (pc_unit_ns.h).
#include "pc_mixed.cuh"
#include "pc_unit_ns.h"

namespace pcg {

namespace {

template <int NS, bool MIX, bool STRICT>
cudaError_t flux_tile(int tile, bool pers, const DevBox* boxes, const int4* tiles, int ntiles, const MechF<NS>& mf,
                      const DevMech<NS>& md, const DevFlags& f, const Geo& g, unsigned long long* counters,
                      cudaStream_t s, const FluxBox* fx) {
  switch (tile) {
    case 1:
      return launch_flux_mixed_at<NS, MIX, TileCube, STRICT>(boxes, tiles, ntiles, mf, md, f, g, counters, s, pers, fx);
    case 2:
      return launch_flux_mixed_at<NS, MIX, TileLong, STRICT>(boxes, tiles, ntiles, mf, md, f, g, counters, s, pers, fx);
    case 3:
      return launch_flux_mixed_at<NS, MIX, TileSmall, STRICT>(boxes, tiles, ntiles, mf, md, f, g, counters, s, pers,
                                                               fx);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

template <int NS>
cudaError_t mixed_tile_ns(int tile, bool persistent, bool strict, const DevBox* boxes, const int4* tiles, int ntiles,
                          const DevMech<NS>& m, const DevFlags& f, const Geo& g, double p_ref,
                          unsigned long long* counters, cudaStream_t s, const FluxBox* fx) {
  const MechF<NS> mf = to_float(m, p_ref);
  return strict ? flux_tile<NS, Physics<NS>::MIX, true>(tile, persistent, boxes, tiles, ntiles, mf, m, f, g, counters, s,
                                                        fx)
                : flux_tile<NS, Physics<NS>::MIX, false>(tile, persistent, boxes, tiles, ntiles, mf, m, f, g, counters,
                                                         s, fx);
}

#define PC_MIXED_TILE_INST(NS)                                                                                      \
  template cudaError_t mixed_tile_ns<NS>(int, bool, bool, const DevBox*, const int4*, int, const DevMech<NS>&,     \
                                         const DevFlags&, const Geo&, double, unsigned long long*, cudaStream_t,  \
                                         const FluxBox*);
PC_UNIT_INSTANTIATE(PC_MIXED_TILE_INST)

#if PC_UNIT_HAS(1)  // the dispatcher lives in the one-species compilation
cudaError_t launch_flux_mixed_tile(int tile, bool persistent, bool strict, int nspec, const DevBox* boxes,
                                   const int4* tiles, int ntiles, const MechSet& ms, const DevFlags& f, const Geo& g,
                                   double p_ref, unsigned long long* counters, cudaStream_t s, const FluxBox* fx) {
  if (ntiles <= 0) return cudaSuccess;
  return with_species(nspec, [&](auto ns) {
    constexpr int NS = decltype(ns)::value;
    return mixed_tile_ns<NS>(tile, persistent, strict, boxes, tiles, ntiles, ms.get<NS>(), f, g, p_ref, counters, s,
                             fx);
  });
}
#endif

}  // namespace pcg
