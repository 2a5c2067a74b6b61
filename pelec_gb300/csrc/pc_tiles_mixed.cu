// pc_tiles_mixed.cu — the mixed-precision flux pass at the tile shapes other
// than the default 8x8x4 (which pc_mol_mixed.cu launches itself).  Compiled
// like pc_mol_mixed.cu, with multiply-add contraction on.
#include "pc_mixed.cuh"

namespace pcg {

namespace {

template <int NS, bool MIX>
cudaError_t flux_tile(int tile, bool pers, const DevBox* boxes, const int4* tiles, int ntiles, const MechF<NS>& mf,
                      const DevMech<NS>& md, const DevFlags& f, const Geo& g, unsigned long long* counters,
                      cudaStream_t s) {
  switch (tile) {
    case 1: return launch_flux_mixed_at<NS, MIX, TileCube>(boxes, tiles, ntiles, mf, md, f, g, counters, s, pers);
    case 2: return launch_flux_mixed_at<NS, MIX, TileLong>(boxes, tiles, ntiles, mf, md, f, g, counters, s, pers);
    case 3: return launch_flux_mixed_at<NS, MIX, TileSmall>(boxes, tiles, ntiles, mf, md, f, g, counters, s, pers);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

cudaError_t launch_flux_mixed_tile(int tile, bool persistent, int nspec, const DevBox* boxes, const int4* tiles,
                                   int ntiles, const MechSet& ms, const DevFlags& f, const Geo& g, double p_ref,
                                   unsigned long long* counters, cudaStream_t s) {
  if (ntiles <= 0) return cudaSuccess;
  return with_species(nspec, [&](auto ns) {
    constexpr int NS = decltype(ns)::value;
    const DevMech<NS>& m = ms.get<NS>();
    const MechF<NS> mf = to_float(m, p_ref);
    return flux_tile<NS, Physics<NS>::MIX>(tile, persistent, boxes, tiles, ntiles, mf, m, f, g, counters, s);
  });
}

}  // namespace pcg
