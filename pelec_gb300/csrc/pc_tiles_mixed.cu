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

cudaError_t launch_flux_mixed_tile(int tile, bool persistent, int variant, const DevBox* boxes, const int4* tiles,
                                   int ntiles, const DevMech<1>& m1, const DevMech<9>& m9, const DevFlags& f,
                                   const Geo& g, double p_ref, unsigned long long* counters, cudaStream_t s) {
  if (ntiles <= 0) return cudaSuccess;
  if (variant == 1) {
    const MechF<1> mf = to_float(m1, p_ref);
    return flux_tile<1, false>(tile, persistent, boxes, tiles, ntiles, mf, m1, f, g, counters, s);
  }
  const MechF<9> mf = to_float(m9, p_ref);
  return flux_tile<9, true>(tile, persistent, boxes, tiles, ntiles, mf, m9, f, g, counters, s);
}

}  // namespace pcg
