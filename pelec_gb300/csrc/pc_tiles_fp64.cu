// pc_tiles_fp64.cu — the FP64 flux pass at the tile shapes other than the
// default 8x8x4 (which pc_mol.cu launches itself), persistent or not.  Same arithmetic as
// pc_mol.cu (compiled without multiply-add contraction): the tile shape only
// changes which thread evaluates a face, never the operations on it, so every
// shape gives bit-identical results.
#include "pc_kernels.cuh"
#include "pc_unit_ns.h"

namespace pcg {

namespace {

template <int NS, class EOS, class TL>
cudaError_t flux_at(const DevBox* boxes, const int4* tiles, int ntiles, const DevMech<NS>& m, const DevFlags& f,
                    const Geo& g, unsigned long long* counters, cudaStream_t s, const FluxBox* fx, bool pers) {
  return launch_flux_fp64<NS, EOS, TL>(boxes, tiles, ntiles, m, f, g, counters, s, fx, pers);
}

template <int NS, class EOS>
cudaError_t flux_tile(int tile, const DevBox* boxes, const int4* tiles, int ntiles, const DevMech<NS>& m,
                      const DevFlags& f, const Geo& g, unsigned long long* counters, cudaStream_t s,
                      const FluxBox* fx, bool pers) {
  switch (tile) {
    case 1: return flux_at<NS, EOS, TileCube>(boxes, tiles, ntiles, m, f, g, counters, s, fx, pers);
    case 2: return flux_at<NS, EOS, TileLong>(boxes, tiles, ntiles, m, f, g, counters, s, fx, pers);
    case 3: return flux_at<NS, EOS, TileSmall>(boxes, tiles, ntiles, m, f, g, counters, s, fx, pers);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

template <int NS>
cudaError_t fp64_tile_ns(int tile, bool persistent, const DevBox* boxes, const int4* tiles, int ntiles,
                         const DevMech<NS>& m, const DevFlags& f, const Geo& g, unsigned long long* counters,
                         cudaStream_t s, const FluxBox* fx) {
  return flux_tile<NS, typename Physics<NS>::EOS>(tile, boxes, tiles, ntiles, m, f, g, counters, s, fx, persistent);
}

#define PC_TILE_INST(NS)                                                                                         \
  template cudaError_t fp64_tile_ns<NS>(int, bool, const DevBox*, const int4*, int, const DevMech<NS>&,          \
                                        const DevFlags&, const Geo&, unsigned long long*, cudaStream_t,          \
                                        const FluxBox*);
PC_UNIT_INSTANTIATE(PC_TILE_INST)

#if PC_UNIT_HAS(1)  // the dispatcher lives in the one-species compilation
cudaError_t launch_flux_fp64_tile(int tile, bool persistent, int nspec, const DevBox* boxes, const int4* tiles,
                                  int ntiles, const MechSet& ms, const DevFlags& f, const Geo& g,
                                  unsigned long long* counters, cudaStream_t s, const FluxBox* fx) {
  if (ntiles <= 0) return cudaSuccess;
  return with_species(nspec, [&](auto ns) {
    constexpr int NS = decltype(ns)::value;
    return fp64_tile_ns<NS>(tile, persistent, boxes, tiles, ntiles, ms.get<NS>(), f, g, counters, s, fx);
  });
}
#endif

}  // namespace pcg
