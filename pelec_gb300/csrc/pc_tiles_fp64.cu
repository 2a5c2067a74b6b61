// pc_tiles_fp64.cu — the FP64 flux pass at the tile shapes other than the
// default 8x8x4 (which pc_mol.cu launches itself), persistent or not.  Same arithmetic as
// pc_mol.cu (compiled without multiply-add contraction): the tile shape only
// changes which thread evaluates a face, never the operations on it, so every
// shape gives bit-identical results.
#include "pc_kernels.cuh"

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

cudaError_t launch_flux_fp64_tile(int tile, bool persistent, int variant, const DevBox* boxes, const int4* tiles,
                                  int ntiles, const DevMech<1>& m1, const DevMech<9>& m9, const DevFlags& f,
                                  const Geo& g, unsigned long long* counters, cudaStream_t s, const FluxBox* fx) {
  if (ntiles <= 0) return cudaSuccess;
  if (variant == 1)
    return flux_tile<1, GammaLawEos<1>>(tile, boxes, tiles, ntiles, m1, f, g, counters, s, fx, persistent);
  return flux_tile<9, IdealMixEos<9>>(tile, boxes, tiles, ntiles, m9, f, g, counters, s, fx, persistent);
}

}  // namespace pcg
