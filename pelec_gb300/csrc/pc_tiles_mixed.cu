// pc_tiles_mixed.cu — the mixed-precision flux pass at the tile shapes other
// than the default 8x8x4 (which pc_mol_mixed.cu launches itself).  Compiled
// like pc_mol_mixed.cu, with multiply-add contraction on.
#include "pc_mixed.cuh"

namespace pcg {

namespace {

template <int NS, bool MIX, class TL>
cudaError_t flux_at(const DevBox* boxes, const int4* tiles, int ntiles, const MechF<NS>& mf, const DevMech<NS>& md,
                    const DevFlags& f, const Geo& g, unsigned long long* counters, cudaStream_t s) {
  constexpr size_t smem = TL::DYN ? sizeof(double) * (7 + NS) * TL::MAXF : 0;
  if (TL::DYN) {
    const cudaError_t e =
        cudaFuncSetAttribute(flux_kernel_mixed<NS, MIX, TL>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  flux_kernel_mixed<NS, MIX, TL><<<ntiles, TL::NT, smem, s>>>(boxes, tiles, mf, md, f, g, counters);
  return cudaGetLastError();
}

template <int NS, bool MIX>
cudaError_t flux_tile(int tile, const DevBox* boxes, const int4* tiles, int ntiles, const MechF<NS>& mf,
                      const DevMech<NS>& md, const DevFlags& f, const Geo& g, unsigned long long* counters,
                      cudaStream_t s) {
  switch (tile) {
    case 1: return flux_at<NS, MIX, TileCube>(boxes, tiles, ntiles, mf, md, f, g, counters, s);
    case 2: return flux_at<NS, MIX, TileLong>(boxes, tiles, ntiles, mf, md, f, g, counters, s);
    case 3: return flux_at<NS, MIX, TileSmall>(boxes, tiles, ntiles, mf, md, f, g, counters, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

cudaError_t launch_flux_mixed_tile(int tile, int variant, const DevBox* boxes, const int4* tiles, int ntiles,
                                   const DevMech<1>& m1, const DevMech<9>& m9, const DevFlags& f, const Geo& g,
                                   double p_ref, unsigned long long* counters, cudaStream_t s) {
  if (ntiles <= 0) return cudaSuccess;
  if (variant == 1) {
    const MechF<1> mf = to_float(m1, p_ref);
    return flux_tile<1, false>(tile, boxes, tiles, ntiles, mf, m1, f, g, counters, s);
  }
  const MechF<9> mf = to_float(m9, p_ref);
  return flux_tile<9, true>(tile, boxes, tiles, ntiles, mf, m9, f, g, counters, s);
}

}  // namespace pcg
