// pc_mol_mixed.cu — launches of the mixed-precision passes (pc_mixed.cuh).
// Compiled separately from pc_mol.cu, with multiply-add contraction on: this
// form is checked against the FP64 oracle by error norms, not bit for bit.
#include "pc_mixed.cuh"

namespace pcg {

cudaError_t launch_flux_mixed_tile(int tile, bool persistent, int variant, const DevBox* boxes, const int4* tiles,
                                   int ntiles, const DevMech<1>& m1, const DevMech<9>& m9, const DevFlags& f,
                                   const Geo& g, double p_ref, unsigned long long* counters, cudaStream_t s);

// Cell pass, then the flux pass at tile shape `tile` (0 = 8x8x4, launched
// here; the others in pc_tiles_mixed.cu), persistent or one CTA per tile.
int launch_mixed(int variant, int tile, bool persistent, const DevBox* boxes, const int2* items, int nitems,
                 const int4* tiles, int ntiles, const DevMech<1>& m1, const DevMech<9>& m9, const DevFlags& f,
                 const Geo& g, double p_ref, unsigned long long* counters, cudaStream_t s, cudaEvent_t e0,
                 cudaEvent_t e1, cudaEvent_t e2) {
  if (e0) cudaEventRecord(e0, s);
  cudaError_t e = cudaSuccess;
  if (variant == 1) {
    const MechF<1> mf = to_float(m1, p_ref);
    if (nitems > 0)
      cell_kernel_mixed<1, GammaLawEos<1>, false, false><<<nitems, kCellThreads, 0, s>>>(boxes, items, m1, mf, f,
                                                                                         counters);
    if (e1) cudaEventRecord(e1, s);
    if (tile == 0)
      e = launch_flux_mixed_at<1, false, TileDefault>(boxes, tiles, ntiles, mf, m1, f, g, counters, s, persistent);
  } else {
    const MechF<9> mf = to_float(m9, p_ref);
    if (nitems > 0)
      cell_kernel_mixed<9, IdealMixEos<9>, true, true><<<nitems, kCellThreads, 0, s>>>(boxes, items, m9, mf, f,
                                                                                       counters);
    if (e1) cudaEventRecord(e1, s);
    if (tile == 0)
      e = launch_flux_mixed_at<9, true, TileDefault>(boxes, tiles, ntiles, mf, m9, f, g, counters, s, persistent);
  }
  if (tile != 0)
    e = launch_flux_mixed_tile(tile, persistent, variant, boxes, tiles, ntiles, m1, m9, f, g, p_ref, counters, s);
  if (e2) cudaEventRecord(e2, s);
  return e == cudaSuccess && cudaGetLastError() == cudaSuccess ? 0 : 3;
}

}  // namespace pcg
