// pc_mol_mixed.cu — launches of the mixed-precision passes (pc_mixed.cuh).
// Compiled separately from pc_mol.cu, with multiply-add contraction on: this
// form is checked against the FP64 oracle by error norms, not bit for bit.
#include "pc_mixed.cuh"

namespace pcg {

cudaError_t launch_flux_mixed_tile(int tile, bool persistent, bool strict, int nspec, const DevBox* boxes,
                                   const int4* tiles, int ntiles, const MechSet& ms, const DevFlags& f, const Geo& g,
                                   double p_ref, unsigned long long* counters, cudaStream_t s, const FluxBox* fx);

// Cell pass, then the flux pass at tile shape `tile` (0 = 8x8x4, launched
// here; the others in pc_tiles_mixed.cu), persistent or one CTA per tile.
// strict: PC_PRECISION_MIXED_FP64 (Newton solve, cell mass fractions and the
// divergence in FP64) instead of their double-float forms.  fx: the face
// fluxes' export (refluxing), or null.
int launch_mixed(int nspec, int tile, bool persistent, bool strict, const DevBox* boxes, const int2* items,
                 int nitems, const int4* tiles, int ntiles, const MechSet& ms, const DevFlags& f, const Geo& g,
                 double p_ref, unsigned long long* counters, cudaStream_t s, cudaEvent_t e0, cudaEvent_t e1,
                 cudaEvent_t e2, const FluxBox* fx) {
  if (e0) cudaEventRecord(e0, s);
  cudaError_t e = with_species(nspec, [&](auto ns) {
    constexpr int NS = decltype(ns)::value;
    using P = Physics<NS>;
    const DevMech<NS>& m = ms.get<NS>();
    const MechF<NS> mf = to_float(m, p_ref);
    if (nitems > 0) {
      if (strict)
        cell_kernel_mixed<NS, typename P::EOS, P::MIX, P::MIX, true>
            <<<nitems, kCellThreads, 0, s>>>(boxes, items, m, mf, f, counters);
      else
        cell_kernel_mixed<NS, typename P::EOS, P::MIX, P::MIX, false>
            <<<nitems, kCellThreads, 0, s>>>(boxes, items, m, mf, f, counters);
    }
    if (e1) cudaEventRecord(e1, s);
    if (tile == 0)
      return strict ? launch_flux_mixed_at<NS, P::MIX, TileDefault, true>(boxes, tiles, ntiles, mf, m, f, g, counters,
                                                                          s, persistent, fx)
                    : launch_flux_mixed_at<NS, P::MIX, TileDefault, false>(boxes, tiles, ntiles, mf, m, f, g,
                                                                           counters, s, persistent, fx);
    return cudaSuccess;
  });
  if (tile != 0)
    e = launch_flux_mixed_tile(tile, persistent, strict, nspec, boxes, tiles, ntiles, ms, f, g, p_ref, counters, s,
                               fx);
  if (e2) cudaEventRecord(e2, s);
  return e == cudaSuccess && cudaGetLastError() == cudaSuccess ? 0 : 3;
}

}  // namespace pcg
