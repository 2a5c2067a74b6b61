// pc_tangent.cu — launches of the tangent passes (pc_tangent.cuh).  Compiled
// without multiply-add contraction: the value part of the Dual arithmetic is
// the FP64 forward's own operation sequence.
#include "pc_tangent.cuh"

namespace pcg {

cudaError_t launch_jvp_passes(int variant, const DevBox* boxes, const TanBox* tans, const int2* items, int nitems,
                              const int4* tiles, int ntiles, const DevMech<1>& m1, const DevMech<9>& m9,
                              const DevFlags& f, const Geo& g, unsigned long long* counters, cudaStream_t s) {
  if (variant == 1) {
    if (nitems > 0)
      cell_tangent_kernel<1, GammaLawEos<1>, ConstantTransport<1>>
          <<<nitems, kCellThreads, 0, s>>>(boxes, tans, items, m1, f, counters);
    if (ntiles > 0)
      flux_tangent_kernel<1, GammaLawEos<1>><<<ntiles, TileTangent::NT, 0, s>>>(boxes, tans, tiles, m1, f, g);
  } else {
    if (nitems > 0)
      cell_tangent_kernel<9, IdealMixEos<9>, SimpleTransport<9>>
          <<<nitems, kCellThreads, 0, s>>>(boxes, tans, items, m9, f, counters);
    if (ntiles > 0)
      flux_tangent_kernel<9, IdealMixEos<9>><<<ntiles, TileTangent::NT, 0, s>>>(boxes, tans, tiles, m9, f, g);
  }
  return cudaGetLastError();
}

}  // namespace pcg
