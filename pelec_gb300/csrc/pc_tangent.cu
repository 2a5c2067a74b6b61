// pc_tangent.cu — launches of the tangent passes (pc_tangent.cuh).  Compiled
// without multiply-add contraction: the value part of the Dual arithmetic is
// the FP64 forward's own operation sequence.
#include "pc_tangent.cuh"

#include <atomic>

namespace pcg {

// Each pass fast, then its exact twin (which returns at once unless the fast
// pass counted a lane whose quotients need an IEEE division).  The flux
// kernels' dynamic shared memory (about 79 KB with 9 species) is above the
// default 48 KB: opt both in once per device, and return a refusal at once.
template <int NS, class EOS, class TR>
static cudaError_t jvp_passes(const DevBox* boxes, const TanBox* tans, const int2* items, int nitems,
                              const int4* tiles, int ntiles, const DevMech<NS>& m, const DevFlags& f, const Geo& g,
                              unsigned long long* counters, cudaStream_t s) {
  static std::atomic<unsigned long long> opted{0};  // bit per device
  if (nitems > 0) {
    cell_tangent_kernel<NS, EOS, TR, false><<<nitems, kCellThreads, 0, s>>>(boxes, tans, items, m, f, counters);
    cell_tangent_kernel<NS, EOS, TR, true><<<nitems, kCellThreads, 0, s>>>(boxes, tans, items, m, f, counters);
  }
  if (ntiles > 0) {
    constexpr size_t smem = tangent_smem_bytes<NS>();
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    const unsigned long long bit = (dev >= 0 && dev < 64) ? (1ull << dev) : 0ull;
    if (!bit || !(opted.load() & bit)) {
      e = cudaFuncSetAttribute(flux_tangent_kernel<NS, EOS, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem);
      if (e == cudaSuccess)
        e = cudaFuncSetAttribute(flux_tangent_kernel<NS, EOS, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem);
      if (e != cudaSuccess) return e;
      opted.fetch_or(bit);
    }
    flux_tangent_kernel<NS, EOS, false><<<ntiles, TileTangent::NT, smem, s>>>(boxes, tans, tiles, m, f, g, counters);
    flux_tangent_kernel<NS, EOS, true><<<ntiles, TileTangent::NT, smem, s>>>(boxes, tans, tiles, m, f, g, counters);
  }
  return cudaGetLastError();
}

cudaError_t launch_jvp_passes(int variant, const DevBox* boxes, const TanBox* tans, const int2* items, int nitems,
                              const int4* tiles, int ntiles, const DevMech<1>& m1, const DevMech<9>& m9,
                              const DevFlags& f, const Geo& g, unsigned long long* counters, cudaStream_t s) {
  if (variant == 1)
    return jvp_passes<1, GammaLawEos<1>, ConstantTransport<1>>(boxes, tans, items, nitems, tiles, ntiles, m1, f, g,
                                                               counters, s);
  return jvp_passes<9, IdealMixEos<9>, SimpleTransport<9>>(boxes, tans, items, nitems, tiles, ntiles, m9, f, g,
                                                           counters, s);
}

}  // namespace pcg
