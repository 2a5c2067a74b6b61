// pc_tangent.cu — launches of the tangent passes (pc_tangent.cuh).  Compiled
// without multiply-add contraction: the value part of the Dual arithmetic is
// the FP64 forward's own operation sequence.
#include "pc_tangent.cuh"
#include "pc_unit_ns.h"

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

template <int NS>
cudaError_t jvp_passes_ns(const DevBox* boxes, const TanBox* tans, const int2* items, int nitems, const int4* tiles,
                          int ntiles, const DevMech<NS>& m, const DevFlags& f, const Geo& g,
                          unsigned long long* counters, cudaStream_t s) {
  using P = Physics<NS>;
  return jvp_passes<NS, typename P::EOS, typename P::TR>(boxes, tans, items, nitems, tiles, ntiles, m, f, g, counters,
                                                         s);
}

#define PC_JVP_INST(NS)                                                                                          \
  template cudaError_t jvp_passes_ns<NS>(const DevBox*, const TanBox*, const int2*, int, const int4*, int,        \
                                         const DevMech<NS>&, const DevFlags&, const Geo&, unsigned long long*,   \
                                         cudaStream_t);
PC_UNIT_INSTANTIATE(PC_JVP_INST)

#if PC_UNIT_HAS(1)  // the dispatcher lives in the one-species compilation
cudaError_t launch_jvp_passes(int nspec, const DevBox* boxes, const TanBox* tans, const int2* items, int nitems,
                              const int4* tiles, int ntiles, const MechSet& ms, const DevFlags& f, const Geo& g,
                              unsigned long long* counters, cudaStream_t s) {
  return with_species(nspec, [&](auto ns) {
    constexpr int NS = decltype(ns)::value;
    return jvp_passes_ns<NS>(boxes, tans, items, nitems, tiles, ntiles, ms.get<NS>(), f, g, counters, s);
  });
}
#endif

}  // namespace pcg
