// pc_adjoint.cu — launches of the adjoint passes (pc_adjoint.cuh).  Compiled
// like pc_mol.cu, without multiply-add contraction, so that the re-evaluated
// forward quantities — and with them every branch decision — are the
// forward pass's own.
#include <algorithm>

#include "pc_adjoint.cuh"
#include "pc_unit_ns.h"

namespace pcg {

// The face adjoint (fast, then its exact twin after clearing the record
// cotangents again, both of which return at once unless the fast pass counted
// a lane that needs a real division), then the cell adjoint.  recbar holds
// nrecbar doubles, cleared by the caller.
template <int NS>
cudaError_t vjp_passes_ns(const DevBox* boxes, const AdjBox* adj, const int2* items, int nitems, const int4* fitems,
                          int nfitems, double* recbar, long long nrecbar, const long long* recbar_off,
                          const DevMech<NS>& m, const DevFlags& f, const Geo& g, unsigned long long* counters,
                          cudaStream_t s) {
  using P = Physics<NS>;
  if (nfitems > 0) {
    face_adjoint_kernel<NS, typename P::EOS, false><<<nfitems, kAdjThreads, 0, s>>>(boxes, adj, fitems, recbar,
                                                                                   recbar_off, m, f, g, counters);
    zero_recbar_if_slow<<<(unsigned)std::min<long long>((nrecbar + 255) / 256, 152LL * 8), 256, 0, s>>>(
        recbar, nrecbar, counters);
    face_adjoint_kernel<NS, typename P::EOS, true><<<nfitems, kAdjThreads, 0, s>>>(boxes, adj, fitems, recbar,
                                                                                  recbar_off, m, f, g, counters);
  }
  if (nitems > 0)
    cell_adjoint_kernel<NS, typename P::EOS, typename P::TR>
        <<<nitems, kCellThreads, 0, s>>>(boxes, adj, items, recbar, recbar_off, m, f);
  return cudaGetLastError();
}

#define PC_VJP_INST(NS)                                                                                          \
  template cudaError_t vjp_passes_ns<NS>(const DevBox*, const AdjBox*, const int2*, int, const int4*, int,       \
                                         double*, long long, const long long*, const DevMech<NS>&,               \
                                         const DevFlags&, const Geo&, unsigned long long*, cudaStream_t);
PC_UNIT_INSTANTIATE(PC_VJP_INST)

#if PC_UNIT_HAS(1)  // the dispatcher lives in the one-species compilation
cudaError_t launch_vjp_passes(int nspec, const DevBox* boxes, const AdjBox* adj, const int2* items, int nitems,
                              const int4* fitems, int nfitems, double* recbar, long long nrecbar,
                              const long long* recbar_off, const MechSet& ms, const DevFlags& f, const Geo& g,
                              unsigned long long* counters, cudaStream_t s) {
  return with_species(nspec, [&](auto ns) {
    constexpr int NS = decltype(ns)::value;
    return vjp_passes_ns<NS>(boxes, adj, items, nitems, fitems, nfitems, recbar, nrecbar, recbar_off, ms.get<NS>(),
                             f, g, counters, s);
  });
}
#endif

}  // namespace pcg
