// pc_adjoint.cu — launches of the adjoint passes (pc_adjoint.cuh).  Compiled
// like pc_mol.cu, without multiply-add contraction, so that the re-evaluated
// forward quantities — and with them every branch decision — are the
// forward pass's own.
#include <algorithm>

#include "pc_adjoint.cuh"

namespace pcg {

// The face adjoint (fast, then its exact twin after clearing the record
// cotangents again, both of which return at once unless the fast pass counted
// a lane that needs a real division), then the cell adjoint.  recbar holds
// nrecbar doubles, cleared by the caller.
cudaError_t launch_vjp_passes(int variant, const DevBox* boxes, const AdjBox* adj, const int2* items, int nitems,
                              const int4* fitems, int nfitems, double* recbar, long long nrecbar,
                              const long long* recbar_off, const DevMech<1>& m1, const DevMech<9>& m9,
                              const DevFlags& f, const Geo& g, unsigned long long* counters, cudaStream_t s) {
  if (nfitems > 0) {
    if (variant == 1)
      face_adjoint_kernel<1, GammaLawEos<1>, false><<<nfitems, kAdjThreads, 0, s>>>(boxes, adj, fitems, recbar,
                                                                                   recbar_off, m1, f, g, counters);
    else
      face_adjoint_kernel<9, IdealMixEos<9>, false><<<nfitems, kAdjThreads, 0, s>>>(boxes, adj, fitems, recbar,
                                                                                   recbar_off, m9, f, g, counters);
    zero_recbar_if_slow<<<(unsigned)std::min<long long>((nrecbar + 255) / 256, 152LL * 8), 256, 0, s>>>(
        recbar, nrecbar, counters);
    if (variant == 1)
      face_adjoint_kernel<1, GammaLawEos<1>, true><<<nfitems, kAdjThreads, 0, s>>>(boxes, adj, fitems, recbar,
                                                                                  recbar_off, m1, f, g, counters);
    else
      face_adjoint_kernel<9, IdealMixEos<9>, true><<<nfitems, kAdjThreads, 0, s>>>(boxes, adj, fitems, recbar,
                                                                                  recbar_off, m9, f, g, counters);
  }
  if (nitems > 0) {
    if (variant == 1)
      cell_adjoint_kernel<1, GammaLawEos<1>, ConstantTransport<1>>
          <<<nitems, kCellThreads, 0, s>>>(boxes, adj, items, recbar, recbar_off, m1, f);
    else
      cell_adjoint_kernel<9, IdealMixEos<9>, SimpleTransport<9>>
          <<<nitems, kCellThreads, 0, s>>>(boxes, adj, items, recbar, recbar_off, m9, f);
  }
  return cudaGetLastError();
}

}  // namespace pcg
