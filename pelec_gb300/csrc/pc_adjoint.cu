// pc_adjoint.cu — launches of the adjoint passes (pc_adjoint.cuh).  Compiled
// like pc_mol.cu, without multiply-add contraction, so that the re-evaluated
// forward quantities — and with them every branch decision — are the
// forward pass's own.
#include "pc_adjoint.cuh"

namespace pcg {

cudaError_t launch_vjp_passes(int variant, const DevBox* boxes, const AdjBox* adj, const int2* items, int nitems,
                              const int4* fitems, int nfitems, double* recbar, const long long* recbar_off,
                              const DevMech<1>& m1, const DevMech<9>& m9, const DevFlags& f, const Geo& g,
                              cudaStream_t s) {
  if (variant == 1) {
    if (nfitems > 0)
      face_adjoint_kernel<1, GammaLawEos<1>><<<nfitems, kAdjThreads, 0, s>>>(boxes, adj, fitems, recbar, recbar_off,
                                                                            m1, f, g);
    if (nitems > 0)
      cell_adjoint_kernel<1, GammaLawEos<1>, ConstantTransport<1>>
          <<<nitems, kCellThreads, 0, s>>>(boxes, adj, items, recbar, recbar_off, m1, f);
  } else {
    if (nfitems > 0)
      face_adjoint_kernel<9, IdealMixEos<9>><<<nfitems, kAdjThreads, 0, s>>>(boxes, adj, fitems, recbar, recbar_off,
                                                                            m9, f, g);
    if (nitems > 0)
      cell_adjoint_kernel<9, IdealMixEos<9>, SimpleTransport<9>>
          <<<nitems, kCellThreads, 0, s>>>(boxes, adj, items, recbar, recbar_off, m9, f);
  }
  return cudaGetLastError();
}

}  // namespace pcg
