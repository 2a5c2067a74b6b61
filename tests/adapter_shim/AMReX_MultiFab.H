// AMReX_MultiFab.H — test stand-in (tests/test_adapter.py): the parts of
// AMReX's MultiFab, MFIter and Gpu namespace that the PeleC adapter
// (pelec_gb300/adapter/PeleC_GB300.H) uses, over host memory, on top of the
// oracle's restated AMReX basics (oracle/ref_shim/amrex_shim.H).
#pragma once
#include <stdexcept>

#include "amrex_shim.H"

namespace amrex {

using Long = long long;

struct MultiFab {
  std::vector<Box> boxes;  // valid boxes
  int ncomp = 0, ngrow = 0;
  std::vector<FArrayBox> fabs;
  MultiFab(const std::vector<Box>& b, int nc, int ng) : boxes(b), ncomp(nc), ngrow(ng) {
    for (const Box& v : b) fabs.emplace_back(grow(v, ng), nc);
  }
  int nComp() const { return ncomp; }
  int nGrow() const { return ngrow; }
  int local_size() const { return (int)boxes.size(); }
  Array4<const Real> const_array(const struct MFIter& m) const;
  Array4<Real> array(const struct MFIter& m);
};

struct MFIter {
  const MultiFab* mf;
  int i = 0;
  MFIter(const MultiFab& m, bool /*tiling*/) : mf(&m) {}
  bool isValid() const { return i < (int)mf->boxes.size(); }
  MFIter& operator++() {
    ++i;
    return *this;
  }
  Box validbox() const { return mf->boxes[i]; }
  int LocalIndex() const { return i; }
};

inline Array4<const Real> MultiFab::const_array(const MFIter& m) const {
  return const_cast<FArrayBox&>(fabs[m.i]).array();
}
inline Array4<Real> MultiFab::array(const MFIter& m) { return fabs[m.i].array(); }

namespace Gpu {
using gpuStream_t = void*;
inline gpuStream_t gpuStream() { return nullptr; }
}  // namespace Gpu

}  // namespace amrex
