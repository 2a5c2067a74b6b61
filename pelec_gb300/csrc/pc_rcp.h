// pc_rcp.h — the call from the driver (pc_mol.cu) into pc_rhs_rcp.cu, the
// second compilation of the FP64 passes with quotients by a shared divisor
// taken as products with its reciprocal (PC_PRECISION_FP64_RCP).  That
// translation unit has its own namespace for the same structures, so they
// cross this call as opaque bytes with their sizes, which it checks.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>

namespace pcg {

struct RcpLaunch {
  int variant;      // species count: 1 (GammaLaw + constant transport), 9 or 21 (ideal mixture + simple transport)
  int tile;         // flux-pass tile shape, 0..3
  bool persistent;  // persistent flux-pass grid
  const void* boxes;  // device DevBox[]
  const void* items;  // device int2[] cell-pass chunks
  int nitems;
  const void* tiles;  // device int4[] flux-pass tiles
  int ntiles;
  const void* mech;  // host DevMech<variant>
  size_t mech_size;
  const void* flags;  // host DevFlags
  size_t flags_size;
  const void* geo;  // host Geo
  size_t geo_size;
  const void* fluxes;  // device FluxBox[] or nullptr
  size_t fluxbox_size, devbox_size;
  unsigned long long* counters;
  cudaStream_t stream;
  cudaEvent_t ev[3];  // recorded before pass 1, between the passes, after pass 2 (each may be null)
};

// Launches both passes on a.stream; cudaSuccess or the first error.
cudaError_t launch_rhs_rcp(const RcpLaunch& a);

}  // namespace pcg
