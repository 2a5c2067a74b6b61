// PelePhysics.H — test stand-in (tests/test_adapter.py): the PelePhysics
// mechanism entry points the adapter reads (get_mw, cp_R, speciesEnthalpy
// of the generated mechanism.H, and the Simple transport's TransParm fits),
// evaluating the table of the test's synthetic mechanism
// (mechanism_table.H, written by the test) with the NASA-7 polynomials.
#pragma once
#include "amrex_shim.H"
#include "mechanism_table.H"

inline void get_mw(amrex::Real* mw) {
  for (int k = 0; k < NUM_SPECIES; ++k) mw[k] = kMW[k];
}
inline void cp_R(amrex::Real* cp, const amrex::Real* tc) {
  const double T = tc[1];
  for (int k = 0; k < NUM_SPECIES; ++k) {
    const double* a = T < kTMID[k] ? kLO[k] : kHI[k];
    cp[k] = a[0] + T * (a[1] + T * (a[2] + T * (a[3] + T * a[4])));
  }
}
inline void speciesEnthalpy(amrex::Real* h, const amrex::Real* tc) {
  const double T = tc[1];
  for (int k = 0; k < NUM_SPECIES; ++k) {
    const double* a = T < kTMID[k] ? kLO[k] : kHI[k];
    h[k] = a[0] + T * (a[1] / 2 + T * (a[2] / 3 + T * (a[3] / 4 + T * a[4] / 5))) + a[5] / T;
  }
}

struct TestTransParm {
  amrex::Real fitmu[NUM_SPECIES * 4], fitlam[NUM_SPECIES * 4], fitdbin[NUM_SPECIES * NUM_SPECIES * 4];
};
