// PeleC.H — ORACLE test infrastructure: stands in for Source/PeleC.H, whose
// class pulls in all of AMReX's AMR machinery, when oracle/ref_build.py
// compiles the hot-path sources.  Those sources need from it only the
// reference's own utility and constant headers (which this file includes
// from the reference tree), the EB types of EB.H and
// PeleC::d_prob_parm_device (MOL.cpp:236).
#pragma once

#include "amrex_shim.H"
#include "PelePhysics.H"
#include "prob.H"
#include "Constants.H"
#include "IndexDefines.H"
#include "Utilities.H"
#include "EB.H"

struct PeleC {
  static ProbParmDevice* d_prob_parm_device;
};
