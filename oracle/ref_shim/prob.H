// prob.H — ORACLE test infrastructure: the problem header a PeleC case
// supplies, reduced to what the hot-path sources name.  The hooks are the
// defaults of Source/ProblemSpecificFunctions.H:100-161, which do nothing
// (problem_modify_transport_coeffs) or decline (problem_eb_state); the
// problem parameters are empty.  Used by oracle/ref_build.py only.
#pragma once

#include "amrex_shim.H"

struct ProbParmDevice {};

struct RefProblemHooks {
  template <class... A>
  static bool problem_eb_state(A&&...) { return false; }
  template <class... A>
  static void problem_modify_transport_coeffs(A&&...) {}
  template <class... A>
  static void set_isothermal_wall_temperature(A&&...) {}
};
using ProblemSpecificFunctions = RefProblemHooks;
