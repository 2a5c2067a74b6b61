// GradUtil.H — ORACLE test infrastructure: empty stand-in for the reference header
// of this name.  The hot-path functions that oracle/ref_build.py compiles
// (pc_compute_hyp_mol_flux, pc_diffusion_flux and what they call) use
// nothing from it; its own includes need the whole of AMReX.
#pragma once
#include "amrex_shim.H"
