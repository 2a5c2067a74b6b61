// EB.H — ORACLE test infrastructure: stands in for the reference header of
// this name, whose own includes need the whole of AMReX's EB library.  The
// hot-path sources that oracle/ref_build.py compiles need from it only the
// EB stencil and boundary-geometry types, which the reference keeps in
// Source/EBStencilTypes.H (included here from the reference tree).
#pragma once
#include "amrex_shim.H"
#include "EBStencilTypes.H"
