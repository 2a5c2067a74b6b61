// AMReX_EBCellFlag.H — ORACLE test infrastructure: the AMReX header of this name, reduced
// to the restated types of amrex_shim.H (oracle/ref_build.py only).
#pragma once
#include "amrex_shim.H"
