"""ctypes mirror of include/pelec_mol.h.

The structures here are byte-for-byte the C structs of the ABI, so the same
objects can be handed to the CUDA library (``libpelec_mol.so``) and to any
other consumer of the header.  Array4 descriptors are built from numpy arrays
(host) or torch tensors (device) laid out as AMReX FArrayBoxes: shape
``(ncomp, nz, ny, nx)`` in C order, i.e. i fastest and the component slowest
(``amrex::Array4``, AMReX_Array4.H).
"""
from __future__ import annotations

import ctypes
from ctypes import c_double, c_int, c_longlong, c_void_p, POINTER

PC_MAX_SPECIES = 21
PC_MOL_ABI_VERSION = 2

PC_OK = 0
PC_ERR_INVALID_ARGUMENT = 1
PC_ERR_UNSUPPORTED = 2
PC_ERR_CUDA = 3
PC_ERR_OUT_OF_MEMORY = 4
PC_ERR_NO_DEVICE = 5
PC_ERR_TOO_LARGE = 6

PC_EOS_GAMMA_LAW = 0
PC_EOS_IDEAL_MIX = 1
PC_TRANSPORT_CONSTANT = 0
PC_TRANSPORT_SIMPLE = 1
PC_PRECISION_FP64 = 0
PC_PRECISION_MIXED = 1
PC_PRECISION_FP64_RCP = 2
PC_PRECISION_MIXED_FP64 = 3

# Conserved-state indices, Source/IndexDefines.H:6-13,60.
URHO, UMX, UMY, UMZ, UEDEN, UEINT, UTEMP, UFS = range(8)

_NS = PC_MAX_SPECIES


class PcMechanism(ctypes.Structure):
    _fields_ = [
        ("nspec", c_int),
        ("pad_", c_int),
        ("mw", c_double * _NS),
        ("gamma", c_double),
        ("nasa_tmid", c_double * _NS),
        ("nasa_lo", (c_double * 7) * _NS),
        ("nasa_hi", (c_double * 7) * _NS),
        ("visc_fit", (c_double * 4) * _NS),
        ("cond_fit", (c_double * 4) * _NS),
        ("diff_fit", ((c_double * 4) * _NS) * _NS),
        ("bulk_ratio", c_double * _NS),
        ("diff_pref", c_double),
        ("const_mu", c_double),
        ("const_xi", c_double),
        ("const_lambda", c_double),
        ("const_rhoD", c_double),
    ]


class PcMolConfig(ctypes.Structure):
    _fields_ = [
        ("nspec", c_int),
        ("eos", c_int),
        ("transport", c_int),
        ("precision", c_int),
        ("do_hydro", c_int),
        ("diffuse_vel", c_int),
        ("diffuse_temp", c_int),
        ("diffuse_spec", c_int),
        ("diffuse_enth", c_int),
        ("plm_iorder", c_int),
        ("use_laxf_flux", c_int),
        ("transport_harmonic_mean", c_int),
        ("check_output", c_int),
        ("newton_max_iter", c_int),
        ("time_passes", c_int),
        ("pad_", c_int),
        ("mixed_p_ref", c_double),
        ("mech", PcMechanism),
    ]


class PcArray4(ctypes.Structure):
    _fields_ = [
        ("p", c_void_p),
        ("jstride", c_longlong),
        ("kstride", c_longlong),
        ("nstride", c_longlong),
        ("begin", c_int * 3),
        ("end", c_int * 3),
        ("ncomp", c_int),
        ("pad_", c_int),
    ]


class PcBoxDesc(ctypes.Structure):
    _fields_ = [
        ("lo", c_int * 3),
        ("hi", c_int * 3),
        ("state", PcArray4),
        ("rhs", PcArray4),
    ]


PC_BC_INTERIOR = 0
PC_BC_OUTFLOW = 1
PC_BC_SYMMETRY = 2
PC_BC_SLIPWALL = 3
PC_BC_NOSLIPWALL = 4

# flux-pass tile shapes (PC_TILE_*): 8x8x4, 8x8x8, 16x8x4, 8x4x4; a launch
# configuration is a shape, + PC_LAUNCH_PERSISTENT for the persistent grid
PC_NUM_TILES = 4
PC_LAUNCH_PERSISTENT = PC_NUM_TILES
PC_NUM_LAUNCH_CONFIGS = 2 * PC_NUM_TILES


class PcGeometry(ctypes.Structure):
    _fields_ = [
        ("domain_lo", c_int * 3),
        ("domain_hi", c_int * 3),
        ("bc_lo", c_int * 3),
        ("bc_hi", c_int * 3),
    ]


def geometry(domain_lo, domain_hi, bc_lo, bc_hi) -> PcGeometry:
    g = PcGeometry()
    for d in range(3):
        g.domain_lo[d] = int(domain_lo[d])
        g.domain_hi[d] = int(domain_hi[d])
        g.bc_lo[d] = int(bc_lo[d])
        g.bc_hi[d] = int(bc_hi[d])
    return g


class PcMolStatus(ctypes.Structure):
    _fields_ = [
        ("cells", c_longlong),
        ("newton_nonconverged", c_longlong),
        ("nonpositive_state", c_longlong),
        ("nonfinite_output", c_longlong),
        ("last_error", c_int),
        ("pad_", c_int),
        ("exact_recomputes", c_longlong),
    ]


def array4(ptr: int, shape, begin) -> PcArray4:
    """Array4 descriptor of a contiguous FAB of ``shape = (ncomp, nz, ny, nx)``
    whose smallEnd is ``begin = (i0, j0, k0)``."""
    nc, nz, ny, nx = (int(s) for s in shape)
    a = PcArray4()
    a.p = ptr
    a.jstride = nx
    a.kstride = nx * ny
    a.nstride = nx * ny * nz
    for d, (b, n) in enumerate(zip(begin, (nx, ny, nz))):
        a.begin[d] = int(b)
        a.end[d] = int(b) + n
    a.ncomp = nc
    return a


def box_desc(lo, hi, state: PcArray4, rhs: PcArray4) -> PcBoxDesc:
    bd = PcBoxDesc()
    for d in range(3):
        bd.lo[d] = int(lo[d])
        bd.hi[d] = int(hi[d])
    bd.state = state
    bd.rhs = rhs
    return bd


def box_array(descs) -> ctypes.Array:
    arr = (PcBoxDesc * len(descs))()
    for i, d in enumerate(descs):
        arr[i] = d
    return arr


__all__ = [n for n in dir() if n.startswith(("Pc", "PC_", "U")) or n in ("array4", "box_desc", "box_array", "geometry")]
_ = POINTER  # re-exported for callers building prototypes
