"""ORACLE — test infrastructure only.

ctypes front end of PeleC's own hot-path code, compiled from the reference
tree by ``oracle/ref_build.py`` into ``oracle/_ref/`` (see ref_harness.cpp
for exactly which reference functions run).  The tests use it to pin the
oracle's restatement (pc_oracle.hpp) to the reference bit for bit; through
that pin the CUDA kernels, which equal the oracle bit for bit, are pinned
too.  Only the parts PelePhysics supplies (EOS, transport, mechanism data)
are not the reference's: the harness runs the oracle's versions of them.

The reference tree is present only where the tests are developed;
``available()`` is False elsewhere (the GPU machines), and the tests that
need it skip there.
"""
from __future__ import annotations

import ctypes
from ctypes import POINTER, c_double, c_int

import numpy as np

from pelec_gb300 import abi

from . import ref_build

_libs: dict = {}


def available() -> bool:
    return ref_build.available()


def library(nspec: int) -> ctypes.CDLL:
    if nspec not in _libs:
        ref_build.build()
        lib = ctypes.CDLL(ref_build.lib_path(nspec))
        lib.ref_nspec.restype = c_int
        lib.ref_mol_rhs.argtypes = [POINTER(abi.PcMolConfig), POINTER(abi.PcBoxDesc), c_int, POINTER(c_double),
                                    POINTER(abi.PcArray4)]
        lib.ref_mol_rhs.restype = c_int
        lib.ref_ctoprim_cell.argtypes = [POINTER(abi.PcMolConfig), POINTER(c_double), POINTER(c_double),
                                         POINTER(c_double)]
        lib.ref_riemann_face.argtypes = [POINTER(abi.PcMolConfig), c_int, POINTER(c_double), POINTER(c_double),
                                         c_double, POINTER(c_double), POINTER(c_double)]
        assert lib.ref_nspec() == nspec
        _libs[nspec] = lib
    return _libs[nspec]


def _dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(POINTER(c_double))


def mol_rhs(cfg: abi.PcMolConfig, boxes, fluxes: bool = False) -> list:
    """The reference's RHS of each BoxState, numpy (NVAR, nz, ny, nx); with
    fluxes=True, (RHS, [Fx, Fy, Fz]) per box like pyoracle.mol_rhs_fluxes."""
    lib = library(cfg.nspec)
    descs, outs, farr = [], [], []
    for st in boxes:
        S = np.ascontiguousarray(st.S, dtype=np.float64)
        nx, ny, nz = st.shape
        R = np.zeros((S.shape[0], nz, ny, nx))
        descs.append(abi.box_desc(st.lo, st.hi, abi.array4(S.ctypes.data, S.shape, st.begin),
                                  abi.array4(R.ctypes.data, R.shape, st.lo)))
        F = [np.zeros((S.shape[0], nz + (d == 2), ny + (d == 1), nx + (d == 0))) for d in range(3)] if fluxes else []
        farr += [abi.array4(f.ctypes.data, f.shape, st.lo) for f in F]
        outs.append((S, R, F))
    arr = abi.box_array(descs)
    fx = (abi.PcArray4 * len(farr))(*farr) if fluxes else None
    dx = (c_double * 3)(*boxes[0].dx)
    rc = lib.ref_mol_rhs(ctypes.byref(cfg), arr, len(descs), dx, fx)
    if rc != 0:
        raise RuntimeError(f"ref_mol_rhs failed with code {rc}")
    return [(R, F) if fluxes else R for _, R, F in outs]


def ctoprim_cell(cfg: abi.PcMolConfig, U: np.ndarray):
    U = np.ascontiguousarray(U, dtype=np.float64)
    q = np.zeros(8 + cfg.nspec)
    qa = np.zeros(6)
    rc = library(cfg.nspec).ref_ctoprim_cell(ctypes.byref(cfg), _dptr(U), _dptr(q), _dptr(qa))
    if rc != 0:
        raise RuntimeError(f"ref_ctoprim_cell failed with code {rc}")
    return q, qa


def riemann_face(cfg: abi.PcMolConfig, left: np.ndarray, right: np.ndarray, cav: float, laxf: bool = False):
    left = np.ascontiguousarray(left, dtype=np.float64)
    right = np.ascontiguousarray(right, dtype=np.float64)
    flux = np.zeros(7 + cfg.nspec)
    us = c_double(0.0)
    rc = library(cfg.nspec).ref_riemann_face(ctypes.byref(cfg), int(laxf), _dptr(left), _dptr(right), cav,
                                             _dptr(flux), ctypes.byref(us))
    if rc != 0:
        raise RuntimeError(f"ref_riemann_face failed with code {rc}")
    return flux, us.value


def compute_temp(cfg: abi.PcMolConfig, boxes) -> None:
    """PeleC::computeTemp (the reference's pc_rst_int_e + pc_cmpTemp) on the
    valid cells of BoxStates, in place."""
    lib = library(cfg.nspec)
    lib.ref_compute_temp.argtypes = [POINTER(abi.PcMolConfig), c_int, POINTER(c_int), POINTER(abi.PcArray4)]
    lohi = (c_int * (6 * len(boxes)))()
    arrs = (abi.PcArray4 * len(boxes))()
    for b, st in enumerate(boxes):
        assert st.S.flags.c_contiguous and st.S.dtype == np.float64
        for d in range(3):
            lohi[6 * b + d] = st.lo[d]
            lohi[6 * b + 3 + d] = st.hi[d]
        arrs[b] = abi.array4(st.S.ctypes.data, st.S.shape, st.begin)
    rc = lib.ref_compute_temp(ctypes.byref(cfg), len(boxes), lohi, arrs)
    if rc != 0:
        raise RuntimeError(f"ref_compute_temp failed with code {rc}")


def est_dt_parts(cfg: abi.PcMolConfig, boxes) -> list:
    """The reference's four estTimeStep cell-limit minima over the boxes'
    valid cells: [hydro, veldif, tempdif, enthdif]."""
    lib = library(cfg.nspec)
    lib.ref_est_dt_parts.argtypes = [POINTER(abi.PcMolConfig), POINTER(abi.PcBoxDesc), c_int, POINTER(c_double),
                                     POINTER(c_double)]
    descs = abi.box_array([abi.box_desc(st.lo, st.hi, abi.array4(st.S.ctypes.data, st.S.shape, st.begin),
                                        abi.array4(st.S.ctypes.data, st.S.shape, st.begin)) for st in boxes])
    parts = (c_double * 4)()
    dx = (c_double * 3)(*boxes[0].dx)
    rc = lib.ref_est_dt_parts(ctypes.byref(cfg), descs, len(boxes), dx, parts)
    if rc != 0:
        raise RuntimeError(f"ref_est_dt_parts failed with code {rc}")
    return list(parts)


FLOP_CLASSES = ("add", "mul", "div", "fma", "sqrt", "exp", "log", "pow", "cmp")
_count_libs: dict = {}


def count_library(nspec: int) -> ctypes.CDLL:
    """The flop-counting build (amrex::Real a counting double)."""
    if nspec not in _count_libs:
        ref_build.build(count=True)
        lib = ctypes.CDLL(ref_build.lib_path(nspec, count=True))
        lib.ref_count_mol_rhs.argtypes = [POINTER(abi.PcMolConfig), POINTER(abi.PcBoxDesc), c_int, POINTER(c_double),
                                          POINTER(ctypes.c_ulonglong)]
        lib.ref_count_mol_rhs.restype = c_int
        _count_libs[nspec] = lib
    return _count_libs[nspec]


def count_mol_rhs(cfg: abi.PcMolConfig, boxes):
    """(counts, RHS list): the floating-point operations of the reference's
    RHS of the BoxStates by class (FLOP_CLASSES), and the RHS it computed
    (the same IEEE operations as mol_rhs)."""
    lib = count_library(cfg.nspec)
    descs, outs = [], []
    for st in boxes:
        S = np.ascontiguousarray(st.S, dtype=np.float64)
        nx, ny, nz = st.shape
        R = np.zeros((S.shape[0], nz, ny, nx))
        descs.append(abi.box_desc(st.lo, st.hi, abi.array4(S.ctypes.data, S.shape, st.begin),
                                  abi.array4(R.ctypes.data, R.shape, st.lo)))
        outs.append((S, R))
    out = (ctypes.c_ulonglong * len(FLOP_CLASSES))()
    dx = (c_double * 3)(*boxes[0].dx)
    rc = lib.ref_count_mol_rhs(ctypes.byref(cfg), abi.box_array(descs), len(descs), dx, out)
    if rc != 0:
        raise RuntimeError(f"ref_count_mol_rhs failed with code {rc}")
    return dict(zip(FLOP_CLASSES, (int(v) for v in out))), [R for _, R in outs]
