"""ORACLE — test infrastructure only.

ctypes front end of the CPU restatement in ``pc_oracle.hpp`` (compiled to
``oracle/_build/libpc_oracle.so`` by ``oracle/build.py``).  Imported only by
tests/, by ``__graft_entry__.smoke()`` and by bench.py's CPU-baseline leg, as
the checker and as the timed CPU baseline; the product never imports it.

Parity status: UNPINNED (the reference cannot be built in this environment
and ships no RHS-level golden vectors; see pc_oracle.hpp).
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_double, c_int, c_longlong, c_void_p

import numpy as np

from pelec_gb300 import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libpc_oracle.so")
_lib = None


def library() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            from . import build as _build  # noqa: F401  (oracle/build.py)

            _build.build()
        lib = ctypes.CDLL(_LIB_PATH)
        lib.oracle_mol_rhs.argtypes = [POINTER(abi.PcMolConfig), POINTER(abi.PcBoxDesc), c_int, POINTER(c_double),
                                       c_int, POINTER(c_longlong)]
        lib.oracle_mol_rhs.restype = c_int
        lib.oracle_ctoprim_cell.argtypes = [POINTER(abi.PcMolConfig), POINTER(c_double), POINTER(c_double),
                                            POINTER(c_double), POINTER(c_int)]
        lib.oracle_transport_cell.argtypes = [POINTER(abi.PcMolConfig), c_double, c_double, POINTER(c_double),
                                              POINTER(c_double)]
        lib.oracle_thermo.argtypes = [POINTER(abi.PcMolConfig), c_double, POINTER(c_double), POINTER(c_double)]
        lib.oracle_riemann_face.argtypes = [POINTER(abi.PcMolConfig), POINTER(c_double), POINTER(c_double), c_double,
                                            POINTER(c_double), POINTER(c_double)]
        lib.oracle_max_threads.restype = c_int
        _lib = lib
    return _lib


def _dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(POINTER(c_double))


def mol_rhs(cfg: abi.PcMolConfig, boxes, nthreads: int = 0) -> list:
    """RHS of each BoxState (valid region), as numpy arrays (NVAR, nz, ny, nx)."""
    lib = library()
    descs, outs = [], []
    for st in boxes:
        S = np.ascontiguousarray(st.S, dtype=np.float64)
        nx, ny, nz = st.shape
        R = np.zeros((S.shape[0], nz, ny, nx))
        descs.append(abi.box_desc(st.lo, st.hi, abi.array4(S.ctypes.data, S.shape, st.begin),
                                  abi.array4(R.ctypes.data, R.shape, st.lo)))
        outs.append((S, R))
    arr = abi.box_array(descs)
    fails = c_longlong(0)
    dx = (c_double * 3)(*boxes[0].dx)
    rc = lib.oracle_mol_rhs(ctypes.byref(cfg), arr, len(descs), dx, int(nthreads), ctypes.byref(fails))
    if rc != 0:
        raise RuntimeError(f"oracle_mol_rhs failed with code {rc}")
    mol_rhs.last_newton_failures = fails.value
    return [R for _, R in outs]


def mol_rhs_sub(cfg: abi.PcMolConfig, S: np.ndarray, fab_begin, lo, hi, dx, nthreads: int = 0) -> np.ndarray:
    """RHS on the valid box [lo, hi] taken inside a larger state FAB ``S``
    whose smallEnd is ``fab_begin`` (no copy of the state)."""
    lib = library()
    S = np.ascontiguousarray(S, dtype=np.float64)
    shape = tuple(h - l + 1 for l, h in zip(lo, hi))
    R = np.zeros((S.shape[0], shape[2], shape[1], shape[0]))
    d = abi.box_desc(lo, hi, abi.array4(S.ctypes.data, S.shape, fab_begin), abi.array4(R.ctypes.data, R.shape, lo))
    arr = abi.box_array([d])
    fails = c_longlong(0)
    dxa = (c_double * 3)(*dx)
    rc = lib.oracle_mol_rhs(ctypes.byref(cfg), arr, 1, dxa, int(nthreads), ctypes.byref(fails))
    if rc != 0:
        raise RuntimeError(f"oracle_mol_rhs failed with code {rc}")
    return R


def ctoprim_cell(cfg: abi.PcMolConfig, U: np.ndarray):
    U = np.ascontiguousarray(U, dtype=np.float64)
    q = np.zeros(8 + cfg.nspec)
    qa = np.zeros(6)
    ok = c_int(0)
    rc = library().oracle_ctoprim_cell(ctypes.byref(cfg), _dptr(U), _dptr(q), _dptr(qa), ctypes.byref(ok))
    if rc != 0:
        raise RuntimeError(f"oracle_ctoprim_cell failed with code {rc}")
    return q, qa, bool(ok.value)


def transport_cell(cfg: abi.PcMolConfig, T: float, rho: float, Y: np.ndarray) -> np.ndarray:
    Y = np.ascontiguousarray(Y, dtype=np.float64)
    out = np.zeros(cfg.nspec + 3)
    rc = library().oracle_transport_cell(ctypes.byref(cfg), T, rho, _dptr(Y), _dptr(out))
    if rc != 0:
        raise RuntimeError(f"oracle_transport_cell failed with code {rc}")
    return out


def thermo(cfg: abi.PcMolConfig, T: float, Y: np.ndarray) -> np.ndarray:
    Y = np.ascontiguousarray(Y, dtype=np.float64)
    out = np.zeros(4)
    rc = library().oracle_thermo(ctypes.byref(cfg), T, _dptr(Y), _dptr(out))
    if rc != 0:
        raise RuntimeError(f"oracle_thermo failed with code {rc}")
    return out


def riemann_face(cfg: abi.PcMolConfig, left: np.ndarray, right: np.ndarray, cav: float):
    left = np.ascontiguousarray(left, dtype=np.float64)
    right = np.ascontiguousarray(right, dtype=np.float64)
    flux = np.zeros(7 + cfg.nspec)
    us = c_double(0.0)
    rc = library().oracle_riemann_face(ctypes.byref(cfg), _dptr(left), _dptr(right), cav, _dptr(flux),
                                       ctypes.byref(us))
    if rc != 0:
        raise RuntimeError(f"oracle_riemann_face failed with code {rc}")
    return flux, us.value


def max_threads() -> int:
    return int(library().oracle_max_threads())


_ = (c_void_p,)
