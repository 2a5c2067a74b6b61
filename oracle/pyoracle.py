"""ORACLE — test infrastructure only.

ctypes front end of the CPU restatement in ``pc_oracle.hpp`` (compiled to
``oracle/_build/libpc_oracle.so`` by ``oracle/build.py``).  Imported only by
tests/, by ``__graft_entry__.smoke()`` and by bench.py's CPU-baseline leg, as
the checker and as the timed CPU baseline; the product never imports it.

Parity status: pinned bit for bit to the reference's own hot-path code
(oracle/refharness.py, tests/test_ref_pinned.py); the EOS, transport and
mechanism data PelePhysics would supply stay unpinned (see pc_oracle.hpp).
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
        lib.oracle_exp_log.argtypes = [c_int, POINTER(c_double), POINTER(c_double), c_longlong]
        lib.oracle_exp_log.restype = None
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


def mol_rhs_fluxes(cfg: abi.PcMolConfig, boxes, nthreads: int = 0):
    """(RHS, [Fx, Fy, Fz]) of each BoxState: the face fluxes times the face
    area on surroundingNodes(valid, d), each (NVAR, nz(+1), ny(+1), nx(+1))."""
    lib = library()
    lib.oracle_mol_rhs_fluxes.argtypes = [POINTER(abi.PcMolConfig), POINTER(abi.PcBoxDesc), c_int,
                                          POINTER(c_double), POINTER(abi.PcArray4), c_int]
    descs, outs, farr = [], [], []
    for st in boxes:
        S = np.ascontiguousarray(st.S, dtype=np.float64)
        nx, ny, nz = st.shape
        R = np.zeros((S.shape[0], nz, ny, nx))
        descs.append(abi.box_desc(st.lo, st.hi, abi.array4(S.ctypes.data, S.shape, st.begin),
                                  abi.array4(R.ctypes.data, R.shape, st.lo)))
        F = [np.zeros((S.shape[0], nz + (d == 2), ny + (d == 1), nx + (d == 0))) for d in range(3)]
        farr += [abi.array4(f.ctypes.data, f.shape, st.lo) for f in F]
        outs.append((S, R, F))
    arr = abi.box_array(descs)
    fx = (abi.PcArray4 * len(farr))(*farr)
    dx = (c_double * 3)(*boxes[0].dx)
    rc = lib.oracle_mol_rhs_fluxes(ctypes.byref(cfg), arr, len(descs), dx, fx, int(nthreads))
    if rc != 0:
        raise RuntimeError(f"oracle_mol_rhs_fluxes failed with code {rc}")
    return [(R, F) for _, R, F in outs]


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


# ---------------------------------------------------------------------------
# Level operations of the MOL advance (oracle side).
# ---------------------------------------------------------------------------
def _state_descs(boxes):
    return abi.box_array([abi.box_desc(st.lo, st.hi, abi.array4(st.S.ctypes.data, st.S.shape, st.begin),
                                       abi.array4(st.S.ctypes.data, st.S.shape, st.begin)) for st in boxes])


def fill_ghosts(boxes, geom: abi.PcGeometry, ngrow: int = 4) -> None:
    """In-place ghost fill of BoxStates that tile the domain."""
    lib = library()
    lib.oracle_fill_ghosts.argtypes = [POINTER(abi.PcBoxDesc), c_int, POINTER(abi.PcGeometry), c_int, c_int]
    for st in boxes:
        assert st.S.flags.c_contiguous and st.S.dtype == np.float64
    rc = lib.oracle_fill_ghosts(_state_descs(boxes), len(boxes), ctypes.byref(geom), ngrow, boxes[0].S.shape[0])
    if rc != 0:
        raise RuntimeError(f"oracle_fill_ghosts failed with code {rc}")


def compute_temp(cfg: abi.PcMolConfig, boxes) -> int:
    """PeleC::computeTemp on the valid cells of BoxStates (in place)."""
    lib = library()
    lib.oracle_compute_temp.argtypes = [POINTER(abi.PcMolConfig), c_int, POINTER(c_int), POINTER(abi.PcArray4),
                                        POINTER(c_longlong)]
    lohi = (c_int * (6 * len(boxes)))()
    arrs = (abi.PcArray4 * len(boxes))()
    for b, st in enumerate(boxes):
        for d in range(3):
            lohi[6 * b + d] = st.lo[d]
            lohi[6 * b + 3 + d] = st.hi[d]
        arrs[b] = abi.array4(st.S.ctypes.data, st.S.shape, st.begin)
    fails = c_longlong(0)
    rc = lib.oracle_compute_temp(ctypes.byref(cfg), len(boxes), lohi, arrs, ctypes.byref(fails))
    if rc != 0:
        raise RuntimeError(f"oracle_compute_temp failed with code {rc}")
    return fails.value


def est_dt(cfg: abi.PcMolConfig, boxes, cfl: float, max_dt: float = 1e30):
    lib = library()
    lib.oracle_est_dt.argtypes = [POINTER(abi.PcMolConfig), POINTER(abi.PcBoxDesc), c_int, POINTER(c_double),
                                  c_double, c_double, POINTER(c_double), POINTER(c_double)]
    dt = c_double(0.0)
    parts = (c_double * 4)()
    dx = (c_double * 3)(*boxes[0].dx)
    rc = lib.oracle_est_dt(ctypes.byref(cfg), _state_descs(boxes), len(boxes), dx, cfl, max_dt, ctypes.byref(dt),
                           parts)
    if rc != 0:
        raise RuntimeError(f"oracle_est_dt failed with code {rc}")
    return dt.value, list(parts)


def _valid(st):
    g = st.ng
    return st.S[:, g:-g, g:-g, g:-g]


def ssprk2_step(cfg: abi.PcMolConfig, boxes, geom: abi.PcGeometry, dt: float):
    """One MOL SSP-RK2 step (PeleC::do_mol_advance without sources) of a list
    of BoxStates; returns the new states (the inputs keep their valid data,
    their ghosts are refilled)."""
    from pelec_gb300 import problems

    fill_ghosts(boxes, geom, boxes[0].ng)
    R = mol_rhs(cfg, boxes)
    new = []
    for st, r in zip(boxes, R):
        S = st.S.copy()
        _valid(problems.BoxState(st.lo, st.hi, S, st.dx))[...] = 1.0 * _valid(st) + dt * r
        new.append(problems.BoxState(st.lo, st.hi, S, st.dx))
    compute_temp(cfg, new)
    fill_ghosts(new, geom, new[0].ng)
    R = mol_rhs(cfg, new)
    for st, old, r in zip(new, boxes, R):
        v = _valid(st)
        v[...] = 0.5 * v + 0.5 * _valid(old)
        v[...] = 1.0 * v + (0.5 * dt) * r
    compute_temp(cfg, new)
    return new


def exp_log(which: int, x: np.ndarray) -> np.ndarray:
    """pc_exp.h's exp (which=0) or log (which=1) of each entry of x."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(x)
    library().oracle_exp_log(int(which), _dptr(x), _dptr(y), x.size)
    return y
