"""Host-side mirror of PeleC's MOL operator interface over the C ABI.

``PeleC::getMOLSrcTerm(const MultiFab& S, MultiFab& MOLSrcTerm, Real time,
Real dt, Real flux_factor)`` (Source/PeleC.H:523-528, Source/Diffusion.cpp:4-681)
is mirrored by :meth:`MOLOperator.getMOLSrcTerm` over :class:`MultiFab`, a
minimal container of device FABs (one torch tensor per box, Array4 layout).
The work itself is done by ``libpelec_mol.so`` (pc_mol_rhs_level); torch only
provides device memory and streams.  There is no CPU fallback: without the
CUDA library or a GPU every call raises.

Error behaviour follows the reference, which aborts on unsupported input
(amrex::Abort, Diffusion.cpp:272,543): a non-zero status code raises
:class:`MOLError` carrying the library's message.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, c_char_p, c_double, c_int, c_void_p

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libpelec_mol.so")
_lib = None


class MOLError(RuntimeError):
    def __init__(self, code: int, where: str):
        super().__init__(f"{where}: {error_string(code)} (code {code})")
        self.code = code


def library() -> ctypes.CDLL:
    """The CUDA library; raises if it has not been built (no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"CUDA library {LIB_PATH} is not built; run `python -m pelec_gb300.build`")
        lib = ctypes.CDLL(LIB_PATH)
        lib.pc_mol_abi_version.restype = c_int
        lib.pc_mol_error_string.argtypes = [c_int]
        lib.pc_mol_error_string.restype = c_char_p
        lib.pc_mol_create.argtypes = [POINTER(c_void_p), POINTER(abi.PcMolConfig)]
        lib.pc_mol_create.restype = c_int
        lib.pc_mol_destroy.argtypes = [c_void_p]
        lib.pc_mol_destroy.restype = None
        for fn in (lib.pc_mol_rhs_level, lib.pc_mol_rhs_level_per_box):
            fn.argtypes = [c_void_p, POINTER(abi.PcBoxDesc), c_int, POINTER(c_double), c_void_p]
            fn.restype = c_int
        lib.pc_mol_last_status.argtypes = [c_void_p, POINTER(abi.PcMolStatus)]
        lib.pc_mol_last_status.restype = c_int
        lib.pc_mol_pass_times.argtypes = [c_void_p, POINTER(c_double), c_int]
        lib.pc_mol_pass_times.restype = c_int
        lib.pc_mol_fill_ghosts.argtypes = [c_void_p, POINTER(abi.PcBoxDesc), c_int, POINTER(abi.PcGeometry), c_int,
                                           c_void_p]
        lib.pc_mol_fill_ghosts.restype = c_int
        lib.pc_mol_lincomb.argtypes = [c_void_p, c_int, POINTER(c_int), POINTER(abi.PcArray4), c_double,
                                       POINTER(abi.PcArray4), c_double, POINTER(abi.PcArray4), c_void_p]
        lib.pc_mol_lincomb.restype = c_int
        lib.pc_mol_compute_temp.argtypes = [c_void_p, c_int, POINTER(c_int), POINTER(abi.PcArray4), c_void_p]
        lib.pc_mol_compute_temp.restype = c_int
        lib.pc_mol_est_dt.argtypes = [c_void_p, POINTER(abi.PcBoxDesc), c_int, POINTER(c_double), c_double, c_double,
                                      POINTER(c_double), c_void_p]
        lib.pc_mol_est_dt.restype = c_int
        lib.pc_mol_graph_create.argtypes = [c_void_p, POINTER(abi.PcBoxDesc), c_int, POINTER(c_double),
                                            POINTER(abi.PcGeometry), c_int, POINTER(c_void_p)]
        lib.pc_mol_graph_create.restype = c_int
        lib.pc_mol_graph_launch.argtypes = [c_void_p, c_void_p]
        lib.pc_mol_graph_launch.restype = c_int
        lib.pc_mol_graph_destroy.argtypes = [c_void_p]
        lib.pc_mol_graph_destroy.restype = None
        lib.pc_mol_graph_status.argtypes = [c_void_p, POINTER(abi.PcMolStatus)]
        lib.pc_mol_graph_status.restype = c_int
        lib.pc_mol_step_graph_create.argtypes = [c_void_p, POINTER(abi.PcBoxDesc), POINTER(abi.PcArray4), c_int,
                                                 POINTER(c_double), POINTER(abi.PcGeometry), c_int, POINTER(c_void_p)]
        lib.pc_mol_step_graph_create.restype = c_int
        lib.pc_mol_step_graph_launch.argtypes = [c_void_p, c_double, c_int, c_void_p]
        lib.pc_mol_step_graph_launch.restype = c_int
        lib.pc_mol_step_graph_status.argtypes = [c_void_p, POINTER(abi.PcMolStatus)]
        lib.pc_mol_step_graph_status.restype = c_int
        lib.pc_mol_step_graph_destroy.argtypes = [c_void_p]
        lib.pc_mol_step_graph_destroy.restype = None
        lib.pc_mol_tile_shape.argtypes = [c_int, POINTER(c_int)]
        lib.pc_mol_tile_shape.restype = c_int
        lib.pc_mol_set_tile.argtypes = [c_void_p, c_int]
        lib.pc_mol_set_tile.restype = c_int
        lib.pc_mol_current_tile.argtypes = [c_void_p, POINTER(c_int)]
        lib.pc_mol_current_tile.restype = c_int
        lib.pc_mol_autotune.argtypes = [c_void_p, POINTER(abi.PcBoxDesc), c_int, POINTER(c_double), c_int,
                                        POINTER(c_int), POINTER(c_double), c_int, c_void_p]
        lib.pc_mol_autotune.restype = c_int
        lib.pc_mol_rhs_level_fluxes.argtypes = [c_void_p, POINTER(abi.PcBoxDesc), c_int, POINTER(c_double),
                                                POINTER(abi.PcArray4), c_void_p]
        lib.pc_mol_rhs_level_fluxes.restype = c_int
        lib.pc_mol_rhs_vjp.argtypes = [c_void_p, POINTER(abi.PcBoxDesc), c_int, POINTER(c_double),
                                       POINTER(abi.PcArray4), POINTER(abi.PcArray4), c_void_p]
        lib.pc_mol_rhs_vjp.restype = c_int
        lib.pc_mol_rhs_jvp.argtypes = [c_void_p, POINTER(abi.PcBoxDesc), c_int, POINTER(c_double),
                                       POINTER(abi.PcArray4), POINTER(abi.PcArray4), c_void_p]
        lib.pc_mol_rhs_jvp.restype = c_int
        lib.pc_mol_fill_ghosts_adjoint.argtypes = lib.pc_mol_fill_ghosts.argtypes
        lib.pc_mol_fill_ghosts_adjoint.restype = c_int
        lib.pc_mol_compute_temp_adjoint.argtypes = [c_void_p, c_int, POINTER(c_int), POINTER(abi.PcArray4),
                                                    POINTER(abi.PcArray4), c_void_p]
        lib.pc_mol_compute_temp_adjoint.restype = c_int
        if lib.pc_mol_abi_version() != abi.PC_MOL_ABI_VERSION:
            raise RuntimeError("libpelec_mol.so ABI version does not match pelec_gb300.abi")
        _lib = lib
    return _lib


def error_string(code: int) -> str:
    try:
        return library().pc_mol_error_string(int(code)).decode()
    except RuntimeError:
        return f"status {code}"


def _check(rc: int, where: str) -> None:
    if rc != abi.PC_OK:
        raise MOLError(rc, where)


class MultiFab:
    """Device FABs of one level: ``fabs[b]`` is a float64 CUDA tensor of shape
    (ncomp, nz+2g, ny+2g, nx+2g) for valid box ``boxes[b] = (lo, hi)``."""

    def __init__(self, boxes, ncomp: int, ngrow: int, device="cuda", fabs=None):
        import torch

        self.boxes = [(tuple(lo), tuple(hi)) for lo, hi in boxes]
        self.ncomp = ncomp
        self.ngrow = ngrow
        if fabs is not None:
            self.fabs = list(fabs)
        else:
            self.fabs = []
            for lo, hi in self.boxes:
                n = [h - l + 1 + 2 * ngrow for l, h in zip(lo, hi)]
                self.fabs.append(torch.zeros((ncomp, n[2], n[1], n[0]), dtype=torch.float64, device=device))

    def array4(self, b: int) -> abi.PcArray4:
        t = self.fabs[b]
        if not t.is_contiguous() or t.dtype.itemsize != 8:
            raise ValueError("FABs must be contiguous float64 tensors")
        lo, _ = self.boxes[b]
        return abi.array4(t.data_ptr(), t.shape, [l - self.ngrow for l in lo])

    def __len__(self):
        return len(self.boxes)


class MOLOperator:
    """One configured MOL right-hand side (a pc_mol_handle)."""

    def __init__(self, cfg: abi.PcMolConfig):
        lib = library()
        self.cfg = cfg
        h = c_void_p()
        _check(lib.pc_mol_create(ctypes.byref(h), ctypes.byref(cfg)), "pc_mol_create")
        self._h = h
        self._descs = None
        self._key = None

    def close(self) -> None:
        if getattr(self, "_h", None) and self._h.value:
            library().pc_mol_destroy(self._h)
            self._h = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _box_descs(self, S: MultiFab, R: MultiFab):
        key = (tuple(t.data_ptr() for t in S.fabs), tuple(t.data_ptr() for t in R.fabs), tuple(S.boxes))
        if key != self._key:
            descs = [abi.box_desc(lo, hi, S.array4(b), R.array4(b)) for b, (lo, hi) in enumerate(S.boxes)]
            self._descs = abi.box_array(descs)
            self._key = key
        return self._descs

    def rhs_level(self, S: MultiFab, R: MultiFab, dx, stream=None, per_box: bool = False) -> None:
        """pc_mol_rhs_level on torch's current stream (or ``stream``)."""
        import torch

        if len(S) != len(R):
            raise ValueError("S and MOLSrcTerm must have the same BoxArray")
        descs = self._box_descs(S, R)
        st = stream if stream is not None else torch.cuda.current_stream()
        dxa = (c_double * 3)(*[float(v) for v in dx])
        fn = library().pc_mol_rhs_level_per_box if per_box else library().pc_mol_rhs_level
        _check(fn(self._h, descs, len(S), dxa, c_void_p(st.cuda_stream)), fn.__name__)

    def rhs_level_fluxes(self, S: MultiFab, R: MultiFab, dx, stream=None):
        """rhs_level plus the face fluxes (times the face areas) for
        refluxing: returns, per box, [Fx, Fy, Fz] as float64 CUDA tensors of
        shape (NVAR, nz(+1), ny(+1), nx(+1)) on surroundingNodes(valid, d)."""
        import torch

        out, arrs = [], []
        for lo, hi in S.boxes:
            n = [h - l + 1 for l, h in zip(lo, hi)]
            F = [torch.empty((S.ncomp, n[2] + (d == 2), n[1] + (d == 1), n[0] + (d == 0)), dtype=torch.float64,
                             device=S.fabs[0].device) for d in range(3)]
            out.append(F)
            arrs += [abi.array4(f.data_ptr(), f.shape, lo) for f in F]
        descs = self._box_descs(S, R)
        dxa = (c_double * 3)(*[float(v) for v in dx])
        fx = (abi.PcArray4 * len(arrs))(*arrs)
        _check(library().pc_mol_rhs_level_fluxes(self._h, descs, len(S), dxa, fx, self._stream(stream)),
               "pc_mol_rhs_level_fluxes")
        return out

    def getMOLSrcTerm(self, S: MultiFab, MOLSrcTerm: MultiFab, time: float, dt: float, flux_factor: float,
                      dx=None) -> None:
        """Mirror of PeleC::getMOLSrcTerm on one level without EB.  ``time`` is
        unused (Diffusion.cpp:8); ``dt`` and ``flux_factor`` only scale flux
        register updates, which are inactive on a single level
        (PeleC.cpp:1432-1439).  ``dx`` is geom.CellSize()."""
        del time, dt, flux_factor
        if dx is None:
            raise ValueError("dx (geom.CellSize()) is required")
        self.rhs_level(S, MOLSrcTerm, dx)

    def pass_times(self):
        """(cell pass ms, flux pass ms) of the last call (cfg.time_passes)."""
        ms = (c_double * 2)()
        _check(library().pc_mol_pass_times(self._h, ms, 2), "pc_mol_pass_times")
        return float(ms[0]), float(ms[1])

    # ---- level operations of the MOL advance ----
    @staticmethod
    def _stream(stream):
        import torch

        return c_void_p((stream if stream is not None else torch.cuda.current_stream()).cuda_stream)

    @staticmethod
    def _lohi(mf: MultiFab):
        arr = (c_int * (6 * len(mf)))()
        for b, (lo, hi) in enumerate(mf.boxes):
            for d in range(3):
                arr[6 * b + d] = lo[d]
                arr[6 * b + 3 + d] = hi[d]
        return arr

    @staticmethod
    def _arrays(mf: MultiFab):
        arr = (abi.PcArray4 * len(mf))()
        for b in range(len(mf)):
            arr[b] = mf.array4(b)
        return arr

    def fill_ghosts(self, S: MultiFab, geom: abi.PcGeometry, ngrow: int | None = None, stream=None) -> None:
        """Fill S's ghost cells from the level's valid data and the domain BCs
        (FillPatcherFill at a single level)."""
        descs = abi.box_array([abi.box_desc(lo, hi, S.array4(b), S.array4(b)) for b, (lo, hi) in enumerate(S.boxes)])
        ng = S.ngrow if ngrow is None else ngrow
        _check(library().pc_mol_fill_ghosts(self._h, descs, len(S), ctypes.byref(geom), ng, self._stream(stream)),
               "pc_mol_fill_ghosts")

    def lincomb(self, dst: MultiFab, a: float, x: MultiFab, b: float, y: MultiFab, stream=None) -> None:
        """dst = a x + b y on the valid cells (MultiFab::LinComb)."""
        _check(library().pc_mol_lincomb(self._h, len(dst), self._lohi(dst), self._arrays(dst), float(a),
                                        self._arrays(x), float(b), self._arrays(y), self._stream(stream)),
               "pc_mol_lincomb")

    def compute_temp(self, S: MultiFab, stream=None) -> None:
        """PeleC::computeTemp on the valid cells."""
        _check(library().pc_mol_compute_temp(self._h, len(S), self._lohi(S), self._arrays(S), self._stream(stream)),
               "pc_mol_compute_temp")

    def est_dt(self, S: MultiFab, dx, cfl: float, max_dt: float = 1e30, stream=None) -> float:
        """PeleC::estTimeStep (synchronous)."""
        descs = abi.box_array([abi.box_desc(lo, hi, S.array4(b), S.array4(b)) for b, (lo, hi) in enumerate(S.boxes)])
        out = c_double(0.0)
        dxa = (c_double * 3)(*[float(v) for v in dx])
        _check(library().pc_mol_est_dt(self._h, descs, len(S), dxa, float(cfl), float(max_dt), ctypes.byref(out),
                                       self._stream(stream)), "pc_mol_est_dt")
        return out.value

    def graph(self, S: MultiFab, R: MultiFab, dx, geom: abi.PcGeometry | None = None,
              ngrow: int | None = None) -> "LevelGraph":
        """CUDA graph of (ghost fill +) RHS on fixed arrays; replay with .launch()."""
        return LevelGraph(self, S, R, dx, geom, S.ngrow if ngrow is None else ngrow)

    def step_graph(self, A: MultiFab, B: MultiFab, R: MultiFab, dx, geom: abi.PcGeometry) -> "StepGraph":
        """CUDA graphs of one SSP-RK2 step between the states A and B (both
        directions) with RHS array R; replay with .launch(dt, reverse)."""
        return StepGraph(self, A, B, R, dx, geom)

    # ---- derivatives ----
    def rhs_vjp(self, S: MultiFab, rhs_bar: MultiFab, state_bar: MultiFab, dx, stream=None) -> None:
        """state_bar = (d RHS / d S)^T rhs_bar on grow(valid, 2) (pc_mol_rhs_vjp).
        rhs_bar has S's BoxArray (valid region); state_bar needs >= 2 ghosts."""
        if state_bar.ngrow < 2:
            raise ValueError("state_bar needs at least 2 ghost cells")
        descs = self._box_descs(S, rhs_bar)
        dxa = (c_double * 3)(*[float(v) for v in dx])
        _check(library().pc_mol_rhs_vjp(self._h, descs, len(S), dxa, self._arrays(rhs_bar), self._arrays(state_bar),
                                        self._stream(stream)), "pc_mol_rhs_vjp")

    def rhs_jvp(self, S: MultiFab, state_dot: MultiFab, R: MultiFab, rhs_dot: MultiFab, dx, stream=None) -> None:
        """R = RHS(S) and rhs_dot = (d RHS / d S) state_dot (pc_mol_rhs_jvp).
        state_dot needs >= 2 ghosts; R and rhs_dot have S's BoxArray."""
        if state_dot.ngrow < 2:
            raise ValueError("state_dot needs at least 2 ghost cells")
        descs = self._box_descs(S, R)
        dxa = (c_double * 3)(*[float(v) for v in dx])
        _check(library().pc_mol_rhs_jvp(self._h, descs, len(S), dxa, self._arrays(state_dot), self._arrays(rhs_dot),
                                        self._stream(stream)), "pc_mol_rhs_jvp")

    def fill_ghosts_adjoint(self, Sbar: MultiFab, geom: abi.PcGeometry, ngrow: int | None = None,
                            stream=None) -> None:
        """Transpose of fill_ghosts on a cotangent MultiFab (ghosts folded
        into the valid cells they were copied from, then zeroed)."""
        descs = abi.box_array([abi.box_desc(lo, hi, Sbar.array4(b), Sbar.array4(b))
                               for b, (lo, hi) in enumerate(Sbar.boxes)])
        ng = Sbar.ngrow if ngrow is None else ngrow
        _check(library().pc_mol_fill_ghosts_adjoint(self._h, descs, len(Sbar), ctypes.byref(geom), ng,
                                                    self._stream(stream)), "pc_mol_fill_ghosts_adjoint")

    def compute_temp_adjoint(self, S: MultiFab, Sbar: MultiFab, stream=None) -> None:
        """Transpose of compute_temp at the post-computeTemp state S, in
        place on the cotangent Sbar."""
        _check(library().pc_mol_compute_temp_adjoint(self._h, len(S), self._lohi(S), self._arrays(S),
                                                     self._arrays(Sbar), self._stream(stream)),
               "pc_mol_compute_temp_adjoint")

    # ---- flux-pass launch configuration (tile shape, persistent or not) ----
    @staticmethod
    def tile_shape(t: int):
        """(tx, ty, tz, threads) of launch configuration t."""
        out = (c_int * 4)()
        _check(library().pc_mol_tile_shape(int(t), out), "pc_mol_tile_shape")
        return tuple(out)

    def set_tile(self, t: int) -> None:
        """Force launch configuration t: tile shape t % PC_NUM_TILES, persistent
        grid when t >= PC_LAUNCH_PERSISTENT (-1: automatic, from the autotune
        cache)."""
        _check(library().pc_mol_set_tile(self._h, int(t)), "pc_mol_set_tile")

    def current_tile(self) -> int:
        out = c_int(0)
        _check(library().pc_mol_current_tile(self._h, ctypes.byref(out)), "pc_mol_current_tile")
        return out.value

    def autotune(self, S: MultiFab, R: MultiFab, dx, reps: int = 3, stream=None):
        """Time every launch configuration on this BoxArray, cache the fastest
        for its box-size histogram; returns (best, [ms per call of each])."""
        descs = self._box_descs(S, R)
        dxa = (c_double * 3)(*[float(v) for v in dx])
        best = c_int(0)
        ms = (c_double * abi.PC_NUM_LAUNCH_CONFIGS)()
        _check(library().pc_mol_autotune(self._h, descs, len(S), dxa, int(reps), ctypes.byref(best), ms,
                                         abi.PC_NUM_LAUNCH_CONFIGS, self._stream(stream)), "pc_mol_autotune")
        return best.value, list(ms)

    def status(self) -> abi.PcMolStatus:
        st = abi.PcMolStatus()
        _check(library().pc_mol_last_status(self._h, ctypes.byref(st)), "pc_mol_last_status")
        return st


class LevelGraph:
    """pc_mol_graph: one launch replays the captured ghost fill and RHS."""

    def __init__(self, op: MOLOperator, S: MultiFab, R: MultiFab, dx, geom, ngrow: int):
        self._op = op  # keeps the handle alive
        self._keep = (S, R)
        descs = abi.box_array([abi.box_desc(lo, hi, S.array4(b), R.array4(b)) for b, (lo, hi) in enumerate(S.boxes)])
        dxa = (c_double * 3)(*[float(v) for v in dx])
        g = c_void_p()
        _check(library().pc_mol_graph_create(op._h, descs, len(S), dxa, ctypes.byref(geom) if geom is not None else None,
                                             int(ngrow), ctypes.byref(g)), "pc_mol_graph_create")
        self._g = g

    def launch(self, stream=None) -> None:
        _check(library().pc_mol_graph_launch(self._g, MOLOperator._stream(stream)), "pc_mol_graph_launch")

    def status(self) -> abi.PcMolStatus:
        """Counters of the last replay (synchronizes its stream)."""
        st = abi.PcMolStatus()
        _check(library().pc_mol_graph_status(self._g, ctypes.byref(st)), "pc_mol_graph_status")
        return st

    def close(self) -> None:
        if getattr(self, "_g", None) and self._g.value:
            library().pc_mol_graph_destroy(self._g)
            self._g = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class StepGraph:
    """pc_mol_step_graph: one launch replays a whole SSP-RK2 step of the level
    (fill, RHS, LinComb, computeTemp, fill, RHS, LinComb, Saxpy, computeTemp),
    from A to B (reverse=False) or from B to A (reverse=True)."""

    def __init__(self, op: MOLOperator, A: MultiFab, B: MultiFab, R: MultiFab, dx, geom: abi.PcGeometry):
        if len(A) != len(B) or len(A) != len(R) or A.ngrow != B.ngrow:
            raise ValueError("A, B and R must share one BoxArray, A and B one ghost width")
        self._op = op  # keeps the parent handle alive
        self._keep = (A, B, R, geom)
        descs = abi.box_array([abi.box_desc(lo, hi, A.array4(b), R.array4(b)) for b, (lo, hi) in enumerate(A.boxes)])
        sb = (abi.PcArray4 * len(B))(*[B.array4(b) for b in range(len(B))])
        dxa = (c_double * 3)(*[float(v) for v in dx])
        g = c_void_p()
        _check(library().pc_mol_step_graph_create(op._h, descs, sb, len(A), dxa, ctypes.byref(geom), int(A.ngrow),
                                                  ctypes.byref(g)), "pc_mol_step_graph_create")
        self._g = g

    def launch(self, dt: float, reverse: bool = False, stream=None) -> None:
        _check(library().pc_mol_step_graph_launch(self._g, float(dt), int(bool(reverse)), MOLOperator._stream(stream)),
               "pc_mol_step_graph_launch")

    def status(self) -> abi.PcMolStatus:
        """Counters of the last replay (synchronizes its stream)."""
        st = abi.PcMolStatus()
        _check(library().pc_mol_step_graph_status(self._g, ctypes.byref(st)), "pc_mol_step_graph_status")
        return st

    def close(self) -> None:
        if getattr(self, "_g", None) and self._g.value:
            library().pc_mol_step_graph_destroy(self._g)
            self._g = c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
