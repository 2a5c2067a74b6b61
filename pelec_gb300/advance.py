"""SSP-RK2 method-of-lines step of one level, as PeleC::do_mol_advance
(Source/Advance.cpp:45-196) without reactions or other sources:

    fill ghosts of S_old;  R = RHS(S_old)
    S_new = S_old + dt R;  computeTemp(S_new)
    fill ghosts of S_new;  R = RHS(S_new)
    S_new = 0.5 S_new + 0.5 S_old;  S_new += 0.5 dt R;  computeTemp(S_new)

``ssprk2_step`` issues every operation as a call into the CUDA library
(mol.MOLOperator); ``Stepper`` replays the same step as one CUDA graph
(pc_mol_step_graph), bit for bit the same arithmetic.  The arrays are
MultiFabs with NG ghost layers (state) and none (RHS).
"""
from __future__ import annotations

from . import mol


def ssprk2_step(op: "mol.MOLOperator", S_old: "mol.MultiFab", S_new: "mol.MultiFab", R: "mol.MultiFab", geom,
                dx, dt: float, stream=None) -> None:
    op.fill_ghosts(S_old, geom, stream=stream)
    op.rhs_level(S_old, R, dx, stream=stream)
    op.lincomb(S_new, 1.0, S_old, dt, R, stream=stream)
    op.compute_temp(S_new, stream=stream)
    op.fill_ghosts(S_new, geom, stream=stream)
    op.rhs_level(S_new, R, dx, stream=stream)
    op.lincomb(S_new, 0.5, S_new, 0.5, S_old, stream=stream)
    op.lincomb(S_new, 1.0, S_new, 0.5 * dt, R, stream=stream)
    op.compute_temp(S_new, stream=stream)


class Stepper:
    """SSP-RK2 steps of a level between two persistent state MultiFabs, one
    CUDA-graph replay per step.  ``step(dt)`` advances the current state into
    the other buffer and makes it current; ``state`` is the current one."""

    def __init__(self, op: "mol.MOLOperator", A: "mol.MultiFab", B: "mol.MultiFab", R: "mol.MultiFab", geom, dx):
        self.graph = op.step_graph(A, B, R, dx, geom)
        self.bufs = (A, B)
        self.cur = 0

    @property
    def state(self) -> "mol.MultiFab":
        return self.bufs[self.cur]

    def step(self, dt: float, stream=None) -> "mol.MultiFab":
        self.graph.launch(dt, reverse=self.cur == 1, stream=stream)
        self.cur = 1 - self.cur
        return self.state

    def close(self) -> None:
        self.graph.close()
