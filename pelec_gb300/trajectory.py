"""Adjoint of an SSP-RK2 trajectory of one level, with checkpointing.

The forward trajectory is N steps of ``advance.ssprk2_step`` (PeleC's
do_mol_advance without sources, Source/Advance.cpp:45-196) with a given,
frozen time-step sequence.  The objective is J = sum over valid cells of
T dV at the final state (T is UTEMP after the last computeTemp).  The
gradient dJ/dU0 is computed in reverse with the transposes of every
operation of a step, each a call into the CUDA library:

    step:   A = fill(S_n);  R0 = RHS(A);  B = A + dt R0;  computeTemp(B)
            fill(B);  R1 = RHS(B);  C = 0.5 B + 0.5 A + 0.5 dt R1;  computeTemp(C)
    adjoint (given Cbar):
            Cbar <- computeTemp^T(C) Cbar
            R1bar = 0.5 dt Cbar;  Bbar = 0.5 Cbar;  Abar = 0.5 Cbar
            Bbar += fill^T(VJP(B, R1bar));  Bbar <- computeTemp^T(B) Bbar
            Abar += Bbar;  R0bar = dt Bbar;  Abar += fill^T(VJP(A, R0bar))

States are kept at every ``every``-th step (checkpoints); the reverse sweep
recomputes each segment forward from its checkpoint, keeping that
segment's stage states (A, B, C per step), and then runs the segment's
adjoint steps backwards.  Memory: (N / every + 3 every) states.

``tangent`` is the forward-mode counterpart: the directional derivative of
J along an initial-state direction, carried through every step with the
dual-number RHS (pc_mol_rhs_jvp), the fill and LinComb applied to the
tangent, and the last computeTemp's transpose for T.  It takes the same
derivative of every branch as the adjoint, so <dJ/dU0, v> and the tangent
agree to round-off wherever the forward map is differentiable or not; a
finite difference differs from both exactly where a limiter or switch is
evaluated at its kink.
"""
from __future__ import annotations

import numpy as np

from . import abi, mol


def _clone(mf: "mol.MultiFab") -> "mol.MultiFab":
    return mol.MultiFab(mf.boxes, mf.ncomp, mf.ngrow, fabs=[t.clone() for t in mf.fabs])


def _zeros_like(mf: "mol.MultiFab", ngrow: int | None = None) -> "mol.MultiFab":
    return mol.MultiFab(mf.boxes, mf.ncomp, mf.ngrow if ngrow is None else ngrow)


class Trajectory:
    """SSP-RK2 trajectory of a level and its adjoint.

    op: mol.MOLOperator (FP64); template: a MultiFab with the level's
    BoxArray and ghost width; geom: abi.PcGeometry for the ghost fill;
    dx: cell size."""

    def __init__(self, op: "mol.MOLOperator", template: "mol.MultiFab", geom, dx, use_graph: bool = True):
        self.op = op
        self.geom = geom
        self.dx = tuple(float(v) for v in dx)
        self.vol = float(np.prod(self.dx))
        self.S_new = _zeros_like(template)
        self.R = _zeros_like(template, 0)
        self.ng = template.ngrow
        self.use_graph = use_graph
        self._stepper = None  # advance.Stepper over two persistent states, made on first use

    def _graph_stepper(self, S0: "mol.MultiFab"):
        from . import advance

        if self._stepper is None:
            A, B = _zeros_like(S0), _zeros_like(S0)
            self._stepper = advance.Stepper(self.op, A, B, _zeros_like(S0, 0), self.geom, self.dx)
        st = self._stepper
        for dst, src in zip(st.state.fabs, S0.fabs):
            dst.copy_(src)
        return st

    # ---- forward ----
    def step(self, S_old: "mol.MultiFab", S_new: "mol.MultiFab", dt: float, keep: bool = False):
        """One SSP-RK2 step S_old -> S_new (advance.ssprk2_step); with keep,
        returns copies of the stage states (A, B, C)."""
        op, R = self.op, self.R
        op.fill_ghosts(S_old, self.geom)
        A = _clone(S_old) if keep else None
        op.rhs_level(S_old, R, self.dx)
        op.lincomb(S_new, 1.0, S_old, dt, R)
        op.compute_temp(S_new)
        op.fill_ghosts(S_new, self.geom)
        B = _clone(S_new) if keep else None
        op.rhs_level(S_new, R, self.dx)
        op.lincomb(S_new, 0.5, S_new, 0.5, S_old)
        op.lincomb(S_new, 1.0, S_new, 0.5 * dt, R)
        op.compute_temp(S_new)
        return (A, B, _clone(S_new)) if keep else None

    def run(self, S0: "mol.MultiFab", dts, every: int = 0):
        """Forward trajectory from S0 (not modified).  Returns the final
        state and the checkpoints {step: state} (every > 0).  With use_graph
        each step is one replay of the step graph (advance.Stepper), the same
        arithmetic as ``step``."""
        ckpt = {}
        if self.use_graph:
            st = self._graph_stepper(S0)
            for n, dt in enumerate(dts):
                if every and n % every == 0:
                    ckpt[n] = _clone(st.state)
                st.step(float(dt))
            return _clone(st.state), ckpt
        S_old, S_new = _clone(S0), _clone(S0)
        for n, dt in enumerate(dts):
            if every and n % every == 0:
                ckpt[n] = _clone(S_old)
            self.step(S_old, S_new, float(dt))
            S_old, S_new = S_new, S_old
        return S_old, ckpt

    def dt_sequence(self, S0: "mol.MultiFab", nsteps: int, cfl: float = 0.3):
        """Time steps of the forward trajectory from S0 at the given CFL
        (estTimeStep before every step); frozen for the gradient."""
        S_old, S_new = _clone(S0), _clone(S0)
        dts = []
        for _ in range(nsteps):
            self.op.fill_ghosts(S_old, self.geom)
            dt = self.op.est_dt(S_old, self.dx, cfl)
            dts.append(dt)
            self.step(S_old, S_new, dt)
            S_old, S_new = S_new, S_old
        return dts

    def objective(self, S: "mol.MultiFab") -> float:
        """J = sum over valid cells of T dV."""
        g = S.ngrow
        tot = 0.0
        for t in S.fabs:
            v = t[abi.UTEMP, g:-g, g:-g, g:-g] if g else t[abi.UTEMP]
            tot += float(v.sum())
        return tot * self.vol

    # ---- forward mode ----
    def tangent(self, S0: "mol.MultiFab", dts, V0: "mol.MultiFab"):
        """(J, dJ): the objective and its derivative along the initial-state
        direction V0 (valid cells; its ghosts, UEINT and UTEMP entries do not
        matter).  Per step, with the state S and its tangent V:
            fill(S), fill(V);  R, Rd = JVP(S, V)
            B = S + dt R,  Vb = V + dt Rd;  computeTemp(B)
            fill(B), fill(Vb); R, Rd = JVP(B, Vb)
            C = 0.5 B + 0.5 S + 0.5 dt R,  Vc = 0.5 Vb + 0.5 V + 0.5 dt Rd;  computeTemp(C)
        The RHS reads UEINT not at all and UTEMP only as its Newton guess, so
        the tangents of those two components (left as LinComb makes them) are
        never used; the final T's tangent is the last computeTemp's transpose
        applied to the cotangent of J, contracted with the last state's
        tangent."""
        op, R = self.op, self.R
        dts = [float(v) for v in dts]
        S_old, S_new = _clone(S0), _clone(S0)
        V_old, V_new = _clone(V0), _zeros_like(V0)
        Rd = _zeros_like(S0, 0)
        for dt in dts:
            op.fill_ghosts(S_old, self.geom)
            op.fill_ghosts(V_old, self.geom)
            op.rhs_jvp(S_old, V_old, R, Rd, self.dx)
            op.lincomb(S_new, 1.0, S_old, dt, R)
            op.lincomb(V_new, 1.0, V_old, dt, Rd)
            op.compute_temp(S_new)
            op.fill_ghosts(S_new, self.geom)
            op.fill_ghosts(V_new, self.geom)
            op.rhs_jvp(S_new, V_new, R, Rd, self.dx)
            op.lincomb(S_new, 0.5, S_new, 0.5, S_old)
            op.lincomb(S_new, 1.0, S_new, 0.5 * dt, R)
            op.lincomb(V_new, 0.5, V_new, 0.5, V_old)
            op.lincomb(V_new, 1.0, V_new, 0.5 * dt, Rd)
            op.compute_temp(S_new)
            S_old, S_new = S_new, S_old
            V_old, V_new = V_new, V_old
        J = self.objective(S_old)
        g = self.ng
        L = _zeros_like(S0)
        for t in L.fabs:
            t[abi.UTEMP, g:-g, g:-g, g:-g] = self.vol
        op.compute_temp_adjoint(S_old, L)
        dJ = 0.0
        for lt, vt in zip(L.fabs, V_old.fabs):
            dJ += float((lt[:, g:-g, g:-g, g:-g] * vt[:, g:-g, g:-g, g:-g]).sum())
        return J, dJ

    # ---- reverse ----
    def _adjoint_step(self, A, B, C, dt: float, Lc: "mol.MultiFab", La: "mol.MultiFab", Lb, Tmp, Rb) -> None:
        op = self.op
        op.compute_temp_adjoint(C, Lc)
        op.lincomb(Rb, 0.5 * dt, Lc, 0.0, Lc)
        op.lincomb(Lb, 0.5, Lc, 0.0, Lc)
        op.lincomb(La, 0.5, Lc, 0.0, Lc)
        op.rhs_vjp(B, Rb, Tmp, self.dx)
        op.fill_ghosts_adjoint(Tmp, self.geom)
        op.lincomb(Lb, 1.0, Lb, 1.0, Tmp)
        op.compute_temp_adjoint(B, Lb)
        op.lincomb(La, 1.0, La, 1.0, Lb)
        op.lincomb(Rb, dt, Lb, 0.0, Lb)
        op.rhs_vjp(A, Rb, Tmp, self.dx)
        op.fill_ghosts_adjoint(Tmp, self.geom)
        op.lincomb(La, 1.0, La, 1.0, Tmp)

    def gradient(self, S0: "mol.MultiFab", dts, every: int = 5):
        """(J, dJ/dS0): the objective and its gradient with respect to the
        valid cells of S0 (a MultiFab like S0; ghosts, UEINT and UTEMP 0)."""
        dts = [float(v) for v in dts]
        N = len(dts)
        final, ckpt = self.run(S0, dts, every)
        J = self.objective(final)
        g = self.ng
        L = _zeros_like(S0)
        for t in L.fabs:
            t[abi.UTEMP, g:-g, g:-g, g:-g] = self.vol
        La, Lb, Tmp = _zeros_like(S0), _zeros_like(S0), _zeros_like(S0)
        Rb = _zeros_like(S0, 0)
        del final
        for start in sorted(ckpt, reverse=True):
            stop = min(start + every, N)
            S_old, S_new = _clone(ckpt[start]), _clone(ckpt[start])
            stages = []
            for n in range(start, stop):
                stages.append(self.step(S_old, S_new, dts[n], keep=True))
                S_old, S_new = S_new, S_old
            for n in range(stop - 1, start - 1, -1):
                A, B, C = stages[n - start]
                self._adjoint_step(A, B, C, dts[n], L, La, Lb, Tmp, Rb)
                L, La = La, L
            del stages
        return J, L
