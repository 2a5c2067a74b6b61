"""torch.autograd wrapper of the MOL right-hand side of one box, for
testing and for composing the RHS with torch code: the forward pass is
pc_mol_rhs_level, the backward pass the hand-written adjoint
pc_mol_rhs_vjp (no torch differentiation of the kernels)."""
from __future__ import annotations

import torch

from . import mol


class _MOLRhs(torch.autograd.Function):
    @staticmethod
    def forward(ctx, S, op, lo, hi, dx, ngrow):
        boxes = [(tuple(lo), tuple(hi))]
        Sm = mol.MultiFab(boxes, S.shape[0], ngrow, fabs=[S.detach().contiguous()])
        R = mol.MultiFab(boxes, S.shape[0], 0)
        op.rhs_level(Sm, R, dx)
        ctx.save_for_backward(Sm.fabs[0])
        ctx.op, ctx.boxes, ctx.dx, ctx.ngrow = op, boxes, dx, ngrow
        return R.fabs[0]

    @staticmethod
    def backward(ctx, rbar):
        (S,) = ctx.saved_tensors
        nvar = S.shape[0]
        Sm = mol.MultiFab(ctx.boxes, nvar, ctx.ngrow, fabs=[S])
        Rb = mol.MultiFab(ctx.boxes, nvar, 0, fabs=[rbar.contiguous()])
        Ub = mol.MultiFab(ctx.boxes, nvar, ctx.ngrow)
        ctx.op.rhs_vjp(Sm, Rb, Ub, ctx.dx)
        return Ub.fabs[0], None, None, None, None, None


def mol_rhs(op: "mol.MOLOperator", S: torch.Tensor, lo, hi, dx, ngrow: int = 4) -> torch.Tensor:
    """RHS of one box: S is the float64 CUDA state (NVAR, nz+2g, ny+2g, nx+2g)
    of valid box [lo, hi] with g = ngrow >= 2 ghost layers; returns the RHS
    (NVAR, nz, ny, nx).  Differentiable: the gradient with respect to S is
    the adjoint of the RHS (zero outside grow(valid, 2))."""
    return _MOLRhs.apply(S, op, lo, hi, dx, ngrow)
