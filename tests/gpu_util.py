"""Helpers for GPU tests: run the CUDA library through its C ABI on BoxStates."""
import numpy as np


def to_multifab(mol, boxes, ngrow):
    import torch

    fabs = [torch.from_numpy(np.ascontiguousarray(st.S)).cuda() for st in boxes]
    return mol.MultiFab([(st.lo, st.hi) for st in boxes], boxes[0].S.shape[0], ngrow, fabs=fabs)


def gpu_rhs(mol, cfg, boxes, per_box=False, op=None, stream=None):
    """RHS of each BoxState on the GPU; returns (list of numpy arrays, status)."""
    import torch

    op = op or mol.MOLOperator(cfg)
    S = to_multifab(mol, boxes, boxes[0].ng)
    R = mol.MultiFab([(st.lo, st.hi) for st in boxes], boxes[0].S.shape[0], 0)
    for t in R.fabs:
        t.fill_(np.nan)  # every valid entry must be written
    op.rhs_level(S, R, boxes[0].dx, per_box=per_box, stream=stream)
    torch.cuda.synchronize()
    st = op.status()
    return [t.cpu().numpy() for t in R.fabs], st
