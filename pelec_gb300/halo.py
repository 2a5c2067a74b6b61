"""Ghost exchange of a level whose boxes are distributed over ranks.

The reference fills the ghost cells of every box before each RHS evaluation
(FillPatcherFill / FillBoundary with the physical BC fill, Source/Advance.cpp:98,
:132; BC types Source/Setup.cpp:34-56); across ranks that is AMReX's
FillBoundary communication.  On one GPU the whole level is filled by one
device kernel (pc_mol_fill_ghosts); with the boxes sharded over ranks
(distribute.distribution_map), each rank holds only its own boxes, and the
ghost cells whose source cell lies in another rank's box arrive by message.

The rule is the device fill's: every ghost cell of grow(valid, ngrow) takes
the value of the one valid cell of the level its index maps to — periodic
directions wrap by the domain length, PC_BC_OUTFLOW clamps to the nearest
interior plane, reflecting faces mirror (normal momentum negated on symmetry
and slip walls, all momenta on no-slip walls).  ``copy_plan`` turns that
rule into box-to-box block copies: grow(valid, ngrow) of a destination box
splits per direction into the part below the domain, inside it and above it;
each of the (up to 27) products maps to a source index vector per direction
(identity, shift, a constant plane, or a reversed range), and its
intersection with each valid box of the level is one plan entry.  Every
rank computes the same plan from the BoxArray, so no sizes are exchanged:
``exchange`` copies entries whose source and destination are both local,
and for each peer packs the blocks it owes in plan order into one buffer,
one send and one receive per peer pair (torch.distributed: gloo on CPU
tensors, NCCL on CUDA tensors), then unpacks in the same order.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import abi

MOMENTUM = (abi.UMX, abi.UMY, abi.UMZ)


@dataclass
class PlanEntry:
    src: int                 # source box index
    dst: int                 # destination box index
    dst_lo: tuple            # first destination cell (i, j, k)
    dst_hi: tuple            # last destination cell
    src_idx: tuple           # per direction, the source index of each destination index (numpy int arrays)
    sign: tuple              # sign of (UMX, UMY, UMZ) in the copy

    @property
    def shape(self) -> tuple:
        return tuple(h - l + 1 for l, h in zip(self.dst_lo, self.dst_hi))


def _segments(blo: int, bhi: int, ng: int, d: int, geom) -> list:
    """Parts of [blo - ng, bhi + ng] in direction d: (first, last, source
    index vector, momentum signs) below, inside and above the domain."""
    lo, hi = geom.domain_lo[d], geom.domain_hi[d]
    L = hi - lo + 1
    periodic = geom.bc_lo[d] == abi.PC_BC_INTERIOR and geom.bc_hi[d] == abi.PC_BC_INTERIOR
    out = []
    g0, g1 = blo - ng, bhi + ng
    parts = [(g0, min(g1, lo - 1), True), (max(g0, lo), min(g1, hi), None), (max(g0, hi + 1), g1, False)]
    for a, b, below in parts:
        if a > b:
            continue
        x = np.arange(a, b + 1)
        sign = [1.0, 1.0, 1.0]
        if below is None:
            src = x
        else:
            bc = geom.bc_lo[d] if below else geom.bc_hi[d]
            if periodic:
                src = x + L if below else x - L
            elif bc == abi.PC_BC_OUTFLOW:
                src = np.full_like(x, lo if below else hi)
            else:  # symmetry, slip and no-slip walls: mirror
                src = 2 * lo - 1 - x if below else 2 * hi + 1 - x
                if bc == abi.PC_BC_NOSLIPWALL:
                    sign = [-1.0, -1.0, -1.0]
                else:
                    sign[d] = -1.0
        out.append((a, b, src, sign, below is None))
    return out


def copy_plan(boxes, geom, ngrow: int) -> list:
    """The block copies that fill grow(valid, ngrow) of every box (list of
    (lo, hi)) outside its own valid region; deterministic, the same on
    every rank."""
    plan = []
    for db, (blo, bhi) in enumerate(boxes):
        segs = [_segments(blo[d], bhi[d], ngrow, d, geom) for d in range(3)]
        for sx in segs[0]:
            for sy in segs[1]:
                for sz in segs[2]:
                    per = (sx, sy, sz)
                    interior = all(p[4] for p in per)
                    sign = tuple(per[0][3][c] * per[1][3][c] * per[2][3][c] for c in range(3))
                    for sb, (alo, ahi) in enumerate(boxes):
                        if interior and sb == db:
                            continue  # the box's own valid cells
                        sel = []
                        for d in range(3):
                            src = per[d][2]
                            m = np.nonzero((src >= alo[d]) & (src <= ahi[d]))[0]
                            if m.size == 0:
                                break
                            # the source vector is monotone, so the match is one run
                            sel.append((int(m[0]), int(m[-1])))
                        if len(sel) < 3:
                            continue
                        dlo = tuple(per[d][0] + sel[d][0] for d in range(3))
                        dhi = tuple(per[d][0] + sel[d][1] for d in range(3))
                        sidx = tuple(per[d][2][sel[d][0]:sel[d][1] + 1] for d in range(3))
                        plan.append(PlanEntry(sb, db, dlo, dhi, sidx, sign))
    return plan


def _gather(fab, begin, e: PlanEntry):
    """The entry's source block from a FAB (ncomp, nz, ny, nx) whose smallEnd
    is ``begin``, momenta signed, as a (ncomp, nz, ny, nx) tensor."""
    import torch

    dev = fab.device
    ii = torch.as_tensor(e.src_idx[0] - begin[0], dtype=torch.long, device=dev)
    jj = torch.as_tensor(e.src_idx[1] - begin[1], dtype=torch.long, device=dev)
    kk = torch.as_tensor(e.src_idx[2] - begin[2], dtype=torch.long, device=dev)
    blk = fab.index_select(1, kk).index_select(2, jj).index_select(3, ii)
    if e.sign != (1.0, 1.0, 1.0):
        blk = blk.clone()
        for c, s in zip(MOMENTUM, e.sign):
            if s != 1.0:
                blk[c].neg_()
    return blk


def _scatter(fab, begin, e: PlanEntry, blk) -> None:
    k0, j0, i0 = (e.dst_lo[d] - begin[d] for d in (2, 1, 0))
    nz, ny, nx = e.shape[2], e.shape[1], e.shape[0]
    fab[:, k0:k0 + nz, j0:j0 + ny, i0:i0 + nx] = blk


def exchange(fabs: dict, boxes, owner, rank: int, geom, ngrow: int, plan=None, group=None) -> None:
    """Fill the ghost cells of this rank's boxes in place.

    fabs: {box index: tensor (ncomp, nz, ny, nx) over grow(valid, ngrow)} for
    the boxes this rank owns (owner[b] == rank); boxes: (lo, hi) of every box
    of the level; plan: copy_plan(boxes, geom, ngrow), computed here if None.
    Collective over ``group`` when it has more than one rank."""
    import torch

    plan = copy_plan(boxes, geom, ngrow) if plan is None else plan
    begin = {b: tuple(boxes[b][0][d] - ngrow for d in range(3)) for b in fabs}
    ncomp = next(iter(fabs.values())).shape[0] if fabs else 0
    sends, recvs = {}, {}
    for e in plan:
        if owner[e.dst] == rank and owner[e.src] == rank:
            _scatter(fabs[e.dst], begin[e.dst], e, _gather(fabs[e.src], begin[e.src], e))
        elif owner[e.src] == rank:
            sends.setdefault(owner[e.dst], []).append(_gather(fabs[e.src], begin[e.src], e).reshape(-1))
        elif owner[e.dst] == rank:
            recvs.setdefault(owner[e.src], []).append(e)
    if not sends and not recvs:
        return
    import torch.distributed as dist

    dev = next(iter(fabs.values())).device
    reqs, bufs = [], {}
    for peer in sorted(recvs):
        n = sum(ncomp * int(np.prod(e.shape)) for e in recvs[peer])
        bufs[peer] = torch.empty(n, dtype=torch.float64, device=dev)
        reqs.append(dist.irecv(bufs[peer], src=peer, group=group))
    out = {peer: torch.cat(parts) for peer, parts in sends.items()}
    for peer in sorted(out):
        reqs.append(dist.isend(out[peer], dst=peer, group=group))
    for r in reqs:
        r.wait()
    for peer in sorted(recvs):
        off = 0
        for e in recvs[peer]:
            nx, ny, nz = e.shape
            n = ncomp * nx * ny * nz
            _scatter(fabs[e.dst], begin[e.dst], e, bufs[peer][off:off + n].reshape(ncomp, nz, ny, nx))
            off += n
