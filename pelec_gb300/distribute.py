"""Distribution of a level's boxes over ranks (one GPU per rank).

The RHS of a box depends only on its own state with filled ghosts, so a
level shards by boxes with no collective on the data path; the reference
distributes a BoxArray with AMReX's DistributionMapping (knapsack by cost
by default) and needs, per RHS, the ghost exchange before the call and one
all-reduce (min) for the time step (PeleC.cpp:939).  Here:

* ``distribution_map`` — deterministic greedy knapsack: boxes in order of
  decreasing cost (cells, unless costs are given), each to the currently
  least-loaded rank (ties to the lowest rank);
* ``local_boxes`` — this rank's box indices;
* ``global_min`` — the time-step all-reduce over a torch.distributed group
  (NCCL between GPUs, gloo on CPU).

The ghost exchange between ranks is pelec_gb300/halo.py (a copy plan from
the BoxArray, one packed message per peer pair); on one GPU the fill is a
device kernel over the whole level (pc_mol_fill_ghosts).
"""
from __future__ import annotations


def box_cells(lo, hi) -> int:
    n = 1
    for a, b in zip(lo, hi):
        n *= b - a + 1
    return n


def distribution_map(boxes, nranks: int, costs=None) -> list:
    """Rank of each box (list of (lo, hi))."""
    if nranks < 1:
        raise ValueError("nranks must be >= 1")
    costs = [box_cells(lo, hi) for lo, hi in boxes] if costs is None else list(costs)
    order = sorted(range(len(boxes)), key=lambda b: (-costs[b], b))
    load = [0] * nranks
    owner = [0] * len(boxes)
    for b in order:
        r = min(range(nranks), key=lambda q: (load[q], q))
        owner[b] = r
        load[r] += costs[b]
    return owner


def local_boxes(boxes, rank: int, nranks: int, costs=None) -> list:
    """Indices of the boxes rank ``rank`` owns."""
    owner = distribution_map(boxes, nranks, costs)
    return [b for b, r in enumerate(owner) if r == rank]


def load_imbalance(boxes, nranks: int, costs=None) -> float:
    """max rank load / mean rank load of the map."""
    costs = [box_cells(lo, hi) for lo, hi in boxes] if costs is None else list(costs)
    owner = distribution_map(boxes, nranks, costs)
    load = [0] * nranks
    for b, r in enumerate(owner):
        load[r] += costs[b]
    return max(load) / (sum(load) / nranks)


def global_min(x: float, group=None) -> float:
    """Minimum of x over the ranks of ``group`` (or x itself without an
    initialised process group)."""
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized():
        return float(x)
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MIN, group=group)
    return float(t.item())
