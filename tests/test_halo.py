"""CPU tests of the inter-rank ghost exchange (pelec_gb300/halo.py): the copy
plan applied on one rank, and the exchange between two gloo ranks, fill
every ghost cell of grow(valid, 4) exactly as the oracle's single-level fill
of the whole BoxArray (periodic wrap, outflow clamp, mirrored walls with
their momentum signs)."""
import os
import pickle
import socket

import numpy as np
import pytest

from pelec_gb300 import abi, distribute, halo, mechanism, problems

NG = 4
NVAR = 16


def _tiling(seed: int):
    """Boxes that tile a 24 x 16 x 12 domain with uneven cuts, and random
    states on their valid cells (ghosts NaN)."""
    rng = np.random.default_rng(seed)
    cuts = [[0, 7, 15, 24], [0, 5, 16], [0, 6, 9, 12]]
    boxes = []
    for k in range(len(cuts[2]) - 1):
        for j in range(len(cuts[1]) - 1):
            for i in range(len(cuts[0]) - 1):
                lo = (cuts[0][i], cuts[1][j], cuts[2][k])
                hi = (cuts[0][i + 1] - 1, cuts[1][j + 1] - 1, cuts[2][k + 1] - 1)
                boxes.append((lo, hi))
    states = []
    for lo, hi in boxes:
        n = [h - l + 1 + 2 * NG for l, h in zip(lo, hi)]
        S = np.full((NVAR, n[2], n[1], n[0]), np.nan)
        S[:, NG:-NG, NG:-NG, NG:-NG] = rng.normal(size=(NVAR, n[2] - 2 * NG, n[1] - 2 * NG, n[0] - 2 * NG))
        states.append(problems.BoxState(lo, hi, S, (1.0, 1.0, 1.0), NG))
    return boxes, states


GEOMS = {
    "periodic": ((0, 0, 0), (0, 0, 0)),
    "outflow_z": ((0, 0, abi.PC_BC_OUTFLOW), (0, 0, abi.PC_BC_OUTFLOW)),
    "walls": ((abi.PC_BC_SYMMETRY, 0, abi.PC_BC_NOSLIPWALL), (abi.PC_BC_SLIPWALL, 0, abi.PC_BC_OUTFLOW)),
}


def _geom(name):
    lo, hi = GEOMS[name]
    return abi.geometry((0, 0, 0), (23, 15, 11), lo, hi)


def _reference(oracle_lib, name, seed):
    boxes, states = _tiling(seed)
    oracle_lib.fill_ghosts(states, _geom(name), NG)
    return boxes, states


@pytest.mark.parametrize("name", list(GEOMS))
def test_copy_plan_on_one_rank_matches_the_level_fill(oracle_lib, name):
    import torch

    boxes, want = _reference(oracle_lib, name, seed=3)
    _, states = _tiling(seed=3)
    fabs = {b: torch.from_numpy(st.S.copy()) for b, st in enumerate(states)}
    halo.exchange(fabs, boxes, [0] * len(boxes), 0, _geom(name), NG)
    for b, st in enumerate(want):
        got = fabs[b].numpy()
        assert not np.isnan(got).any(), b
        np.testing.assert_array_equal(got, st.S, err_msg=f"box {b}")


def test_copy_plan_covers_each_ghost_cell_once():
    boxes, _ = _tiling(seed=0)
    plan = halo.copy_plan(boxes, _geom("walls"), NG)
    for b, (lo, hi) in enumerate(boxes):
        n = [h - l + 1 + 2 * NG for l, h in zip(lo, hi)]
        hits = np.zeros((n[2], n[1], n[0]), int)
        for e in plan:
            if e.dst != b:
                continue
            s = [e.dst_lo[d] - (lo[d] - NG) for d in range(3)]
            hits[s[2]:s[2] + e.shape[2], s[1]:s[1] + e.shape[1], s[0]:s[0] + e.shape[0]] += 1
        assert (hits[NG:-NG, NG:-NG, NG:-NG] == 0).all()
        hits[NG:-NG, NG:-NG, NG:-NG] = 1
        assert (hits == 1).all(), b


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, outdir, name):
    import torch
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    boxes, states = _tiling(seed=5)
    owner = distribute.distribution_map(boxes, world)
    fabs = {b: torch.from_numpy(states[b].S.copy()) for b in range(len(boxes)) if owner[b] == rank}
    halo.exchange(fabs, boxes, owner, rank, _geom(name), NG)
    with open(os.path.join(outdir, f"rank{rank}.pkl"), "wb") as f:
        pickle.dump({b: t.numpy() for b, t in fabs.items()}, f)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("name", ["periodic", "walls"])
def test_two_rank_exchange_matches_the_level_fill(oracle_lib, tmp_path, name):
    import torch.multiprocessing as mp

    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path), name), nprocs=world, join=True)
    boxes, want = _reference(oracle_lib, name, seed=5)
    owner = distribute.distribution_map(boxes, world)
    assert set(owner) == {0, 1}
    seen = {}
    for r in range(world):
        got = pickle.load(open(tmp_path / f"rank{r}.pkl", "rb"))
        for b, a in got.items():
            assert owner[b] == r and b not in seen
            seen[b] = a
    assert sorted(seen) == list(range(len(boxes)))
    for b, a in seen.items():
        np.testing.assert_array_equal(a, want[b].S, err_msg=f"box {b}")


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(GEOMS))
def test_copy_plan_on_device_tensors_matches_the_device_fill(cuda_lib, name):
    """The plan's block copies on CUDA tensors (what each rank runs on its own
    GPU) give bit for bit the level fill kernel pc_mol_fill_ghosts."""
    import torch

    mol = cuda_lib
    boxes, states = _tiling(seed=7)
    mech = mechanism.h2_air_synthetic()
    op = mol.MOLOperator(problems.make_config(mech))
    S = mol.MultiFab(boxes, NVAR, NG, fabs=[torch.from_numpy(st.S.copy()).cuda() for st in states])
    op.fill_ghosts(S, _geom(name))
    fabs = {b: torch.from_numpy(st.S.copy()).cuda() for b, st in enumerate(states)}
    halo.exchange(fabs, boxes, [0] * len(boxes), 0, _geom(name), NG)
    torch.cuda.synchronize()
    for b in range(len(boxes)):
        assert torch.equal(fabs[b], S.fabs[b]), b
