"""CPU tests of the multi-rank path (world size 2, gloo): the distribution
map of a level's boxes, and a sharded RHS + time-step evaluation whose
per-box results and all-reduced time step equal a serial run."""
import hashlib
import os
import pickle
import socket

import numpy as np
import pytest

from pelec_gb300 import distribute, problems


def test_distribution_map_covers_and_balances():
    mech, boxes = problems.level_boxes(nboxes=40, seed=3, edges=(8, 16, 24, 32))
    bb = [(b.lo, b.hi) for b in boxes]
    for n in (1, 2, 3, 8):
        owner = distribute.distribution_map(bb, n)
        assert len(owner) == len(bb) and set(owner) <= set(range(n))
        assert owner == distribute.distribution_map(bb, n)  # deterministic
        shards = [distribute.local_boxes(bb, r, n) for r in range(n)]
        assert sorted(i for s in shards for i in s) == list(range(len(bb)))
        if n <= 3:
            assert distribute.load_imbalance(bb, n) < 1.1
    assert distribute.distribution_map(bb, 1) == [0] * len(bb)
    with pytest.raises(ValueError):
        distribute.distribution_map(bb, 0)


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _level():
    return problems.level_boxes(nboxes=6, seed=81, edges=(6, 8, 10))


def _digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _worker(rank, world, port, outdir):
    import torch.distributed as dist

    from oracle import pyoracle

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mech, boxes = _level()
    cfg = problems.make_config(mech)
    mine = distribute.local_boxes([(b.lo, b.hi) for b in boxes], rank, world)
    R = pyoracle.mol_rhs(cfg, [boxes[i] for i in mine], nthreads=1)
    digests = {i: _digest(r) for i, r in zip(mine, R)}
    dt_local = pyoracle.est_dt(cfg, [boxes[i] for i in mine], 0.3)[0] if mine else float("inf")
    dt = distribute.global_min(dt_local)
    gathered = [None] * world
    dist.all_gather_object(gathered, (digests, dt))
    if rank == 0:
        with open(os.path.join(outdir, "result.pkl"), "wb") as f:
            pickle.dump(gathered, f)
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_level_matches_serial(oracle_lib, tmp_path):
    import torch.multiprocessing as mp

    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    gathered = pickle.load(open(tmp_path / "result.pkl", "rb"))
    mech, boxes = _level()
    cfg = problems.make_config(mech)
    want = [_digest(r) for r in oracle_lib.mol_rhs(cfg, boxes, nthreads=1)]
    dt_serial = oracle_lib.est_dt(cfg, boxes, 0.3)[0]
    seen = {}
    for digests, dt in gathered:
        assert dt == dt_serial
        for i, d in digests.items():
            assert i not in seen  # each box on one rank
            seen[i] = d
    assert sorted(seen) == list(range(len(boxes)))
    for i, d in seen.items():
        assert d == want[i], i
