"""GPU tests of the batched-level machinery: every flux-pass launch
configuration (tile shape, one CTA per tile or a persistent grid) gives the
same RHS bit for bit (and the oracle's to 1e-12), the autotuner caches its
choice per box-size histogram, and a captured CUDA graph of ghost fill + RHS
replays to the direct calls' result.
"""
import numpy as np
import pytest

from conftest import rel_maxnorm
from gpu_util import to_multifab
from pelec_gb300 import abi, mechanism, problems

pytestmark = pytest.mark.gpu


def _rhs_at_tile(mol, op, boxes, tile):
    import torch

    op.set_tile(tile)
    S = to_multifab(mol, boxes, boxes[0].ng)
    R = mol.MultiFab([(st.lo, st.hi) for st in boxes], boxes[0].S.shape[0], 0)
    for t in R.fabs:
        t.fill_(np.nan)
    op.rhs_level(S, R, boxes[0].dx)
    torch.cuda.synchronize()
    assert op.current_tile() == tile
    return [t.cpu().numpy() for t in R.fabs]


def _ragged_level():
    """Uneven boxes plus boxes smaller than every tile and with odd extents."""
    mech, boxes = problems.level_boxes(nboxes=6, seed=31, edges=(8, 12, 16, 24))
    _, big = problems.level_boxes(nboxes=3, seed=32, edges=(24,))
    for st, shp in zip(big, [(1, 1, 1), (3, 5, 2), (17, 9, 5)]):
        nx, ny, nz = shp
        S = np.ascontiguousarray(st.S[:, : nz + 8, : ny + 8, : nx + 8])
        lo = (st.lo[0] + 10000, 0, 0)  # disjoint from the first boxes
        boxes.append(problems.BoxState(lo=lo, hi=tuple(l + n - 1 for l, n in zip(lo, shp)), S=S, dx=st.dx))
    return mech, boxes


@pytest.mark.parametrize("precision", [abi.PC_PRECISION_FP64, abi.PC_PRECISION_MIXED, abi.PC_PRECISION_MIXED_FP64])
def test_every_tile_shape_gives_identical_rhs(cuda_lib, oracle_lib, precision):
    mol = cuda_lib
    mech, boxes = _ragged_level()
    cfg = problems.make_config(mech, precision=precision)
    op = mol.MOLOperator(cfg)
    outs = [_rhs_at_tile(mol, op, boxes, t) for t in range(abi.PC_NUM_LAUNCH_CONFIGS)]
    for t in range(1, abi.PC_NUM_LAUNCH_CONFIGS):
        for b, (g0, gt) in enumerate(zip(outs[0], outs[t])):
            np.testing.assert_array_equal(gt, g0, err_msg=f"tile {t} box {b}")
    if precision == abi.PC_PRECISION_FP64:
        refs = oracle_lib.mol_rhs(cfg, boxes)
        for g, r in zip(outs[2], refs):
            assert rel_maxnorm(g, r).max() <= 1e-12


def test_every_tile_shape_single_species(cuda_lib, oracle_lib):
    mol = cuda_lib
    mech, st = problems.tgv(20, seed=33)
    cfg = problems.make_config(mech)
    op = mol.MOLOperator(cfg)
    outs = [_rhs_at_tile(mol, op, [st], t)[0] for t in range(abi.PC_NUM_LAUNCH_CONFIGS)]
    for t in range(1, abi.PC_NUM_LAUNCH_CONFIGS):
        np.testing.assert_array_equal(outs[t], outs[0])
    ref, = oracle_lib.mol_rhs(cfg, [st])
    assert rel_maxnorm(outs[3], ref).max() <= 1e-12


@pytest.mark.parametrize("precision", [abi.PC_PRECISION_FP64, abi.PC_PRECISION_MIXED, abi.PC_PRECISION_MIXED_FP64])
def test_persistent_grid_strides_over_every_tile(cuda_lib, precision):
    """A 64^3 flame has more tiles than the GPU holds CTAs at any shape, so
    each CTA of a persistent launch takes a run of several tiles (handing the
    z face and slope layers up each column): same RHS bit for bit as one CTA
    per tile, and every cell counted once."""
    mol = cuda_lib
    mech, st, _ = problems.flame((64, 64, 64), w_noise=1.0)
    cfg = problems.make_config(mech, precision=precision)
    op = mol.MOLOperator(cfg)
    for shape in range(abi.PC_NUM_TILES):
        one, = _rhs_at_tile(mol, op, [st], shape)
        pers, = _rhs_at_tile(mol, op, [st], shape + abi.PC_LAUNCH_PERSISTENT)
        np.testing.assert_array_equal(pers, one, err_msg=f"shape {shape}")
        assert np.isfinite(pers).all()
        assert op.status().cells == 64 ** 3
    if precision == abi.PC_PRECISION_FP64:
        # the exported face fluxes too: a persistent CTA hands the z face layer
        # between consecutive tiles of a column instead of evaluating it again
        import torch

        out = []
        for t in (0, abi.PC_LAUNCH_PERSISTENT):
            op.set_tile(t)
            S = to_multifab(mol, [st], st.ng)
            R = mol.MultiFab([(st.lo, st.hi)], st.S.shape[0], 0)
            F = op.rhs_level_fluxes(S, R, st.dx)[0]
            torch.cuda.synchronize()
            out.append([f.cpu().numpy() for f in F] + [R.fabs[0].cpu().numpy()])
        for a, b in zip(*out):
            np.testing.assert_array_equal(a, b)


def test_autotune_caches_choice_per_histogram(cuda_lib):
    import torch

    mol = cuda_lib
    mech, boxes = _ragged_level()
    cfg = problems.make_config(mech)
    op = mol.MOLOperator(cfg)
    S = to_multifab(mol, boxes, boxes[0].ng)
    R = mol.MultiFab(S.boxes, S.ncomp, 0)
    best, ms = op.autotune(S, R, boxes[0].dx, reps=2)
    assert 0 <= best < abi.PC_NUM_LAUNCH_CONFIGS and len(ms) == abi.PC_NUM_LAUNCH_CONFIGS
    assert all(m > 0 for m in ms) and ms[best] == min(ms)
    ref = [t.clone() for t in R.fabs]
    R2 = mol.MultiFab(S.boxes, S.ncomp, 0)
    op.rhs_level(S, R2, boxes[0].dx)
    torch.cuda.synchronize()
    assert op.current_tile() == best  # looked up by the histogram
    for a, b in zip(R2.fabs, ref):
        assert torch.equal(a, b)
    # a different BoxArray falls back to the default shape
    op.rhs_level(to_multifab(mol, boxes[:2], 4), mol.MultiFab(S.boxes[:2], S.ncomp, 0), boxes[0].dx)
    torch.cuda.synchronize()
    assert op.current_tile() == 0


@pytest.mark.parametrize("precision", [abi.PC_PRECISION_FP64, abi.PC_PRECISION_MIXED])
def test_graph_replay_equals_direct_calls(cuda_lib, precision):
    """Graph of ghost fill + RHS on a 2x2x2 split periodic flame: the replay
    equals fill_ghosts + rhs_level (bit for bit, in either precision), reads
    the arrays' current contents on every replay, and is not disturbed by
    later calls through the handle."""
    import torch

    from test_gpu_advance import _split

    mol = cuda_lib
    mech, st, _ = problems.flame((24, 16, 16), seed=34)
    cfg = problems.make_config(mech, precision=precision)
    geom = abi.geometry((0, 0, 0), (23, 15, 15), (0, 0, 0), (0, 0, 0))
    boxes = _split(st, 2)
    op = mol.MOLOperator(cfg)

    def direct(S):
        Sd = mol.MultiFab(S.boxes, S.ncomp, S.ngrow, fabs=[t.clone() for t in S.fabs])
        R = mol.MultiFab(S.boxes, S.ncomp, 0)
        op.fill_ghosts(Sd, geom)
        op.rhs_level(Sd, R, st.dx)
        torch.cuda.synchronize()
        return R

    S = to_multifab(mol, boxes, 4)
    Rg = mol.MultiFab(S.boxes, S.ncomp, 0)
    g = op.graph(S, Rg, st.dx, geom)
    want = direct(S)
    for t in Rg.fabs:
        t.fill_(np.nan)
    g.launch()
    torch.cuda.synchronize()
    for a, b in zip(Rg.fabs, want.fabs):
        assert torch.equal(a, b)
    assert g.status().cells == 24 * 16 * 16
    # change the state in place, use the handle on another BoxArray, replay
    for t in S.fabs:
        t[abi.URHO] *= 1.001
        t[abi.UEDEN] *= 1.001
    other = to_multifab(mol, boxes[:1], 4)
    op.rhs_level(other, mol.MultiFab(other.boxes, other.ncomp, 0), st.dx)
    want2 = direct(S)
    g.launch()
    torch.cuda.synchronize()
    for a, b in zip(Rg.fabs, want2.fabs):
        assert torch.equal(a, b)
    g.close()


def test_c3_full_level_against_oracle(cuda_lib, oracle_lib):
    """C3: the full 400-box level (edges per axis from {8,16,24,32,48,64},
    seeded; 9-species flame at per-box offsets) in one batched launch: FP64
    bit for bit equal to the oracle on every box, and the mixed form within
    1e-5 relative L2 of it per component over the whole level."""
    import torch

    mol = cuda_lib
    mech, boxes = problems.level_boxes(400, seed=3)
    ref = oracle_lib.mol_rhs(problems.make_config(mech), boxes)
    S = to_multifab(mol, boxes, boxes[0].ng)
    R = mol.MultiFab([(st.lo, st.hi) for st in boxes], boxes[0].S.shape[0], 0)
    op = mol.MOLOperator(problems.make_config(mech))
    op.rhs_level(S, R, boxes[0].dx)
    torch.cuda.synchronize()
    for b, (t, r) in enumerate(zip(R.fabs, ref)):
        np.testing.assert_array_equal(t.cpu().numpy(), r, err_msg=f"box {b}")
    assert op.status().cells == sum(st.ncells for st in boxes)
    opm = mol.MOLOperator(problems.make_config(mech, precision=abi.PC_PRECISION_MIXED))
    opm.rhs_level(S, R, boxes[0].dx)
    torch.cuda.synchronize()
    num = np.zeros(S.ncomp)
    den = np.zeros(S.ncomp)
    for t, r in zip(R.fabs, ref):
        a = t.cpu().numpy()
        num += ((a - r) ** 2).sum(axis=(1, 2, 3))
        den += (r ** 2).sum(axis=(1, 2, 3))
    l2 = np.sqrt(num / np.maximum(den, 1e-300))
    print("C3 mixed rel L2 per component:", l2)
    l2[abi.UTEMP] = 0.0  # identically zero in both
    assert l2.max() <= 1e-5, l2


def test_21_species_level_every_tile_and_autotune(cuda_lib, oracle_lib):
    """A 21-species level: every launch configuration gives the same RHS bit
    for bit, equal to the oracle; the autotuner times and caches a choice for
    this species count on the handle."""
    mol = cuda_lib
    mech, boxes = problems.level_boxes(nboxes=4, seed=33, edges=(8, 12, 16), mech=mechanism.drm_synthetic())
    cfg = problems.make_config(mech)
    refs = oracle_lib.mol_rhs(cfg, boxes)
    op = mol.MOLOperator(cfg)
    # the FP64 flux pass of the 8x8x8 and 16x8x4 tiles needs 278 and 343 KB
    # of shared memory per CTA at 21 species, more than a CTA may have
    too_big = {1, 2, 1 + abi.PC_NUM_LAUNCH_CONFIGS // 2, 2 + abi.PC_NUM_LAUNCH_CONFIGS // 2}
    for t in range(abi.PC_NUM_LAUNCH_CONFIGS):
        if t in too_big:
            with pytest.raises(mol.MOLError) as err:
                op.set_tile(t)
            assert err.value.code == abi.PC_ERR_UNSUPPORTED
            continue
        out = _rhs_at_tile(mol, op, boxes, t)
        for a, r in zip(out, refs):
            np.testing.assert_array_equal(a, r, err_msg=f"configuration {t}")
    op.set_tile(-1)
    S = to_multifab(mol, boxes, boxes[0].ng)
    R = mol.MultiFab([(st.lo, st.hi) for st in boxes], boxes[0].S.shape[0], 0)
    best, ms = op.autotune(S, R, boxes[0].dx, reps=2)
    assert 0 <= best < abi.PC_NUM_LAUNCH_CONFIGS and best not in too_big
    assert all((m == -1.0) if t in too_big else (m > 0) for t, m in enumerate(ms)), ms
    op.rhs_level(S, R, boxes[0].dx)
    assert op.current_tile() == best
