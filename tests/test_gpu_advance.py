"""GPU tests of the level operations around the RHS — ghost fill, LinComb,
computeTemp, the time-step estimate — and of SSP-RK2 trajectories built from
them (PeleC::do_mol_advance, Source/Advance.cpp:45-196), against the oracle.
"""
import numpy as np
import pytest

from conftest import rel_maxnorm
from pelec_gb300 import abi, advance, problems

pytestmark = pytest.mark.gpu


def _mf(mol, boxes, ngrow):
    import torch

    fabs = [torch.from_numpy(np.ascontiguousarray(st.S)).cuda() for st in boxes]
    return mol.MultiFab([(st.lo, st.hi) for st in boxes], boxes[0].S.shape[0], ngrow, fabs=fabs)


def _split(st, nsplit):
    """Split a BoxState's valid box into nsplit^3 boxes, each with 4 ghosts
    (ghost contents garbage so the fill must produce them)."""
    from pelec_gb300.problems import BoxState

    n = st.shape
    out = []
    edges = [np.linspace(0, n[d], nsplit + 1).astype(int) for d in range(3)]
    rng = np.random.default_rng(0)
    for kz in range(nsplit):
        for jy in range(nsplit):
            for ix in range(nsplit):
                lo = (edges[0][ix], edges[1][jy], edges[2][kz])
                hi = (edges[0][ix + 1] - 1, edges[1][jy + 1] - 1, edges[2][kz + 1] - 1)
                S = rng.normal(size=(st.S.shape[0], hi[2] - lo[2] + 9, hi[1] - lo[1] + 9, hi[0] - lo[0] + 9))
                S[:, 4:-4, 4:-4, 4:-4] = st.S[:, 4 + lo[2]:5 + hi[2], 4 + lo[1]:5 + hi[1], 4 + lo[0]:5 + hi[0]]
                out.append(BoxState(lo=lo, hi=hi, S=np.ascontiguousarray(S), dx=st.dx))
    return out


BCS = {
    "periodic": ((0, 0, 0), (0, 0, 0)),
    "outflow_z": ((0, 0, abi.PC_BC_OUTFLOW), (0, 0, abi.PC_BC_OUTFLOW)),
    "walls": ((abi.PC_BC_SYMMETRY, 0, abi.PC_BC_NOSLIPWALL), (abi.PC_BC_SLIPWALL, 0, abi.PC_BC_OUTFLOW)),
}


@pytest.mark.parametrize("bc", sorted(BCS))
def test_fill_ghosts_multibox_matches_oracle(cuda_lib, oracle_lib, bc):
    mol = cuda_lib
    mech, st, _ = problems.flame((16, 12, 20), seed=51)
    lo_bc, hi_bc = BCS[bc]
    geom = abi.geometry((0, 0, 0), (15, 11, 19), lo_bc, hi_bc)
    boxes = _split(st, 2)
    ref = [problems.BoxState(b.lo, b.hi, b.S.copy(), b.dx) for b in boxes]
    oracle_lib.fill_ghosts(ref, geom, 4)
    op = mol.MOLOperator(problems.make_config(mech))
    S = _mf(mol, boxes, 4)
    op.fill_ghosts(S, geom)
    for t, r in zip(S.fabs, ref):
        np.testing.assert_array_equal(t.cpu().numpy(), r.S)


def test_fill_ghosts_single_box_periodic_equals_generator(cuda_lib):
    """A periodic flame box: the fill reproduces the generator's own periodic
    x/y ghosts exactly."""
    mol = cuda_lib
    mech, st, _ = problems.flame((12, 10, 8), seed=52)
    problems.fill_ghosts(st.S, 4, ("periodic",) * 3)
    want = st.S.copy()
    S = _mf(mol, [st], 4)
    for t in S.fabs:  # poison the ghosts
        t[:, :4] = np.nan
    op = mol.MOLOperator(problems.make_config(mech))
    op.fill_ghosts(S, abi.geometry((0, 0, 0), (11, 9, 7), (0, 0, 0), (0, 0, 0)))
    np.testing.assert_array_equal(S.fabs[0].cpu().numpy(), want)


def test_compute_temp_and_lincomb_bitwise(cuda_lib, oracle_lib):
    import torch

    mol = cuda_lib
    mech, st, _ = problems.flame((16, 16, 16), seed=53)
    cfg = problems.make_config(mech)
    R, = oracle_lib.mol_rhs(cfg, [st])
    dt = 2e-9
    # oracle: S* = S + dt R, then computeTemp
    ref = problems.BoxState(st.lo, st.hi, st.S.copy(), st.dx)
    ref.valid(ref.S)[...] = 1.0 * st.valid(st.S) + dt * R
    oracle_lib.compute_temp(cfg, [ref])
    op = mol.MOLOperator(cfg)
    S = _mf(mol, [st], 4)
    Snew = _mf(mol, [st], 4)
    Rm = mol.MultiFab([(st.lo, st.hi)], 16, 0, fabs=[torch.from_numpy(R).cuda()])
    op.lincomb(Snew, 1.0, S, dt, Rm)
    op.compute_temp(Snew)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(st.valid(Snew.fabs[0].cpu().numpy()), ref.valid(ref.S))
    assert op.status().newton_nonconverged == 0


@pytest.mark.parametrize("phys", ["tgv", "flame"])
def test_est_dt_matches_oracle(cuda_lib, oracle_lib, phys):
    mol = cuda_lib
    if phys == "tgv":
        mech, st = problems.tgv(16, seed=54)
    else:
        mech, st, _ = problems.flame((16, 16, 16), seed=54)
    cfg = problems.make_config(mech)
    want, _ = oracle_lib.est_dt(cfg, [st], 0.3)
    op = mol.MOLOperator(cfg)
    got = op.est_dt(_mf(mol, [st], 4), st.dx, 0.3)
    assert abs(got - want) <= 1e-14 * want, (got, want)


def test_ssprk2_trajectory_matches_oracle(cuda_lib, oracle_lib):
    """Five MOL steps on a periodic 16^3 flame: GPU states equal the oracle's
    to the transport-ulp level and conserve every periodic total."""
    import torch

    mol = cuda_lib
    mech, st, _ = problems.flame((16, 16, 16), seed=55)
    cfg = problems.make_config(mech)
    geom = abi.geometry((0, 0, 0), (15, 15, 15), (0, 0, 0), (0, 0, 0))
    oracle_lib.fill_ghosts([st], geom, 4)
    dt, _ = oracle_lib.est_dt(cfg, [st], 0.3)
    op = mol.MOLOperator(cfg)
    S_old = _mf(mol, [st], 4)
    S_new = _mf(mol, [st], 4)
    R = mol.MultiFab([(st.lo, st.hi)], 16, 0)
    ref = [st]
    for _ in range(5):
        ref = oracle_lib.ssprk2_step(cfg, ref, geom, dt)
        advance.ssprk2_step(op, S_old, S_new, R, geom, st.dx, dt)
        S_old, S_new = S_new, S_old
    torch.cuda.synchronize()
    gpu = st.valid(S_old.fabs[0].cpu().numpy())
    want = st.valid(ref[0].S)
    err = rel_maxnorm(gpu, want)
    print("5-step trajectory rel max-norm per component:", err)
    assert err.max() <= 1e-11, err
    tot0 = st.valid(st.S).sum(axis=(1, 2, 3))
    tot1 = gpu.sum(axis=(1, 2, 3))
    scale = np.abs(st.valid(st.S)).sum(axis=(1, 2, 3))
    for n in [abi.URHO, abi.UMX, abi.UMY, abi.UMZ, abi.UEDEN] + [abi.UFS + k for k in range(9)]:
        assert abs(tot1[n] - tot0[n]) <= 1e-13 * scale[n], n


def test_c4_mixed_256_ten_steps_conservation(cuda_lib):
    """C4: 256^3 flame, mixed precision, 10 SSP-RK2 steps at CFL 0.3 (z made
    periodic so that every total is closed): domain totals of mass, momentum,
    energy and species stay constant to FP64 round-off."""
    import torch

    mol = cuda_lib
    mech, st, _ = problems.flame((256, 256, 256), seed=56)
    cfgm = problems.make_config(mech, precision=abi.PC_PRECISION_MIXED)
    geom = abi.geometry((0, 0, 0), (255, 255, 255), (0, 0, 0), (0, 0, 0))
    op = mol.MOLOperator(cfgm)
    S_old = _mf(mol, [st], 4)
    del st.S
    S_new = mol.MultiFab(S_old.boxes, 16, 4)
    R = mol.MultiFab(S_old.boxes, 16, 0)
    op.fill_ghosts(S_old, geom)
    dt = op.est_dt(S_old, (1e-3,) * 3, 0.3)
    v = lambda t: t[:, 4:-4, 4:-4, 4:-4]
    tot0 = v(S_old.fabs[0]).sum(dim=(1, 2, 3)).cpu().numpy()
    scale = v(S_old.fabs[0]).abs().sum(dim=(1, 2, 3)).cpu().numpy()
    for _ in range(10):
        advance.ssprk2_step(op, S_old, S_new, R, geom, (1e-3,) * 3, dt)
        S_old, S_new = S_new, S_old
    torch.cuda.synchronize()
    final = v(S_old.fabs[0])
    assert bool(torch.isfinite(final).all())
    tot1 = final.sum(dim=(1, 2, 3)).cpu().numpy()
    drift = np.abs(tot1 - tot0) / scale
    print("C4 10-step relative drift of totals:", drift)
    for n in [abi.URHO, abi.UMX, abi.UMY, abi.UMZ, abi.UEDEN] + [abi.UFS + k for k in range(9)]:
        assert drift[n] <= 1e-13, (n, drift[n])


@pytest.mark.parametrize("case", ["flame_periodic_outflow", "split_walls"])
def test_step_graph_equals_host_driven_steps(cuda_lib, case):
    """Five SSP-RK2 steps as CUDA-graph replays (pc_mol_step_graph, both
    directions A -> B -> A ...) equal five host-driven advance.ssprk2_step
    calls bit for bit, on one box and on a split level with walls."""
    import torch

    mol = cuda_lib
    if case == "split_walls":
        mech, st, _ = problems.flame((16, 12, 20), seed=57)
        lo_bc, hi_bc = BCS["walls"]
        geom = abi.geometry((0, 0, 0), (15, 11, 19), lo_bc, hi_bc)
        boxes = _split(st, 2)
    else:
        mech, st, _ = problems.flame((24, 16, 20), seed=58)
        geom = abi.geometry(st.lo, st.hi, (0, 0, abi.PC_BC_OUTFLOW), (0, 0, abi.PC_BC_OUTFLOW))
        boxes = [st]
    cfg = problems.make_config(mech)
    op = mol.MOLOperator(cfg)
    S_old, S_new = _mf(mol, boxes, 4), _mf(mol, boxes, 4)
    R = mol.MultiFab(S_old.boxes, S_old.ncomp, 0)
    A, B = _mf(mol, boxes, 4), mol.MultiFab(S_old.boxes, S_old.ncomp, 4)
    R2 = mol.MultiFab(S_old.boxes, S_old.ncomp, 0)
    stepper = advance.Stepper(op, A, B, R2, geom, st.dx)
    op.fill_ghosts(S_old, geom)
    dt = op.est_dt(S_old, st.dx, 0.3)
    for n in range(5):
        advance.ssprk2_step(op, S_old, S_new, R, geom, st.dx, dt * (1.0 + 0.01 * n))
        S_old, S_new = S_new, S_old
        stepper.step(dt * (1.0 + 0.01 * n))
    torch.cuda.synchronize()
    g = 4
    for b in range(len(boxes)):
        want = S_old.fabs[b][:, g:-g, g:-g, g:-g].cpu().numpy()
        got = stepper.state.fabs[b][:, g:-g, g:-g, g:-g].cpu().numpy()
        np.testing.assert_array_equal(got, want, err_msg=f"box {b}")
    st_ = stepper.graph.status()
    assert st_.newton_nonconverged == 0 and st_.nonfinite_output == 0
    stepper.close()
