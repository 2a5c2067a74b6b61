"""GPU tests of the trajectory adjoint: the transposes of the ghost fill and
of computeTemp, the checkpointed SSP-RK2 adjoint against finite differences
of the GPU and oracle trajectories (J = sum of T dV at the last step), the
inflow-parameter gradient, and the torch.autograd wrapper."""
import dataclasses

import numpy as np
import pytest

from gpu_util import to_multifab
from pelec_gb300 import abi, problems

pytestmark = pytest.mark.gpu

GRAD_REL = 1e-6


def _flame(shape=(16, 16, 16), seed=71, params=None):
    # w noise keeps the limiter away from its kink at mc(0, 0); see problems.flame
    return problems.flame(shape, seed=seed, w_noise=1.0, params=params)


def _geom(st):
    return abi.geometry(st.lo, st.hi, (0, 0, abi.PC_BC_OUTFLOW), (0, 0, abi.PC_BC_OUTFLOW))


def test_fill_ghosts_adjoint_is_the_transpose(cuda_lib):
    """<fill(x), y> = <x, fill^T(y)> on a split level with reflecting and
    outflow faces (momentum sign flips included)."""
    import torch

    from test_gpu_advance import BCS, _split

    mol = cuda_lib
    mech, st, _ = problems.flame((16, 12, 20), seed=72)
    lo_bc, hi_bc = BCS["walls"]
    geom = abi.geometry((0, 0, 0), (15, 11, 19), lo_bc, hi_bc)
    boxes = _split(st, 2)
    op = mol.MOLOperator(problems.make_config(mech))
    rng = np.random.default_rng(3)
    X = to_multifab(mol, boxes, 4)
    Y = mol.MultiFab(X.boxes, X.ncomp, 4, fabs=[torch.from_numpy(rng.normal(size=t.shape)).cuda() for t in X.fabs])
    Y0 = [t.clone() for t in Y.fabs]
    op.fill_ghosts(X, geom)
    op.fill_ghosts_adjoint(Y, geom)
    torch.cuda.synchronize()
    a = sum(float((x * y).sum()) for x, y in zip(X.fabs, Y0))
    # x before the fill on its valid cells only: the filled ghosts are functions of them
    xv = [t.clone() for t in X.fabs]
    for t in xv:
        t[:, :4] = 0
        t[:, -4:] = 0
        t[:, :, :4] = 0
        t[:, :, -4:] = 0
        t[:, :, :, :4] = 0
        t[:, :, :, -4:] = 0
    b = sum(float((x * y).sum()) for x, y in zip(xv, Y.fabs))
    assert abs(a - b) <= 1e-12 * abs(a), (a, b)
    for t in Y.fabs:  # ghosts zeroed
        assert float(t[:, :4].abs().sum()) == 0.0


def test_compute_temp_adjoint_matches_finite_differences(cuda_lib):
    import torch

    mol = cuda_lib
    mech, st, _ = _flame((12, 10, 8))
    op = mol.MOLOperator(problems.make_config(mech))
    rng = np.random.default_rng(4)
    S = to_multifab(mol, [st], 4)
    op.compute_temp(S)
    base = S.fabs[0].clone()
    s = rng.normal(size=st.S.shape[0])
    s[abi.UEINT] = s[abi.UTEMP] = 0.0
    v = torch.from_numpy(s[:, None, None, None] * st.S).cuda()
    lam = torch.from_numpy(rng.normal(size=st.S.shape)).cuda()
    Lb = mol.MultiFab(S.boxes, S.ncomp, 4, fabs=[lam.clone()])
    op.compute_temp_adjoint(S, Lb)

    def ct(h):
        T = mol.MultiFab(S.boxes, S.ncomp, 4, fabs=[base + h * v])
        op.compute_temp(T)
        return T.fabs[0]

    g = 4
    val = (slice(None), slice(g, -g), slice(g, -g), slice(g, -g))
    h = 1e-7
    fd = (ct(h) - ct(-h)) / (2 * h)
    a = float((fd[val] * lam[val]).sum())
    b = float((v[val] * Lb.fabs[0][val]).sum())
    print("computeTemp adjoint", b, "FD", a)
    assert abs(a - b) <= 1e-6 * abs(b)


def _setup(mol, nsteps, every, shape=(16, 16, 16), params=None):
    from pelec_gb300 import trajectory

    mech, st, fp = _flame(shape, params=params)
    op = mol.MOLOperator(problems.make_config(mech))
    S0 = to_multifab(mol, [st], 4)
    tr = trajectory.Trajectory(op, S0, _geom(st), st.dx)
    return mech, st, fp, op, S0, tr


def test_trajectory_gradient_matches_gpu_finite_differences(cuda_lib):
    import torch

    mol = cuda_lib
    mech, st, fp, op, S0, tr = _setup(mol, 6, 2)
    dts = tr.dt_sequence(S0, 6, 0.3)
    J, L = tr.gradient(S0, dts, every=2)
    torch.cuda.synchronize()
    rng = np.random.default_rng(8)
    g = 4
    for trial in range(3):
        s = rng.normal(size=st.S.shape[0])
        s[abi.UEINT] = s[abi.UTEMP] = 0.0
        v = torch.from_numpy(s[:, None, None, None] * st.S).cuda()
        v[:, :g] = 0
        v[:, -g:] = 0
        v[:, :, :g] = 0
        v[:, :, -g:] = 0
        v[:, :, :, :g] = 0
        v[:, :, :, -g:] = 0
        ad = float((L.fabs[0] * v).sum())
        errs = {}
        for h in (1e-6, 1e-7):
            Jp = tr.objective(tr.run(mol.MultiFab(S0.boxes, S0.ncomp, 4, fabs=[S0.fabs[0] + h * v]), dts)[0])
            Jm = tr.objective(tr.run(mol.MultiFab(S0.boxes, S0.ncomp, 4, fabs=[S0.fabs[0] - h * v]), dts)[0])
            errs[h] = abs((Jp - Jm) / (2 * h) - ad) / abs(ad)
        print("trajectory trial", trial, "dJ.v adjoint", ad, "rel err vs FD", errs)
        assert min(errs.values()) <= GRAD_REL, errs


def test_checkpoint_interval_does_not_change_the_gradient(cuda_lib):
    import torch

    mol = cuda_lib
    mech, st, fp, op, S0, tr = _setup(mol, 6, 1, shape=(12, 12, 12))
    dts = tr.dt_sequence(S0, 6, 0.3)
    grads = []
    for every in (1, 2, 3, 6):
        J, L = tr.gradient(S0, dts, every=every)
        grads.append(L.fabs[0].clone())
    torch.cuda.synchronize()
    for gr in grads[1:]:
        err = float((gr - grads[0]).abs().max() / grads[0].abs().max())
        assert err <= 1e-12, err


def test_trajectory_gradient_matches_oracle_finite_differences(cuda_lib, oracle_lib):
    """FD of the oracle's CPU trajectory (fill, RHS, LinComb, computeTemp
    restated in C++) against the GPU adjoint."""
    import torch

    mol = cuda_lib
    mech, st, fp, op, S0, tr = _setup(mol, 4, 2, shape=(12, 12, 12))
    dts = tr.dt_sequence(S0, 4, 0.3)
    J, L = tr.gradient(S0, dts, every=2)
    torch.cuda.synchronize()
    cfg = problems.make_config(mech)
    geom = _geom(st)
    rng = np.random.default_rng(12)
    s = rng.normal(size=st.S.shape[0])
    s[abi.UEINT] = s[abi.UTEMP] = 0.0
    v = s[:, None, None, None] * st.S
    g = 4
    mask = np.zeros(st.S.shape[1:], bool)
    mask[g:-g, g:-g, g:-g] = True
    v = v * mask
    ad = float((L.fabs[0].cpu().numpy() * v).sum())

    def Jcpu(h):
        boxes = [problems.BoxState(st.lo, st.hi, st.S + h * v, st.dx)]
        for dt in dts:
            boxes = oracle_lib.ssprk2_step(cfg, boxes, geom, dt)
        T = boxes[0].S[abi.UTEMP, g:-g, g:-g, g:-g]
        return float(T.sum()) * float(np.prod(st.dx))

    h = 1e-7
    fd = (Jcpu(h) - Jcpu(-h)) / (2 * h)
    print("oracle FD", fd, "adjoint", ad, "rel", abs(fd - ad) / abs(ad))
    assert abs(fd - ad) <= GRAD_REL * abs(ad)


def test_inflow_parameter_gradient(cuda_lib):
    """dJ/da for the amplitudes of the first three wrinkle modes: the
    adjoint gradient contracted with dU0/da (central differences of the
    initial-condition generator) against FD of J in a."""
    import torch

    mol = cuda_lib
    mech, st, fp, op, S0, tr = _setup(mol, 4, 2, shape=(12, 12, 16))
    dts = tr.dt_sequence(S0, 4, 0.3)
    J, L = tr.gradient(S0, dts, every=2)
    lam = L.fabs[0].cpu().numpy()

    def U0(amps):
        p = dataclasses.replace(fp, amps=np.asarray(amps, float))
        return _flame((12, 12, 16), params=p)[1].S

    for m in range(3):
        ha = 1e-3 * max(fp.amps[m], 1e-6)
        a_p, a_m = fp.amps.copy(), fp.amps.copy()
        a_p[m] += ha
        a_m[m] -= ha
        dU = (U0(a_p) - U0(a_m)) / (2 * ha)
        ad = float((lam * dU).sum())

        def Ja(amps):
            S = mol.MultiFab(S0.boxes, S0.ncomp, 4, fabs=[torch.from_numpy(U0(amps)).cuda()])
            return tr.objective(tr.run(S, dts)[0])

        h = 1e-6 * fp.amps[m]
        a_p, a_m = fp.amps.copy(), fp.amps.copy()
        a_p[m] += h
        a_m[m] -= h
        fd = (Ja(a_p) - Ja(a_m)) / (2 * h)
        print("mode", m, "dJ/da adjoint", ad, "FD", fd, "rel", abs(fd - ad) / abs(ad))
        assert abs(fd - ad) <= 1e-5 * abs(ad)


def test_autograd_wrapper_backward_is_the_adjoint(cuda_lib):
    import torch

    from pelec_gb300 import autograd

    mol = cuda_lib
    mech, st, _ = _flame((12, 10, 8))
    op = mol.MOLOperator(problems.make_config(mech))
    S = torch.from_numpy(st.S.copy()).cuda().requires_grad_(True)
    R = autograd.mol_rhs(op, S, st.lo, st.hi, st.dx)
    mu = torch.from_numpy(np.random.default_rng(2).normal(size=R.shape)).cuda()
    (R * mu).sum().backward()
    Sm = to_multifab(mol, [st], 4)
    Rb = mol.MultiFab(Sm.boxes, Sm.ncomp, 0, fabs=[mu.clone()])
    Ub = mol.MultiFab(Sm.boxes, Sm.ncomp, 4)
    op.rhs_vjp(Sm, Rb, Ub, st.dx)
    torch.cuda.synchronize()
    ref = Ub.fabs[0]
    err = float((S.grad - ref).abs().max() / ref.abs().max())
    assert err <= 1e-13, err
    assert float(S.grad[:, :2].abs().sum()) == 0.0  # outside grow(valid, 2)
