"""GPU tests of the trajectory adjoint: the transposes of the ghost fill and
of computeTemp, the checkpointed SSP-RK2 adjoint against finite differences
of the GPU and oracle trajectories (J = sum of T dV at the last step) and
against the forward-mode tangent of the trajectory, the C5 configuration
(64^3, 50 steps) against finite differences of the oracle's CPU trajectory
(tests/golden/c5_fd.npz), the inflow-parameter gradient, and the
torch.autograd wrapper."""
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


def _direction(st, s):
    """A state direction: component n of U0 scaled by s[n], valid cells only."""
    import torch

    v = torch.from_numpy(s[:, None, None, None] * st.S).cuda()
    g = st.ng
    for ax in (1, 2, 3):
        v.narrow(ax, 0, g).zero_()
        v.narrow(ax, v.shape[ax] - g, g).zero_()
    return v


def test_trajectory_gradient_matches_gpu_finite_differences(cuda_lib):
    """<dJ/dU0, v> from the checkpointed adjoint against a central difference
    (fixed h = 1e-6, a relative step of the state) of the GPU trajectory."""
    import torch

    mol = cuda_lib
    mech, st, fp, op, S0, tr = _setup(mol, 6, 2)
    dts = tr.dt_sequence(S0, 6, 0.3)
    J, L = tr.gradient(S0, dts, every=2)
    torch.cuda.synchronize()
    rng = np.random.default_rng(8)
    h = 1e-6
    for trial in range(3):
        s = rng.normal(size=st.S.shape[0])
        s[abi.UEINT] = s[abi.UTEMP] = 0.0
        v = _direction(st, s)
        ad = float((L.fabs[0] * v).sum())
        Jp = tr.objective(tr.run(mol.MultiFab(S0.boxes, S0.ncomp, 4, fabs=[S0.fabs[0] + h * v]), dts)[0])
        Jm = tr.objective(tr.run(mol.MultiFab(S0.boxes, S0.ncomp, 4, fabs=[S0.fabs[0] - h * v]), dts)[0])
        err = abs((Jp - Jm) / (2 * h) - ad) / abs(ad)
        print("trajectory trial", trial, "dJ.v adjoint", ad, "rel err vs FD", err)
        assert err <= GRAD_REL, err


@pytest.mark.parametrize("w_noise", [1.0, 0.0])
def test_trajectory_tangent_equals_adjoint(cuda_lib, w_noise):
    """Forward mode through the whole trajectory (dual-number RHS, fill and
    LinComb of the tangent, computeTemp's transpose for the final T) gives
    the adjoint's <dJ/dU0, v> to round-off, with or without the limiter at
    its kink (w_noise = 0: p and w uniform at t = 0)."""
    import torch

    from pelec_gb300 import trajectory

    mol = cuda_lib
    mech, st, fp = problems.flame((16, 12, 20), seed=71, w_noise=w_noise)
    op = mol.MOLOperator(problems.make_config(mech))
    S0 = to_multifab(mol, [st], 4)
    tr = trajectory.Trajectory(op, S0, _geom(st), st.dx)
    dts = tr.dt_sequence(S0, 5, 0.3)
    J, L = tr.gradient(S0, dts, every=2)
    rng = np.random.default_rng(81)
    for trial in range(3):
        s = rng.normal(size=st.S.shape[0])
        s[abi.UEINT] = s[abi.UTEMP] = 0.0
        v = _direction(st, s)
        ad = float((L.fabs[0] * v).sum())
        J2, tan = tr.tangent(S0, dts, mol.MultiFab(S0.boxes, S0.ncomp, 4, fabs=[v]))
        torch.cuda.synchronize()
        print("w_noise", w_noise, "trial", trial, "adjoint", ad, "tangent", tan)
        assert J2 == J
        assert abs(tan - ad) <= 1e-11 * abs(ad), (tan, ad)


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
    """dJ/da for the amplitudes of the first three wrinkle modes: the adjoint
    gradient contracted with dU0/da (central differences of the smooth
    initial-condition generator) equals the forward-mode tangent of the
    trajectory along dU0/da to round-off, and a central difference of J in a
    to GRAD_REL.  The difference of J is summed cell by cell from the two
    final temperature fields (exactly rounded, math.fsum), so the rounding of
    two sums of T does not enter, and the step is small (1e-9 cm): a step of
    1e-7 cm moves some limiter argument across its switch, an error of order
    the step (a few 1e-6 of dJ/da here) that no extrapolation removes."""
    import math

    import torch

    mol = cuda_lib
    mech, st, fp, op, S0, tr = _setup(mol, 4, 2, shape=(12, 12, 16))
    dts = tr.dt_sequence(S0, 4, 0.3)
    J, L = tr.gradient(S0, dts, every=2)
    lam = L.fabs[0].cpu().numpy()
    g = S0.ngrow

    def U0(amps):
        p = dataclasses.replace(fp, amps=np.asarray(amps, float))
        return _flame((12, 12, 16), params=p)[1].S

    def T_final(m, step):
        amps = fp.amps.copy()
        amps[m] += step
        S = mol.MultiFab(S0.boxes, S0.ncomp, 4, fabs=[torch.from_numpy(U0(amps)).cuda()])
        return tr.run(S, dts)[0].fabs[0][abi.UTEMP, g:-g, g:-g, g:-g].cpu().numpy()

    def fd(m, h):
        dT = T_final(m, h) - T_final(m, -h)
        return math.fsum(dT.ravel().tolist()) * tr.vol / (2 * h)

    for m in range(3):
        ha = 1e-3 * max(fp.amps[m], 1e-6)
        dU = (U0(fp.amps + ha * (np.arange(8) == m)) - U0(fp.amps - ha * (np.arange(8) == m))) / (2 * ha)
        ad = float((lam * dU).sum())
        _, tan = tr.tangent(S0, dts, mol.MultiFab(S0.boxes, S0.ncomp, 4, fabs=[torch.from_numpy(dU).cuda()]))
        d9, d8 = fd(m, 1e-9), fd(m, 1e-8)
        print("mode", m, "dJ/da adjoint", ad, "tangent", tan, "FD at 1e-9 cm", d9, "rel", abs(d9 - ad) / abs(ad),
              "at 1e-8 cm: rel", abs(d8 - ad) / abs(ad))
        assert abs(tan - ad) <= 1e-10 * abs(ad)
        assert abs(d9 - ad) <= GRAD_REL * abs(ad)


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


def _c5_fixture():
    import os

    path = os.path.join(os.path.dirname(__file__), "golden", "c5_fd.npz")
    if not os.path.exists(path):
        pytest.skip("tests/golden/c5_fd.npz not generated (tests/golden/make_c5_fd.py)")
    return np.load(path)


@pytest.mark.parametrize("tag", ["wnoise", "config"])
def test_c5_gradient_against_oracle_trajectory_fd(cuda_lib, tag):
    """C5 (64^3 flame, 9 species, FP64, 50 SSP-RK2 steps at CFL 0.3, J = sum
    of T dV, checkpoint every 5): the adjoint dJ/dU0 on the 20 seeded state
    directions of tests/golden/make_c5_fd.py against central differences of
    the ORACLE's CPU trajectory (h = 1e-6 relative), and against the
    forward-mode tangent of the GPU trajectory.

    With w noise every direction agrees with the finite difference to 1e-6.
    In the configuration's own state p and w are uniform up to rounding, so
    the limiter's acoustic slopes and the slopes of w are evaluated at
    arguments of rounding size: a step of 1e-6 moves them across the
    limiter's kink, and the difference quotient measures a different branch
    than the derivative of the branch the trajectory takes.  There the
    tangent, which follows the same branches as the adjoint, must agree to
    round-off, and the finite differences only to the size of that kink."""
    import torch

    from pelec_gb300 import trajectory

    fx = _c5_fixture()
    shape = tuple(int(v) for v in fx["shape"])
    mech, st, fp = problems.flame(shape, seed=int(fx["seed"]), w_noise=1.0 if tag == "wnoise" else 0.0)
    op = cuda_lib.MOLOperator(problems.make_config(mech))
    S0 = to_multifab(cuda_lib, [st], 4)
    tr = trajectory.Trajectory(op, S0, _geom(st), st.dx)
    dts = [float(v) for v in fx[f"{tag}_dts"]]
    J, L = tr.gradient(S0, dts, every=5)
    torch.cuda.synchronize()
    assert abs(J - float(fx[f"{tag}_J0"])) <= 1e-12 * abs(J), (J, float(fx[f"{tag}_J0"]))
    h = float(fx["h_state"])
    fd_errs, tan_errs = [], []
    for d, s in enumerate(fx[f"{tag}_scales"]):
        v = _direction(st, s)
        ad = float((L.fabs[0] * v).sum())
        fd = (float(fx[f"{tag}_Jp"][d]) - float(fx[f"{tag}_Jm"][d])) / (2 * h)
        fd_errs.append(abs(fd - ad) / abs(ad))
        if tag == "config" or d < 4:
            _, tan = tr.tangent(S0, dts, cuda_lib.MultiFab(S0.boxes, S0.ncomp, 4, fabs=[v]))
            tan_errs.append(abs(tan - ad) / abs(ad))
    print(tag, "FD rel errors: max %.3e median %.3e" % (max(fd_errs), float(np.median(fd_errs))),
          "tangent rel errors: max %.3e" % max(tan_errs))
    assert max(tan_errs) <= 1e-10, tan_errs
    if tag == "wnoise":
        assert max(fd_errs) <= GRAD_REL, fd_errs
    else:
        assert max(fd_errs) <= 1e-4, fd_errs


def test_c5_wrinkle_amplitude_gradient_against_oracle_fd(cuda_lib):
    """C5 (b): dJ/da for the first three wrinkle amplitudes — the adjoint
    contracted with dU0/da, and the tangent along dU0/da — against the
    central difference of the oracle's CPU trajectory in a at a step of
    1e-8 cm (J differences summed cell by cell).  A step in a moves the
    flame and some limiter arguments across their switches, an error of
    order the step (no Richardson extrapolation applies); the difference at
    twice the step is printed beside it to show that trend."""
    import torch

    from pelec_gb300 import trajectory

    fx = _c5_fixture()
    shape = tuple(int(v) for v in fx["shape"])
    mech, st, fp = problems.flame(shape, seed=int(fx["seed"]))
    np.testing.assert_array_equal(fp.amps, fx["config_amps"])
    op = cuda_lib.MOLOperator(problems.make_config(mech))
    S0 = to_multifab(cuda_lib, [st], 4)
    tr = trajectory.Trajectory(op, S0, _geom(st), st.dx)
    dts = [float(v) for v in fx["config_dts"]]
    J, L = tr.gradient(S0, dts, every=5)
    lam = L.fabs[0].cpu().numpy()
    h = float(fx["h_amp"])

    def U0(amps):
        return problems.flame(shape, seed=int(fx["seed"]), params=dataclasses.replace(fp, amps=amps))[1].S

    for m in range(3):
        ha = 1e-3 * max(fp.amps[m], 1e-6)
        e = ha * (np.arange(len(fp.amps)) == m)
        dU = (U0(fp.amps + e) - U0(fp.amps - e)) / (2 * ha)
        ad = float((lam * dU).sum())
        _, tan = tr.tangent(S0, dts, cuda_lib.MultiFab(S0.boxes, S0.ncomp, 4, fabs=[torch.from_numpy(dU).cuda()]))
        dJ1, dJ2 = (float(x) for x in fx["config_dJamp"][m])
        fd = dJ1 / (2 * h)
        fd2 = dJ2 / (4 * h)
        print("mode", m, "adjoint", ad, "tangent", tan, "FD", fd, "rel", abs(fd - ad) / abs(ad),
              "FD at twice the step: rel", abs(fd2 - ad) / abs(ad))
        assert abs(tan - ad) <= 1e-10 * abs(ad)
        assert abs(fd - ad) <= GRAD_REL * abs(ad)
