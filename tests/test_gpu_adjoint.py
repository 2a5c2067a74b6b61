"""GPU tests of the hand-written adjoint of the RHS (pc_mol_rhs_vjp) against
central finite differences of the oracle's RHS: for a seeded cotangent mu and
direction v, <VJP(mu), v> must equal d/dh <mu, RHS(U + h v)>."""
import numpy as np
import pytest

from gpu_util import to_multifab
from pelec_gb300 import abi, mechanism, problems

pytestmark = pytest.mark.gpu

# relative agreement of the adjoint with central differences of the oracle
FD_REL = 2e-6


def _case(kind):
    # w noise keeps the limiter away from its kink at mc(0, 0) (uniform p and
    # w), where no linear derivative matches finite differences.
    if kind == "flame":
        mech, st, _ = problems.flame((12, 10, 8), seed=61, w_noise=1.0)
    elif kind == "flame21":  # the 21-species (DRM19-sized) synthetic mechanism
        mech, st, _ = problems.flame((10, 8, 8), seed=64, w_noise=1.0, mech=mechanism.drm_synthetic())
    elif kind == "flame_noslope":
        mech, st, _ = problems.flame((10, 8, 12), seed=63, w_noise=1.0)
    else:
        mech, st = problems.tgv(12, seed=62)
    cfg = problems.make_config(mech, plm_iorder=1 if kind == "flame_noslope" else 4)
    return mech, st, cfg


def _vjp(mol, cfg, st, mu):
    import torch

    op = mol.MOLOperator(cfg)
    S = to_multifab(mol, [st], st.ng)
    Rb = mol.MultiFab(S.boxes, S.ncomp, 0, fabs=[torch.from_numpy(np.ascontiguousarray(mu)).cuda()])
    Ub = mol.MultiFab(S.boxes, S.ncomp, 2)
    for t in Ub.fabs:
        t.fill_(np.nan)  # every entry of grow(valid, 2) must be written
    op.rhs_vjp(S, Rb, Ub, st.dx)
    torch.cuda.synchronize()
    return Ub.fabs[0].cpu().numpy()


def _direction(st, rng):
    """Seeded direction on grow(valid, 2), scaled per component by its RMS."""
    g = st.S[:, 2:-2, 2:-2, 2:-2]
    v = rng.normal(size=g.shape)
    scale = np.sqrt((g ** 2).mean(axis=(1, 2, 3)))
    v *= scale[:, None, None, None]
    v[abi.UEINT] = 0.0
    v[abi.UTEMP] = 0.0
    return v


def _scale_direction(st, rng):
    """Seeded direction that keeps the forward away from its kinks: each
    conserved component is scaled by its own random factor, v_n = s_n U_n.
    The MOL limiter is positively homogeneous, so a componentwise scaling
    moves its arguments almost proportionally and crosses a min/max switch
    only where two arguments agree to within the step; exact zeros stay zero
    and extrapolated ghost layers stay copies of their boundary cell.
    Returned on grow(valid, 2)."""
    s = rng.normal(size=st.S.shape[0])
    s[abi.UEINT] = 0.0
    s[abi.UTEMP] = 0.0
    return np.ascontiguousarray(s[:, None, None, None] * st.S[:, 2:-2, 2:-2, 2:-2])


def _fd(oracle_lib, cfg, st, mu, v, h):
    """Central difference of <mu, RHS(U + t v)> at t = 0, with the RHS
    difference taken cell by cell before the weighted sum (no cancellation
    of the large terms of the sum)."""
    def R(t):
        S = st.S.copy()
        S[:, 2:-2, 2:-2, 2:-2] += t * v
        return oracle_lib.mol_rhs(cfg, [problems.BoxState(st.lo, st.hi, S, st.dx)])[0]

    return float((mu * (R(h) - R(-h))).sum()) / (2.0 * h)


# Steps of the difference quotients, relative changes of the state, fixed.
# Over a whole box a step of 1e-7 or more moves some limiter argument across
# a min/max switch (errors up to 1e-2 on these flames), where the quotient
# measures another branch than the derivative; the directions below are
# therefore local (a few seeded cells), so that the few limiters they reach
# sit far from their switches.  Three nearby steps give the same truncation
# error but independent rounding: their mean is the estimate, their spread
# the estimate's rounding noise (1e-9 of the derivative for directions over
# all components; a few 1e-6 for a direction in the density or momentum
# alone, whose derivative is 1e-4 of the RHS terms it moves).
FD_STEPS = (0.8e-7, 1e-7, 1.25e-7)


def _fd_estimate(oracle_lib, cfg, st, mu, v):
    """(mean, spread) of the central differences at FD_STEPS."""
    vals = np.array([_fd(oracle_lib, cfg, st, mu, v, h) for h in FD_STEPS])
    return float(vals.mean()), float(np.ptp(vals))


def _local_direction(st, rng, ncells=6):
    """A direction confined to ncells seeded valid cells: each conserved
    component of the cell scaled by its own seeded factor.  On grow(valid, 2).

    The cells avoid the first and last valid layer in z.  On the flames z is
    an outflow direction, whose ghost cells are copies of those layers, and
    the difference quotients here hold the ghosts fixed: moving a boundary
    cell alone breaks the exact tie ghost = cell, which sits on kinks of the
    forward (the limiter at mc(0, d), the Riemann solver's shock/rarefaction
    switch at p* = p), so the central difference averages two branches there
    (errors of 1e-2 of the derivative, the same for every step size).  A
    trajectory refills the ghosts and keeps the tie."""
    v = np.zeros_like(st.S[:, 2:-2, 2:-2, 2:-2])
    nz, ny, nx = v.shape[1:]
    for _ in range(ncells):
        k = int(rng.integers(3, nz - 3))
        j, i = (int(rng.integers(2, n - 2)) for n in (ny, nx))
        s = rng.normal(size=st.S.shape[0])
        s[abi.UEINT] = 0.0
        s[abi.UTEMP] = 0.0
        v[:, k, j, i] = s * st.S[:, k + 2, j + 2, i + 2]
    return v


@pytest.mark.parametrize("kind", ["tgv", "flame", "flame_noslope"])
def test_vjp_matches_oracle_finite_differences(cuda_lib, oracle_lib, kind):
    """<VJP(mu), v> against central differences of <mu, RHS(U + h v)>
    computed by the oracle, along local directions (a few seeded cells)."""
    mech, st, cfg = _case(kind)
    rng = np.random.default_rng(7)
    nx, ny, nz = st.shape
    mu = rng.normal(size=(st.S.shape[0], nz, ny, nx))
    Ub = _vjp(cuda_lib, cfg, st, mu)
    assert np.all(np.isfinite(Ub))
    assert not Ub[abi.UEINT].any() and not Ub[abi.UTEMP].any()
    for trial in range(4):
        v = _local_direction(st, rng)
        ad = float((Ub * v).sum())
        fd, noise = _fd_estimate(oracle_lib, cfg, st, mu, v)
        err = abs(fd - ad) / abs(ad)
        print(kind, "trial", trial, "adjoint", ad, "rel err vs FD:", err, "FD noise", noise / abs(ad))
        assert abs(fd - ad) <= FD_REL * abs(ad) + noise, (err, noise / abs(ad))


def test_vjp_component_groups(cuda_lib, oracle_lib):
    """Directions confined to one group of conserved components at a time:
    each link of the chain rule (density, momentum, energy through the EOS
    solve, species through the mixture rules) is checked on its own."""
    mech, st, cfg = _case("flame")
    rng = np.random.default_rng(9)
    nx, ny, nz = st.shape
    mu = rng.normal(size=(st.S.shape[0], nz, ny, nx))
    Ub = _vjp(cuda_lib, cfg, st, mu)
    groups = {"rho": [abi.URHO], "mom": [abi.UMX, abi.UMY, abi.UMZ], "E": [abi.UEDEN],
              "spec": [abi.UFS + k for k in range(9)]}
    for name, comps in groups.items():
        v = _local_direction(st, rng)
        keep = np.zeros(v.shape[0], bool)
        keep[comps] = True
        v[~keep] = 0.0
        ad = float((Ub * v).sum())
        fd, noise = _fd_estimate(oracle_lib, cfg, st, mu, v)
        err = abs(fd - ad) / abs(ad)
        print("group", name, "adjoint", ad, "rel err", err, "FD noise", noise / abs(ad))
        assert abs(fd - ad) <= FD_REL * abs(ad) + noise, (name, err, noise / abs(ad))


def _jvp(mol, cfg, st, v):
    """(RHS, J v) on the GPU; v covers grow(valid, 2)."""
    import torch

    op = mol.MOLOperator(cfg)
    S = to_multifab(mol, [st], st.ng)
    Sd = mol.MultiFab(S.boxes, S.ncomp, 2, fabs=[torch.from_numpy(np.ascontiguousarray(v)).cuda()])
    R = mol.MultiFab(S.boxes, S.ncomp, 0)
    Rd = mol.MultiFab(S.boxes, S.ncomp, 0)
    op.rhs_jvp(S, Sd, R, Rd, st.dx)
    torch.cuda.synchronize()
    return R.fabs[0].cpu().numpy(), Rd.fabs[0].cpu().numpy()


@pytest.mark.parametrize("kind", ["tgv", "flame", "flame_noslope", "flame21"])
def test_jvp_primal_is_the_rhs(cuda_lib, kind):
    from gpu_util import gpu_rhs

    mech, st, cfg = _case(kind)
    v = _direction(st, np.random.default_rng(3))
    R, _ = _jvp(cuda_lib, cfg, st, v)
    (want,), _ = gpu_rhs(cuda_lib, cfg, [st])
    np.testing.assert_array_equal(R, want)


@pytest.mark.parametrize("kind", ["tgv", "flame", "flame_noslope", "flame21"])
def test_dot_product_adjoint_vs_tangent(cuda_lib, kind):
    """<mu, J v> from the dual-number tangent equals <J^T mu, v> from the
    hand-written adjoint to round-off, for seeded mu and v."""
    mech, st, cfg = _case(kind)
    rng = np.random.default_rng(11)
    nx, ny, nz = st.shape
    for trial in range(3):
        mu = rng.normal(size=(st.S.shape[0], nz, ny, nx))
        v = _direction(st, rng)
        _, Jv = _jvp(cuda_lib, cfg, st, v)
        Ub = _vjp(cuda_lib, cfg, st, mu)
        a = float((mu * Jv).sum())
        b = float((Ub * v).sum())
        scale = float(np.abs(mu * Jv).sum())
        print(kind, "trial", trial, "<mu,Jv> =", a, "<J^T mu, v> =", b, "rel", abs(a - b) / abs(a),
              "vs sum|terms|", abs(a - b) / scale)
        assert abs(a - b) <= 1e-10 * scale, (a, b)


@pytest.mark.parametrize("kind", ["tgv", "flame"])
def test_jvp_matches_oracle_finite_differences(cuda_lib, oracle_lib, kind):
    """The dual-number tangent against central differences of the oracle RHS,
    cell by cell.  A step that crosses a limiter switch at some face spoils
    the difference quotient of the cells next to it, so the check is that
    99% of the cells agree to 1e-5 of the component's RMS tangent."""
    mech, st, cfg = _case(kind)
    rng = np.random.default_rng(5)
    v = _scale_direction(st, rng)
    _, Jv = _jvp(cuda_lib, cfg, st, v)
    comps = [abi.URHO, abi.UMX, abi.UMY, abi.UMZ, abi.UEDEN] + [abi.UFS + k for k in range(mech.nspec)]

    def R(t):
        S = st.S.copy()
        S[:, 2:-2, 2:-2, 2:-2] += t * v
        return oracle_lib.mol_rhs(cfg, [problems.BoxState(st.lo, st.hi, S, st.dx)])[0]

    h = 1e-7
    fd = (R(h) - R(-h)) / (2 * h)
    bad = 0.0
    for n in comps:
        rms = np.sqrt((Jv[n] ** 2).mean())
        bad = max(bad, float((np.abs(fd[n] - Jv[n]) > 1e-5 * rms).mean()))
    print(kind, "h", h, "largest fraction of cells off by more than 1e-5 RMS:", bad)
    assert bad <= 0.01, bad
