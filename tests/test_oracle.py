"""CPU tests of the oracle (the CPU restatement of getMOLSrcTerm).

The oracle is pinned bit for bit to PeleC's own hot-path code compiled from
the reference tree (tests/test_ref_pinned.py) and to golden fixtures that
code computed (tests/golden/).  The tests here add what the reference's own
tests and physics pin: conservation of mass/momentum/energy on periodic
domains (the intent of Tests/test_masscons.py:20-28, rtol 1e-13), a uniform
state giving a zero RHS, axis-permutation symmetry, zero species diffusion
for one species, second-order convergence (Tests/CMakeLists.txt:134-173),
the Riemann solver's exact Euler flux for equal states, and Newton recovery
of T.
"""
import os

import numpy as np
import pytest

from conftest import divergence_scale
from pelec_gb300 import abi, mechanism, problems

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _uniform_state(mech, n=6):
    T = np.full((n + 8,) * 3, 1200.0)
    if mech.nspec == 1:
        Y = np.ones((1,) + T.shape)
    else:
        Y = np.array([0.02, 0.2, 0.1, 1e-4, 2e-4, 3e-4, 1e-5, 2e-6, 0.0])
        Y[-1] = 1.0 - Y[:-1].sum()
        Y = np.broadcast_to(Y[:, None, None, None], (9,) + T.shape).copy()
    p = np.full(T.shape, mechanism.P_ATM)
    rho = p * mech.wbar(Y) / (mechanism.RU * T)
    u = np.full(T.shape, 30.0)
    v = np.full(T.shape, -12.0)
    w = np.full(T.shape, 7.0)
    S = problems.conserved(mech, rho, u, v, w, T, Y)
    return problems.BoxState(lo=(0, 0, 0), hi=(n - 1,) * 3, S=S, dx=(1e-3,) * 3)


@pytest.mark.parametrize("which", ["gamma", "mix"])
def test_uniform_state_gives_zero_rhs(oracle_lib, which):
    mech = mechanism.gamma_law_single() if which == "gamma" else mechanism.h2_air_synthetic()
    st = _uniform_state(mech)
    R, = oracle_lib.mol_rhs(problems.make_config(mech), [st])
    # Fluxes are equal on every face; their differences vanish exactly.
    assert np.abs(R).max() == 0.0


def test_tgv_periodic_conservation(oracle_lib):
    mech, st = problems.tgv(16, seed=3)
    (R, F), = oracle_lib.mol_rhs_fluxes(problems.make_config(mech), [st])
    scale = divergence_scale(F, st.dx[0] * st.dx[1] * st.dx[2])
    for n in (abi.URHO, abi.UMX, abi.UMY, abi.UMZ, abi.UEDEN):
        assert abs(R[n].sum()) <= 1e-15 * scale[n], n
    # Single species: rho*Y equation equals the continuity equation.
    assert np.array_equal(R[abi.UFS], R[abi.URHO])
    assert np.all(R[abi.UTEMP] == 0.0)


def test_flame_periodic_xy_conservation(oracle_lib):
    mech, st, _ = problems.flame((8, 8, 8), seed=2)
    # make z periodic too so every conserved total must vanish
    problems.fill_ghosts(st.S, 4, ("periodic",) * 3)
    (R, F), = oracle_lib.mol_rhs_fluxes(problems.make_config(mech), [st])
    scale = divergence_scale(F, st.dx[0] * st.dx[1] * st.dx[2])
    for n in [abi.URHO, abi.UMX, abi.UMY, abi.UMZ, abi.UEDEN] + [abi.UFS + k for k in range(9)]:
        assert abs(R[n].sum()) <= 1e-15 * scale[n], n
    # Species equations sum to the continuity equation (Sum rhoY_k = rho).
    assert np.allclose(R[abi.UFS:].sum(axis=0), R[abi.URHO], rtol=0, atol=1e-10 * np.abs(R[abi.URHO]).max())


def test_axis_permutation_symmetry(oracle_lib):
    mech, st = problems.tgv(12, seed=5)
    cfg = problems.make_config(mech)
    R, = oracle_lib.mol_rhs(cfg, [st])
    # swap x and y: array axes (n, z, y, x) -> (n, z, x, y), momentum UMX<->UMY
    S2 = st.S.transpose(0, 1, 3, 2).copy()
    S2[[abi.UMX, abi.UMY]] = S2[[abi.UMY, abi.UMX]]
    st2 = problems.BoxState(lo=st.lo, hi=st.hi, S=np.ascontiguousarray(S2), dx=st.dx)
    R2, = oracle_lib.mol_rhs(cfg, [st2])
    R2b = R2.transpose(0, 1, 3, 2).copy()
    R2b[[abi.UMX, abi.UMY]] = R2b[[abi.UMY, abi.UMX]]
    scale = np.abs(R).max(axis=(1, 2, 3)) + 1e-300
    err = np.abs(R2b - R).max(axis=(1, 2, 3)) / scale
    assert err.max() < 1e-12


def test_second_order_convergence_of_diffusion(oracle_lib):
    """Viscous-only RHS of a smooth shear wave converges at second order."""
    mech = mechanism.gamma_law_single(mu=1.0)
    errs = []
    for n in (16, 32):
        dx = 2 * np.pi / n
        x = (np.arange(-4, n + 4) + 0.5) * dx
        Z, Yg, X = np.meshgrid(x, x, x, indexing="ij")
        u = np.zeros_like(X)
        v = np.sin(X)
        w = np.zeros_like(X)
        rho = np.full(X.shape, 1.0)
        T = np.full(X.shape, 300.0)
        S = problems.conserved(mech, rho, u, v, w, T, np.ones((1,) + X.shape))
        st = problems.BoxState(lo=(0, 0, 0), hi=(n - 1,) * 3, S=S, dx=(dx,) * 3)
        cfg = problems.make_config(mech, do_hydro=0, diffuse=0, diffuse_vel=1)
        R, = oracle_lib.mol_rhs(cfg, [st])
        xc = (np.arange(n) + 0.5) * dx
        exact = -np.sin(xc)  # d/dx(mu dv/dx) with mu = 1, rho v_t = ...
        # the RHS of rho*v is +d/dx(mu dv/dx) = -sin(x)
        errs.append(np.abs(R[abi.UMY][0, 0, :] - exact).max())
    order = np.log2(errs[0] / errs[1])
    assert order > 1.9


def test_riemann_equal_states_is_euler_flux(oracle_lib):
    mech = mechanism.h2_air_synthetic()
    cfg = problems.make_config(mech)
    Y = np.array([0.02, 0.2, 0.1, 1e-4, 2e-4, 3e-4, 1e-5, 2e-6, 0.0])
    Y[-1] = 1 - Y.sum()
    rho, un, ut1, ut2, p = 3.1e-4, 250.0, -3.0, 4.0, 1.2e6
    st = np.concatenate([[rho, un, ut1, ut2, p], Y])
    F, ustar = oracle_lib.riemann_face(cfg, st, st, 9e4)
    e = oracle_lib.thermo(cfg, p * oracle_lib.thermo(cfg, 1000.0, Y)[3] / (rho * mechanism.RU), Y)[0]
    assert abs(ustar - un) <= 1e-12 * un
    assert np.isclose(F[abi.URHO], rho * un, rtol=1e-13)
    assert np.isclose(F[abi.UMX], rho * un * un + p, rtol=1e-13)
    assert np.isclose(F[abi.UMY], rho * un * ut1, rtol=1e-13)
    assert np.isclose(F[abi.UEDEN], un * (rho * e + 0.5 * rho * (un ** 2 + ut1 ** 2 + ut2 ** 2) + p), rtol=1e-12)
    assert np.allclose(F[abi.UFS:], rho * un * Y, rtol=1e-12, atol=1e-300)


def test_ctoprim_recovers_temperature(oracle_lib):
    mech = mechanism.h2_air_synthetic()
    cfg = problems.make_config(mech)
    Y = np.array([0.02, 0.2, 0.1, 1e-4, 2e-4, 3e-4, 1e-5, 2e-6, 0.0])
    Y[-1] = 1 - Y.sum()
    for T in (310.0, 999.0, 1001.0, 2400.0):
        rho = 2e-4
        e = mech.mixture_e(np.array(T), Y)
        U = np.zeros(16)
        U[abi.URHO] = rho
        U[abi.UMX] = rho * 10.0
        U[abi.UEDEN] = rho * (float(e) + 50.0)
        U[abi.UTEMP] = T * 0.8  # Newton must recover T from a poor guess
        U[abi.UFS:] = rho * Y
        q, qa, ok = oracle_lib.ctoprim_cell(cfg, U)
        assert ok
        assert abs(q[7] - T) <= 1e-11 * T
        assert np.isclose(q[5], rho * mechanism.RU / mech.wbar(Y) * T, rtol=1e-13)


def _golden_cases(g):
    """(name, BoxState, config, expected RHS) of every RHS in the fixtures."""
    from golden.make_golden import FLAME_FLAGS

    out = []
    for case, flag_sets in (("tgv8", {"": {}}), ("flame6", {"": {}, **FLAME_FLAGS}), ("flame576", {"": {}})):
        S = np.ascontiguousarray(g[f"{case}_S"])
        n = [S.shape[3] - 8, S.shape[2] - 8, S.shape[1] - 8]
        mech = mechanism.gamma_law_single() if case.startswith("tgv") else mechanism.h2_air_synthetic()
        st = problems.BoxState(lo=(0, 0, 0), hi=tuple(v - 1 for v in n), S=S, dx=tuple(g[f"{case}_dx"]))
        for name, flags in flag_sets.items():
            key = f"{case}_{name}_R" if name else f"{case}_R"
            out.append((key, st, problems.make_config(mech, **flags), g[key]))
    return out


def test_golden_fixtures(oracle_lib):
    """The oracle reproduces, bit for bit, the fixtures that PeleC's own
    hot-path code computed (tests/golden/make_golden.py): every flag case and
    the exported face fluxes."""
    g = np.load(os.path.join(GOLDEN, "mol_rhs_golden.npz"))
    for key, st, cfg, ref in _golden_cases(g):
        R, = oracle_lib.mol_rhs(cfg, [st])
        np.testing.assert_array_equal(R, ref, err_msg=key)
    key, st, cfg, _ = _golden_cases(g)[1]
    (R, F), = oracle_lib.mol_rhs_fluxes(cfg, [st])
    for d in range(3):
        np.testing.assert_array_equal(F[d], g[f"flame6_F{d}"], err_msg=f"flux {d}")


def test_generators_are_deterministic():
    """The committed fixtures' inputs are what the seeded generators produce."""
    g = np.load(os.path.join(GOLDEN, "mol_rhs_golden.npz"))
    _, st = problems.tgv(8, seed=11)
    np.testing.assert_allclose(st.S, g["tgv8_S"], rtol=1e-14, atol=0)
    _, st, _ = problems.flame((6, 6, 6), seed=12)
    np.testing.assert_allclose(st.S, g["flame6_S"], rtol=1e-14, atol=0)
    _, st, _ = problems.flame((5, 7, 6), seed=13)
    np.testing.assert_allclose(st.S, g["flame576_S"], rtol=1e-14, atol=0)


def test_rhs_conditioning(oracle_lib):
    """One random ulp on the input state moves the oracle's own RHS by more
    than the 1e-12 FP64 parity bar (flame z-momentum, where the 1 atm pressure
    flux cancels between faces): parity at that bar needs the same IEEE
    operation sequence, not merely a correct one."""
    from conftest import rel_maxnorm

    mech, st, _ = problems.flame((16, 16, 24), seed=6)
    cfg = problems.make_config(mech)
    R0, = oracle_lib.mol_rhs(cfg, [st])
    rng = np.random.default_rng(0)
    S1 = st.S * (1.0 + 2.0 ** -52 * rng.choice([-1.0, 1.0], st.S.shape))
    R1, = oracle_lib.mol_rhs(cfg, [problems.BoxState(lo=st.lo, hi=st.hi, S=S1, dx=st.dx)])
    err = rel_maxnorm(R1, R0)
    assert err.max() > 1e-11


def test_oracle_ssprk2_conserves_and_is_stable(oracle_lib):
    """Three MOL steps at the estTimeStep CFL-0.3 time step on a periodic
    flame: finite, positive radicals, closed totals."""
    geom = abi.geometry((0, 0, 0), (11, 11, 11), (0, 0, 0), (0, 0, 0))
    mech, st, _ = problems.flame((12, 12, 12), seed=8)
    cfg = problems.make_config(mech)
    oracle_lib.fill_ghosts([st], geom, 4)
    dt, parts = oracle_lib.est_dt(cfg, [st], 0.3)
    assert 0 < dt <= 0.3 * min(parts)
    t0 = st.valid(st.S).sum(axis=(1, 2, 3))
    scale = np.abs(st.valid(st.S)).sum(axis=(1, 2, 3))
    new = [st]
    for _ in range(3):
        new = oracle_lib.ssprk2_step(cfg, new, geom, dt)
    v = new[0].valid(new[0].S)
    assert np.all(np.isfinite(v))
    assert (v[abi.UFS:] / v[abi.URHO]).min() > -1e-12
    t1 = v.sum(axis=(1, 2, 3))
    for n in [abi.URHO, abi.UMX, abi.UMY, abi.UMZ, abi.UEDEN]:
        assert abs(t1[n] - t0[n]) <= 1e-13 * scale[n], n


def test_oracle_fill_ghosts_periodic_matches_generator(oracle_lib):
    mech, st, _ = problems.flame((8, 6, 10), seed=9)
    problems.fill_ghosts(st.S, 4, ("periodic",) * 3)
    want = st.S.copy()
    st.S[:, :4] = -1.0
    st.S[:, :, :, -4:] = -1.0
    oracle_lib.fill_ghosts([st], abi.geometry((0, 0, 0), (7, 5, 9), (0, 0, 0), (0, 0, 0)), 4)
    np.testing.assert_array_equal(st.S, want)


def test_oracle_face_fluxes_difference_to_the_rhs(oracle_lib):
    """The oracle's exported face fluxes (refluxing data) difference to its
    own RHS: RHS = -div(F) / V, bit for bit."""
    mech, st, _ = problems.flame((8, 6, 10), seed=93)
    cfg = problems.make_config(mech)
    (R, F), = oracle_lib.mol_rhs_fluxes(cfg, [st])
    R2, = oracle_lib.mol_rhs(cfg, [st])
    np.testing.assert_array_equal(R, R2)
    fx, fy, fz = F
    # pc_flux_div's order (Diffterm.H:475-481), elementwise in numpy: the same bits
    div = fx[..., 1:] - fx[..., :-1] + fy[:, :, 1:] - fy[:, :, :-1] + fz[:, 1:] - fz[:, :-1]
    vol = st.dx[0] * st.dx[1] * st.dx[2]
    np.testing.assert_array_equal(-div / vol, R)


def _ulp_err(got, x, fn):
    """|got - f(x)| in ulps of the correctly rounded f(x), f by 60-digit decimal."""
    import math
    from decimal import Decimal, getcontext

    getcontext().prec = 60
    out = []
    for g, xi in zip(got, x):
        exact = fn(Decimal(float(xi)))
        cr = float(exact)
        ulp = math.ulp(cr)
        out.append(abs(Decimal(float(g)) - exact) / Decimal(ulp))
    return np.array([float(v) for v in out])


def test_shared_exp_is_within_one_ulp(oracle_lib):
    """pc_exp.h's exp (the transport's, on the GPU and in the oracle) against
    60-digit decimal exp: within one ulp everywhere tried, correctly rounded
    in nearly every case; the library function beyond |x| >= 700."""
    from oracle import pyoracle

    rng = np.random.default_rng(5)
    x = np.concatenate([rng.uniform(-50, 50, 4000), rng.uniform(-699, 699, 1000),
                        rng.uniform(-1e-3, 1e-3, 500), [0.0, -0.0, 1e-300, -1e-300, 1.0, -1.0, 699.9, -699.9]])
    y = pyoracle.exp_log(0, x)
    err = _ulp_err(y, x, lambda d: d.exp())
    assert err.max() < 1.0, err.max()
    assert (err <= 0.5).mean() > 0.99
    big = np.array([700.0, -700.0, 710.0, -746.0, np.inf, -np.inf])
    with np.errstate(over="ignore"):
        np.testing.assert_array_equal(pyoracle.exp_log(0, big), np.exp(big))
    assert np.isnan(pyoracle.exp_log(0, np.array([np.nan])))[0]


def test_shared_log_is_within_one_ulp(oracle_lib):
    from oracle import pyoracle

    rng = np.random.default_rng(6)
    x = np.concatenate([10.0 ** rng.uniform(-300, 300, 3000), rng.uniform(200.0, 4000.0, 1000),
                        1.0 + rng.uniform(-0.02, 0.02, 1000), [1.0, 2.0, 0.5, 1e-308, 1.7e308, 1.0 + 2.0 ** -52]])
    y = pyoracle.exp_log(1, x)
    err = _ulp_err(y, x, lambda d: d.ln())
    err = err[x != 1.0]
    assert err.max() < 1.0, err.max()
    assert (err <= 0.5).mean() > 0.99
    assert pyoracle.exp_log(1, np.array([1.0]))[0] == 0.0
    edge = np.array([0.0, 1e-320, np.inf])
    with np.errstate(divide="ignore"):
        np.testing.assert_array_equal(pyoracle.exp_log(1, edge), np.log(edge))
