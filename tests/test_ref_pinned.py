"""The oracle pinned bit for bit to PeleC's OWN hot-path code.

oracle/ref_build.py compiles the reference's source files where they lie in
the reference tree (Source/MOL.cpp with MOL.H and Riemann.H, Diffterm.H,
Utilities.H, TransCoeff.H, Timestep.H), against stand-ins for the absent
AMReX and PelePhysics headers; oracle/ref_harness.cpp calls them in
getMOLSrcTerm's order.  These tests compare the oracle's restatement
(oracle/pc_oracle.hpp) with that build: equal bits on every output, for the
full C1 and C2 boxes, the flag matrix, ragged and multi-box levels, the
exported face fluxes, single Riemann faces (default and Lax-Friedrichs, the
u* = 0 switch and the rarefaction fan included), single-cell ctoprim, and
the level operations computeTemp and estTimeStep.  The GPU kernels equal the
oracle bit for bit (tests/test_gpu_parity.py), so they are pinned through it.

Not pinned: what PelePhysics supplies (equation of state, transport,
mechanism data).  The reference build runs the oracle's versions of those.

The reference tree exists only where the tests are developed, so these tests
skip elsewhere; the fixtures it produced (tests/golden/) travel instead.
"""
import numpy as np
import pytest

from pelec_gb300 import abi, mechanism, problems

refharness = pytest.importorskip("oracle.refharness")
if not refharness.available():
    pytest.skip("reference sources not present", allow_module_level=True)

FLAGS = {
    "default": {},
    "hydro_only": dict(diffuse=0),
    "diffusion_only": dict(do_hydro=0),
    "laxf": dict(use_laxf_flux=1),
    "first_order": dict(plm_iorder=1),
    "arithmetic_mean": dict(harmonic=0),
    "temp_only": dict(do_hydro=0, diffuse=0, diffuse_temp=1),
    "spec_only": dict(do_hydro=0, diffuse=0, diffuse_spec=1),
    "vel_only": dict(do_hydro=0, diffuse=0, diffuse_vel=1),
    "enth_only": dict(do_hydro=0, diffuse=0, diffuse_enth=1),
    "nothing": dict(do_hydro=0, diffuse=0),
}


def _same(a, b, what):
    np.testing.assert_array_equal(a, b, err_msg=f"{what}: oracle and reference differ")


def test_c1_tgv_64_full_box(oracle_lib):
    mech, st = problems.tgv(64, seed=0)
    cfg = problems.make_config(mech)
    _same(oracle_lib.mol_rhs(cfg, [st])[0], refharness.mol_rhs(cfg, [st])[0], "C1 64^3")


def test_c2_flame_128_full_box(oracle_lib):
    mech, st, _ = problems.flame((128, 128, 128), seed=1)
    cfg = problems.make_config(mech)
    _same(oracle_lib.mol_rhs(cfg, [st])[0], refharness.mol_rhs(cfg, [st])[0], "C2 128^3")


@pytest.mark.parametrize("case", sorted(FLAGS))
@pytest.mark.parametrize("phys", ["tgv", "flame"])
def test_flag_matrix(oracle_lib, phys, case):
    if phys == "tgv":
        mech, st = problems.tgv(16, seed=3)
    else:
        mech, st, _ = problems.flame((12, 10, 14), seed=4)
    cfg = problems.make_config(mech, **FLAGS[case])
    _same(oracle_lib.mol_rhs(cfg, [st])[0], refharness.mol_rhs(cfg, [st])[0], f"{phys}/{case}")


def test_flame_with_w_noise_and_ragged_level(oracle_lib):
    """Non-uniform w (the limiter away from mc(0,0)) and an uneven BoxArray."""
    mech, st, _ = problems.flame((9, 13, 11), seed=6, w_noise=1.0)
    cfg = problems.make_config(mech)
    _same(oracle_lib.mol_rhs(cfg, [st])[0], refharness.mol_rhs(cfg, [st])[0], "w-noise flame")
    mech, boxes = problems.level_boxes(nboxes=5, seed=21, edges=(1, 3, 8, 16))
    cfg = problems.make_config(mech)
    for b, (a, r) in enumerate(zip(oracle_lib.mol_rhs(cfg, boxes), refharness.mol_rhs(cfg, boxes))):
        _same(a, r, f"level box {b}")


def test_face_fluxes(oracle_lib):
    """The fluxes getMOLSrcTerm hands to the flux registers."""
    mech, st, _ = problems.flame((8, 6, 10), seed=8)
    cfg = problems.make_config(mech)
    (Ra, Fa), = oracle_lib.mol_rhs_fluxes(cfg, [st])
    (Rb, Fb), = refharness.mol_rhs(cfg, [st], fluxes=True)
    _same(Ra, Rb, "RHS")
    for d in range(3):
        _same(Fa[d], Fb[d], f"flux {d}")


def _face_states(rng, ns, n):
    """Random Riemann face states [rho, un, ut1, ut2, p, Y...], from subsonic
    to strongly supersonic, with exact u* = 0 pairs and zero species."""
    out = []
    for t in range(n):
        rho = 1e-3 * rng.uniform(0.2, 2.0, 2)
        p = 1e6 * rng.uniform(0.3, 3.0, 2)
        u = rng.normal(0.0, [100.0, 3e4, 2e5][t % 3], 2)
        if t % 7 == 0:  # mirror states: u* = 0 exactly
            rho[1], p[1], u[1] = rho[0], p[0], -u[0]
        Y = rng.dirichlet(np.ones(ns), 2) if ns > 1 else np.ones((2, 1))
        if ns > 1 and t % 5 == 0:
            Y[:, 3] = 0.0
            Y /= Y.sum(axis=1, keepdims=True)
        L = np.concatenate([[rho[0], u[0], rng.normal(0, 50), rng.normal(0, 50), p[0]], Y[0]])
        R = np.concatenate([[rho[1], u[1], rng.normal(0, 50), rng.normal(0, 50), p[1]], Y[1]])
        out.append((L, R, 0.5 * (np.sqrt(1.4 * p[0] / rho[0]) + np.sqrt(1.4 * p[1] / rho[1]))))
    return out


@pytest.mark.parametrize("which", ["gamma", "mix"])
def test_riemann_faces(oracle_lib, which):
    mech = mechanism.gamma_law_single() if which == "gamma" else mechanism.h2_air_synthetic()
    cfg = problems.make_config(mech)
    rng = np.random.default_rng(17)
    fans = 0
    for L, R, cav in _face_states(rng, mech.nspec, 300):
        fa, ua = oracle_lib.riemann_face(cfg, L, R, cav)
        fb, ub = refharness.riemann_face(cfg, L, R, cav)
        _same(fa, fb, "riemann flux")
        assert ua == ub
        fans += abs(ua) > 0 and abs(fa[abi.URHO] - fb[abi.URHO]) == 0 and abs(L[1] - R[1]) > 1e5
        fl, _ = refharness.riemann_face(cfg, L, R, cav, laxf=True)
        assert np.all(np.isfinite(fl))
    assert fans > 0  # strongly supersonic pairs were exercised


def test_laxf_faces_match_oracle_flux_path(oracle_lib):
    """Lax-Friedrichs faces reach the oracle only through the RHS: a box whose
    RHS agrees bit for bit under use_laxf_flux with strong shear."""
    mech, st = problems.tgv(10, seed=9, noise=0.2)
    cfg = problems.make_config(mech, use_laxf_flux=1)
    _same(oracle_lib.mol_rhs(cfg, [st])[0], refharness.mol_rhs(cfg, [st])[0], "laxf strong noise")


@pytest.mark.parametrize("which", ["gamma", "mix"])
def test_ctoprim_cells(oracle_lib, which):
    if which == "gamma":
        mech, st = problems.tgv(6, seed=2)
    else:
        mech, st, _ = problems.flame((6, 6, 6), seed=2)
    cfg = problems.make_config(mech)
    S = st.S.reshape(st.S.shape[0], -1)
    for c in range(0, S.shape[1], 37):
        U = S[:, c].copy()
        U[abi.UTEMP] *= 0.9  # a poor Newton guess
        qa, xa, _ = oracle_lib.ctoprim_cell(cfg, U)
        qb, xb = refharness.ctoprim_cell(cfg, U)
        _same(qa, qb, "q")
        _same(xa, xb, "qaux")


@pytest.mark.parametrize("which", ["gamma", "mix"])
def test_compute_temp_and_est_dt(oracle_lib, which):
    if which == "gamma":
        mech, st = problems.tgv(12, seed=3)
    else:
        mech, st, _ = problems.flame((10, 8, 12), seed=4)
    cfg = problems.make_config(mech)
    a = problems.BoxState(st.lo, st.hi, st.S.copy(), st.dx)
    b = problems.BoxState(st.lo, st.hi, st.S.copy(), st.dx)
    for x in (a, b):  # stale internal energy and temperature, as after a stage update
        x.S[abi.UTEMP] *= 0.9
        x.S[abi.UEDEN] *= 1.0 + 1e-3
    oracle_lib.compute_temp(cfg, [a])
    refharness.compute_temp(cfg, [b])
    _same(a.S, b.S, "computeTemp")
    assert oracle_lib.est_dt(cfg, [st], 0.3)[1] == refharness.est_dt_parts(cfg, [st])


@pytest.mark.parametrize("case", ["default", "laxf", "first_order", "arithmetic_mean", "spec_only"])
def test_21_species(oracle_lib, case):
    """NUM_SPECIES = 21 (the synthetic DRM19-sized mechanism; the reference
    built with -DPC_REF_NS=21)."""
    mech, st, _ = problems.flame((10, 8, 12), seed=4, mech=mechanism.drm_synthetic())
    cfg = problems.make_config(mech, **FLAGS.get(case, {}))
    _same(oracle_lib.mol_rhs(cfg, [st])[0], refharness.mol_rhs(cfg, [st])[0], f"21 species/{case}")
