"""GPU parity of the CUDA MOL right-hand side against the oracle.

Every call goes through the C ABI (libpelec_mol.so via ctypes).  The stated
bar for the plain FP64 form is per component max|gpu - oracle| / max|oracle|
<= 1e-12 (RTOL below); the kernels evaluate the oracle's IEEE operation
sequence, transport exp/log included (pc_exp.h), so every check here also
asserts the results are identical bit for bit.
"""
import numpy as np
import pytest

from conftest import divergence_scale, rel_maxnorm
from gpu_util import gpu_rhs, to_multifab
from pelec_gb300 import abi, mechanism, problems

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _check(gpu, ref, rtol=RTOL, what=""):
    err = rel_maxnorm(gpu, ref)
    assert np.all(np.isfinite(gpu)), what
    assert err.max() <= rtol, f"{what}: per-component rel max-norm error {err}"
    np.testing.assert_array_equal(gpu, ref, err_msg=f"{what}: not bit-identical")
    return err


def test_tgv_64_c1_parity(cuda_lib, oracle_lib):
    """Config C1: 64^3 periodic Taylor-Green, GammaLaw, constant transport."""
    mech, st = problems.tgv(64, seed=0)
    cfg = problems.make_config(mech)
    ref, = oracle_lib.mol_rhs(cfg, [st])
    (gpu,), status = gpu_rhs(cuda_lib, cfg, [st])
    err = _check(gpu, ref, what="tgv64")
    print("tgv64 rel max-norm per component:", err)
    assert status.cells == 64 ** 3
    assert status.newton_nonconverged == 0 and status.nonpositive_state == 0 and status.nonfinite_output == 0


def test_flame_small_parity(cuda_lib, oracle_lib):
    mech, st, _ = problems.flame((16, 12, 20), seed=4)
    cfg = problems.make_config(mech)
    ref, = oracle_lib.mol_rhs(cfg, [st])
    (gpu,), status = gpu_rhs(cuda_lib, cfg, [st])
    err = _check(gpu, ref, what="flame 16x12x20")
    print("flame small rel max-norm per component:", err)
    assert status.cells == 16 * 12 * 20


def test_flame_128_c2_parity(cuda_lib, oracle_lib):
    """Config C2: 128^3 flame, 9 species, periodic x/y, extrapolated z."""
    mech, st, _ = problems.flame((128, 128, 128), seed=1)
    cfg = problems.make_config(mech)
    ref, = oracle_lib.mol_rhs(cfg, [st])
    (gpu,), status = gpu_rhs(cuda_lib, cfg, [st])
    err = _check(gpu, ref, what="flame 128^3")
    print("flame 128^3 rel max-norm per component:", err)
    assert status.newton_nonconverged == 0 and status.nonfinite_output == 0


FLAG_CASES = {
    "hydro_only": dict(diffuse=0),
    "diffusion_only": dict(do_hydro=0),
    "laxf": dict(use_laxf_flux=1),
    "first_order": dict(plm_iorder=1),
    "arithmetic_mean": dict(harmonic=0),
    "temp_only": dict(do_hydro=0, diffuse=0, diffuse_temp=1),
    "spec_only": dict(do_hydro=0, diffuse=0, diffuse_spec=1),
    "vel_only": dict(do_hydro=0, diffuse=0, diffuse_vel=1),
    "nothing": dict(do_hydro=0, diffuse=0),
}


@pytest.mark.parametrize("case", sorted(FLAG_CASES))
@pytest.mark.parametrize("phys", ["tgv", "flame"])
def test_flag_matrix(cuda_lib, oracle_lib, case, phys):
    if phys == "tgv":
        mech, st = problems.tgv(12, seed=7)
    else:
        mech, st, _ = problems.flame((10, 9, 12), seed=8)
    cfg = problems.make_config(mech, **FLAG_CASES[case])
    ref, = oracle_lib.mol_rhs(cfg, [st])
    (gpu,), _ = gpu_rhs(cuda_lib, cfg, [st])
    _check(gpu, ref, what=f"{phys}/{case}")


def test_golden_fixtures_on_gpu(cuda_lib):
    """Every fixture that PeleC's own hot-path code computed
    (tests/golden/make_golden.py), flag cases and face fluxes included."""
    import os

    from test_oracle import _golden_cases

    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "mol_rhs_golden.npz"))
    cases = _golden_cases(g)
    for key, st, cfg, ref in cases:
        (gpu,), _ = gpu_rhs(cuda_lib, cfg, [st])
        _check(gpu, ref, what=key)
    key, st, cfg, ref = cases[1]
    op = cuda_lib.MOLOperator(cfg)
    S = to_multifab(cuda_lib, [st], st.ng)
    R = cuda_lib.MultiFab([(st.lo, st.hi)], st.S.shape[0], 0)
    F, = op.rhs_level_fluxes(S, R, st.dx)
    for d in range(3):
        np.testing.assert_array_equal(F[d].cpu().numpy(), g[f"flame6_F{d}"], err_msg=f"flux {d}")


def test_uneven_level_batched_vs_per_box(cuda_lib, oracle_lib):
    """A BoxArray of uneven boxes: one batched launch == per-box launches
    (bit for bit) == oracle (1e-12)."""
    mech, boxes = problems.level_boxes(nboxes=7, seed=21, edges=(8, 16, 24))
    cfg = problems.make_config(mech)
    refs = oracle_lib.mol_rhs(cfg, boxes)
    batched, st1 = gpu_rhs(cuda_lib, cfg, boxes)
    perbox, st2 = gpu_rhs(cuda_lib, cfg, boxes, per_box=True)
    for b, (g1, g2, r) in enumerate(zip(batched, perbox, refs)):
        np.testing.assert_array_equal(g1, g2)
        _check(g1, r, what=f"box {b}")
    assert st1.cells == sum(b.ncells for b in boxes)


def test_tiny_and_odd_boxes(cuda_lib, oracle_lib):
    """Boxes smaller than a tile and with odd extents (ragged tiles)."""
    mech, boxes = problems.level_boxes(nboxes=3, seed=5, edges=(24,))
    shapes = [(1, 1, 1), (3, 5, 2), (9, 17, 5)]
    out = []
    for st, shp in zip(boxes, shapes):
        nx, ny, nz = shp
        S = np.ascontiguousarray(st.S[:, : nz + 8, : ny + 8, : nx + 8])
        out.append(problems.BoxState(lo=st.lo, hi=tuple(l + n - 1 for l, n in zip(st.lo, shp)), S=S, dx=st.dx))
    cfg = problems.make_config(mech)
    refs = oracle_lib.mol_rhs(cfg, out)
    gpus, _ = gpu_rhs(cuda_lib, cfg, out)
    for g, r in zip(gpus, refs):
        _check(g, r, what="tiny")


def test_periodic_flame_conservation(cuda_lib):
    """Fully periodic 32^3 flame: domain totals of every conserved RHS vanish
    to round-off (Tests/test_masscons.py:20-28 checks the same totals)."""
    mech, st, _ = problems.flame((32, 32, 32), seed=9)
    problems.fill_ghosts(st.S, 4, ("periodic",) * 3)
    op = cuda_lib.MOLOperator(problems.make_config(mech))
    R = cuda_lib.MultiFab([(st.lo, st.hi)], st.S.shape[0], 0)
    F, = op.rhs_level_fluxes(to_multifab(cuda_lib, [st], st.ng), R, st.dx)
    gpu = R.fabs[0].cpu().numpy()
    scale = divergence_scale([f.cpu().numpy() for f in F], st.dx[0] * st.dx[1] * st.dx[2])
    for n in [abi.URHO, abi.UMX, abi.UMY, abi.UMZ, abi.UEDEN] + [abi.UFS + k for k in range(9)]:
        assert abs(gpu[n].sum()) <= 1e-15 * scale[n], n


def test_negative_density_is_reported_not_trapped(cuda_lib):
    """A corrupt ghost cell (rho < 0) is counted in the status; the call and
    the context survive."""
    mech, st, _ = problems.flame((8, 8, 8), seed=3)
    S = st.S.copy()
    S[abi.URHO, 2, 6, 6] = -abs(S[abi.URHO, 2, 6, 6])  # z ghost layer 2 (inside grow(valid,2))
    bad = problems.BoxState(lo=st.lo, hi=st.hi, S=S, dx=st.dx)
    (gpu,), status = gpu_rhs(cuda_lib, problems.make_config(mech), [bad])
    assert status.nonpositive_state >= 1
    # the context is still usable
    (gpu2,), status2 = gpu_rhs(cuda_lib, problems.make_config(mech), [st])
    assert status2.nonpositive_state == 0 and np.all(np.isfinite(gpu2))


def test_invalid_arguments(cuda_lib):
    import torch

    mol = cuda_lib
    mech, st, _ = problems.flame((8, 8, 8), seed=3)
    op = mol.MOLOperator(problems.make_config(mech))
    # state with a single ghost layer: rejected before any launch
    S1 = torch.from_numpy(np.ascontiguousarray(st.S[:, 3:-3, 3:-3, 3:-3])).cuda()
    S = mol.MultiFab([(st.lo, st.hi)], 16, 1, fabs=[S1])
    R = mol.MultiFab([(st.lo, st.hi)], 16, 0)
    with pytest.raises(mol.MOLError) as ei:
        op.rhs_level(S, R, st.dx)
    assert ei.value.code == abi.PC_ERR_INVALID_ARGUMENT
    # a box too large for the 32-bit chunk indexing
    with pytest.raises(mol.MOLError):
        big = mol.MultiFab([((0, 0, 0), (5000, 0, 0))], 16, 0, fabs=[torch.zeros(16, 1, 1, 1, dtype=torch.float64,
                                                                                        device="cuda")])
        op.rhs_level(big, big, st.dx)
    # unsupported physics combination
    cfg = problems.make_config(mech)
    cfg.eos = abi.PC_EOS_GAMMA_LAW
    with pytest.raises(mol.MOLError) as ei:
        mol.MOLOperator(cfg)
    assert ei.value.code == abi.PC_ERR_UNSUPPORTED
    # empty level: a no-op
    op.rhs_level(mol.MultiFab([], 16, 4, fabs=[]), mol.MultiFab([], 16, 0, fabs=[]), st.dx)


def test_getMOLSrcTerm_mirror(cuda_lib, oracle_lib):
    """The reference-shaped entry point gives the same answer."""
    import torch

    mol = cuda_lib
    mech, st = problems.tgv(16, seed=2)
    cfg = problems.make_config(mech)
    op = mol.MOLOperator(cfg)
    S = mol.MultiFab([(st.lo, st.hi)], 8, 4, fabs=[torch.from_numpy(st.S).cuda()])
    R = mol.MultiFab([(st.lo, st.hi)], 8, 0)
    op.getMOLSrcTerm(S, R, time=0.0, dt=1e-6, flux_factor=0.5, dx=st.dx)
    ref, = oracle_lib.mol_rhs(cfg, [st])
    _check(R.fabs[0].cpu().numpy(), ref, what="getMOLSrcTerm")


def test_face_flux_export_matches_oracle(cuda_lib, oracle_lib):
    """The exported face fluxes (refluxing data) equal the oracle's bit for
    bit, and the RHS is unchanged by the export and equals -div(F)/V of the
    exported fluxes, summed in pc_flux_div's order, bit for bit."""
    import torch

    mol = cuda_lib
    mech, boxes = problems.level_boxes(nboxes=3, seed=91, edges=(8, 12, 20))
    cfg = problems.make_config(mech)
    refs = oracle_lib.mol_rhs_fluxes(cfg, boxes)
    op = mol.MOLOperator(cfg)
    S = to_multifab(mol, boxes, boxes[0].ng)
    R = mol.MultiFab([(b.lo, b.hi) for b in boxes], S.ncomp, 0)
    F = op.rhs_level_fluxes(S, R, boxes[0].dx)
    torch.cuda.synchronize()
    plain, _ = gpu_rhs(mol, cfg, boxes)
    vol = boxes[0].dx[0] * boxes[0].dx[1] * boxes[0].dx[2]
    for b, ((Rref, Fref), Fg, Rg) in enumerate(zip(refs, F, R.fabs)):
        Rg = Rg.cpu().numpy()
        np.testing.assert_array_equal(Rg, plain[b])
        for d in range(3):
            got = Fg[d].cpu().numpy()
            scale = np.abs(Fref[d]).max(axis=(1, 2, 3))
            err = np.abs(got - Fref[d]).max(axis=(1, 2, 3)) / np.where(scale > 0, scale, 1.0)
            assert err.max() <= 1e-12, (b, d, err)
            np.testing.assert_array_equal(got, Fref[d], err_msg=f"box {b} direction {d}")
        fx, fy, fz = (Fg[d].cpu().numpy() for d in range(3))
        div = fx[..., 1:] - fx[..., :-1] + fy[:, :, 1:] - fy[:, :, :-1] + fz[:, 1:] - fz[:, :-1]
        np.testing.assert_array_equal(-div / vol, Rg)


@pytest.mark.parametrize("case", ["default", "laxf", "first_order", "diffusion_only"])
def test_flame_21_species_parity(cuda_lib, oracle_lib, case):
    """NUM_SPECIES = 21 (the synthetic DRM19-sized mechanism): bit for bit
    equal to the oracle, which is bit for bit the reference's own code at 21
    species too (tests/test_ref_pinned.py)."""
    kw = {"default": {}, "laxf": dict(use_laxf_flux=1), "first_order": dict(plm_iorder=1),
          "diffusion_only": dict(do_hydro=0)}[case]
    mech, st, _ = problems.flame((16, 12, 20), seed=24, mech=mechanism.drm_synthetic())
    cfg = problems.make_config(mech, **kw)
    ref, = oracle_lib.mol_rhs(cfg, [st])
    (gpu,), status = gpu_rhs(cuda_lib, cfg, [st])
    _check(gpu, ref, what=f"21 species/{case}")
    assert status.cells == 16 * 12 * 20 and status.newton_nonconverged == 0
