"""GPU tests of PC_PRECISION_FP64_RCP: the FP64 passes with each quotient by a
shared divisor taken as a product with the divisor's correctly rounded
reciprocal (within one ulp of the correctly rounded quotient).

Its results differ from the oracle's arithmetic by rounding, so the measure
is the one round-off obeys: per component n, max|rhs - ref| over the scale
of the terms the RHS is the difference of, max over faces of |F_n| / V
(F_n the exported face flux times area).  A relative max-norm of the RHS
itself is no such measure: where a component's RHS cancels to far below its
fluxes (the C2 flame's z momentum, whose pressure is uniform) one ulp of a
face pressure is a large part of it — a build of the default form with
multiply-add contraction differs from the oracle there by 6e-10 relative.
Measured (C2 flame, TGV, the flag matrix): about 1e-15 of that scale for
momentum, species and energy; about 1e-12 for density on the low-Mach flame
(one ulp of the face pressure moves u* by ulp(p)/(rho c), against
velocities of a few cm/s) and 4e-13 for the energy diffusion of the nearly
isothermal TGV (one ulp of T against its small differences).  Bar:
FLUX_RTOL = 1e-11 of that scale; conservation to round-off; identical
results across launch configurations.
"""
import numpy as np
import pytest

from conftest import divergence_scale
from gpu_util import gpu_rhs, to_multifab
from pelec_gb300 import abi, problems

pytestmark = pytest.mark.gpu

FLUX_RTOL = 1e-11
RCP = abi.PC_PRECISION_FP64_RCP


def _flux_scaled_err(got, ref_rhs, ref_fluxes, dx):
    """Per component: max|got - ref_rhs| / (max_d max|F_d| / V)."""
    vol = float(np.prod(dx))
    scale = np.max([np.abs(F).max(axis=(1, 2, 3)) for F in ref_fluxes], axis=0) / vol
    err = np.abs(got - ref_rhs).max(axis=(1, 2, 3))
    return err / np.where(scale > 0, scale, 1.0)


def _check(got, ref_rhs, ref_fluxes, dx, what):
    assert np.all(np.isfinite(got)), what
    err = _flux_scaled_err(got, ref_rhs, ref_fluxes, dx)
    assert err.max() <= FLUX_RTOL, f"{what}: per-component flux-scaled error {err}"
    return err


def _oracle_case(oracle_lib, mech, boxes, **kw):
    return oracle_lib.mol_rhs_fluxes(problems.make_config(mech, **kw), boxes)


def test_tgv_64_c1(cuda_lib, oracle_lib):
    mech, st = problems.tgv(64, seed=0)
    (ref, F), = _oracle_case(oracle_lib, mech, [st])
    (gpu,), status = gpu_rhs(cuda_lib, problems.make_config(mech, precision=RCP), [st])
    print("tgv64 rcp flux-scaled error:", _check(gpu, ref, F, st.dx, "tgv64").max())
    assert status.cells == 64 ** 3 and status.nonfinite_output == 0


def test_flame_128_c2_against_fp64(cuda_lib):
    """C2 (128^3 flame, 9 species) against the default FP64 form on the GPU
    (the oracle's arithmetic bit for bit) and its exported fluxes."""
    import torch

    mol = cuda_lib
    mech, st, _ = problems.flame((128, 128, 128), seed=1)
    op = mol.MOLOperator(problems.make_config(mech))
    S = to_multifab(mol, [st], st.ng)
    R = mol.MultiFab([(st.lo, st.hi)], st.S.shape[0], 0)
    F, = op.rhs_level_fluxes(S, R, st.dx)
    torch.cuda.synchronize()
    exact = R.fabs[0].cpu().numpy()
    F = [f.cpu().numpy() for f in F]
    op.close()
    (gpu,), status = gpu_rhs(mol, problems.make_config(mech, precision=RCP), [st])
    print("flame 128^3 rcp flux-scaled error:", _check(gpu, exact, F, st.dx, "flame 128^3").max())
    assert status.newton_nonconverged == 0 and status.nonfinite_output == 0


FLAG_CASES = {
    "full": {},
    "hydro_only": dict(diffuse=0),
    "diffusion_only": dict(do_hydro=0),
    "laxf": dict(use_laxf_flux=1),
    "first_order": dict(plm_iorder=1),
    "arithmetic_mean": dict(harmonic=0),
}


@pytest.mark.parametrize("case", sorted(FLAG_CASES))
@pytest.mark.parametrize("phys", ["tgv", "flame"])
def test_flag_matrix(cuda_lib, oracle_lib, case, phys):
    if phys == "tgv":
        mech, st = problems.tgv(12, seed=7)
    else:
        mech, st, _ = problems.flame((10, 9, 12), seed=8)
    (ref, F), = _oracle_case(oracle_lib, mech, [st], **FLAG_CASES[case])
    (gpu,), _ = gpu_rhs(cuda_lib, problems.make_config(mech, precision=RCP, **FLAG_CASES[case]), [st])
    _check(gpu, ref, F, st.dx, f"{phys}/{case}")


def test_uneven_level_and_tiny_boxes(cuda_lib, oracle_lib):
    """Uneven boxes with ragged tiles: batched == per box (bit for bit), both
    within FLUX_RTOL of the oracle."""
    mech, boxes = problems.level_boxes(nboxes=6, seed=21, edges=(8, 16, 24))
    _, big = problems.level_boxes(nboxes=2, seed=22, edges=(24,))
    for st, shp in zip(big, [(1, 1, 1), (9, 17, 5)]):
        nx, ny, nz = shp
        S = np.ascontiguousarray(st.S[:, : nz + 8, : ny + 8, : nx + 8])
        lo = (st.lo[0] + 10000, 0, 0)
        boxes.append(problems.BoxState(lo=lo, hi=tuple(l + n - 1 for l, n in zip(lo, shp)), S=S, dx=st.dx))
    refs = _oracle_case(oracle_lib, mech, boxes)
    cfg = problems.make_config(mech, precision=RCP)
    batched, st1 = gpu_rhs(cuda_lib, cfg, boxes)
    perbox, _ = gpu_rhs(cuda_lib, cfg, boxes, per_box=True)
    for b, (g1, g2, (r, F)) in enumerate(zip(batched, perbox, refs)):
        np.testing.assert_array_equal(g1, g2)
        _check(g1, r, F, boxes[b].dx, f"box {b}")
    assert st1.cells == sum(b.ncells for b in boxes)


def test_every_launch_configuration_identical(cuda_lib):
    import torch

    mol = cuda_lib
    mech, st, _ = problems.flame((40, 24, 20), seed=12, w_noise=1.0)
    op = mol.MOLOperator(problems.make_config(mech, precision=RCP))
    outs = []
    for t in range(abi.PC_NUM_LAUNCH_CONFIGS):
        op.set_tile(t)
        S = to_multifab(mol, [st], st.ng)
        R = mol.MultiFab([(st.lo, st.hi)], st.S.shape[0], 0)
        op.rhs_level(S, R, st.dx)
        torch.cuda.synchronize()
        assert op.current_tile() == t
        outs.append(R.fabs[0].cpu().numpy())
    for t in range(1, len(outs)):
        np.testing.assert_array_equal(outs[t], outs[0], err_msg=f"configuration {t}")


def test_periodic_flame_conservation(cuda_lib):
    mech, st, _ = problems.flame((32, 32, 32), seed=9)
    problems.fill_ghosts(st.S, 4, ("periodic",) * 3)
    op = cuda_lib.MOLOperator(problems.make_config(mech, precision=RCP))
    R = cuda_lib.MultiFab([(st.lo, st.hi)], st.S.shape[0], 0)
    F, = op.rhs_level_fluxes(to_multifab(cuda_lib, [st], st.ng), R, st.dx)
    gpu = R.fabs[0].cpu().numpy()
    scale = divergence_scale([f.cpu().numpy() for f in F], st.dx[0] * st.dx[1] * st.dx[2])
    for n in [abi.URHO, abi.UMX, abi.UMY, abi.UMZ, abi.UEDEN] + [abi.UFS + k for k in range(9)]:
        assert abs(gpu[n].sum()) <= 1e-15 * scale[n], n


def test_face_flux_export(cuda_lib, oracle_lib):
    """Exported face fluxes within FLUX_RTOL of the oracle's (per component, of
    its largest flux in any direction); the RHS is the one without the
    export."""
    import torch

    mol = cuda_lib
    mech, boxes = problems.level_boxes(nboxes=3, seed=91, edges=(8, 12, 20))
    refs = _oracle_case(oracle_lib, mech, boxes)
    cfg = problems.make_config(mech, precision=RCP)
    op = mol.MOLOperator(cfg)
    S = to_multifab(mol, boxes, boxes[0].ng)
    R = mol.MultiFab([(b.lo, b.hi) for b in boxes], S.ncomp, 0)
    F = op.rhs_level_fluxes(S, R, boxes[0].dx)
    torch.cuda.synchronize()
    plain, _ = gpu_rhs(mol, cfg, boxes)
    for b, ((Rref, Fref), Fg, Rg) in enumerate(zip(refs, F, R.fabs)):
        np.testing.assert_array_equal(Rg.cpu().numpy(), plain[b])
        _check(plain[b], Rref, Fref, boxes[b].dx, f"box {b} rhs")
        scale = np.max([np.abs(Fref[d]).max(axis=(1, 2, 3)) for d in range(3)], axis=0)
        for d in range(3):
            got = Fg[d].cpu().numpy()
            err = np.abs(got - Fref[d]).max(axis=(1, 2, 3)) / np.where(scale > 0, scale, 1.0)
            assert err.max() <= FLUX_RTOL, (b, d, err)


def test_derivatives_are_fp64_only(cuda_lib):
    """The VJP and JVP differentiate the default FP64 form; an RCP handle
    reports PC_ERR_UNSUPPORTED for them instead of mixing the two."""
    mol = cuda_lib
    mech, st, _ = problems.flame((8, 8, 8), seed=3)
    op = mol.MOLOperator(problems.make_config(mech, precision=RCP))
    S = to_multifab(mol, [st], st.ng)
    Rbar = mol.MultiFab([(st.lo, st.hi)], st.S.shape[0], 0)
    Sbar = mol.MultiFab([(st.lo, st.hi)], st.S.shape[0], 2)
    with pytest.raises(mol.MOLError) as ei:
        op.rhs_vjp(S, Rbar, Sbar, st.dx)
    assert ei.value.code == abi.PC_ERR_UNSUPPORTED
    R = mol.MultiFab([(st.lo, st.hi)], st.S.shape[0], 0)
    with pytest.raises(mol.MOLError) as ei:
        op.rhs_jvp(S, Sbar, R, Rbar, st.dx)
    assert ei.value.code == abi.PC_ERR_UNSUPPORTED
