"""GPU tests of the exact twins of the FP64 passes.

The fast cell and flux passes take each quotient by a shared divisor as the
product with the divisor's reciprocal, corrected in integer arithmetic; the
operands that correction does not cover (subnormal, infinite or NaN values,
quotients next to a power of two) are counted, and a twin of the pass,
launched right after it, evaluates the whole pass again with IEEE divisions
when that count is not zero.  These states put subnormal numbers into those
quotients so that the twins run, and the result must still equal the
oracle's bit for bit.
"""
import numpy as np
import pytest

from gpu_util import gpu_rhs
from pelec_gb300 import problems

pytestmark = pytest.mark.gpu


def _same(gpu, ref, what):
    assert np.all(np.isfinite(gpu)), what
    np.testing.assert_array_equal(gpu, ref, err_msg=f"{what}: not bit-identical to the oracle")


def test_subnormal_species_densities_run_the_exact_cell_pass(cuda_lib, oracle_lib):
    """rho Y_k subnormal in a scatter of cells (ghosts included): the cell
    pass's Y_k = rho Y_k / rho has a subnormal numerator there."""
    mech, st, _ = problems.flame((12, 10, 14), seed=41)
    rng = np.random.default_rng(41)
    S = st.S
    n_h2o = 7 + 2
    mask = rng.random(S.shape[1:]) < 0.05
    S[n_h2o][mask] = rng.integers(1, 1 << 40, mask.sum()) * 5e-324
    cfg = problems.make_config(mech)
    ref, = oracle_lib.mol_rhs(cfg, [st])
    for per_box in (False, True):
        (gpu,), status = gpu_rhs(cuda_lib, cfg, [st], per_box=per_box)
        _same(gpu, ref, f"subnormal rho Y, per_box={per_box}")
        assert status.exact_recomputes > 0
        assert status.cells == 12 * 10 * 14


def test_subnormal_velocities_run_the_exact_flux_pass(cuda_lib, oracle_lib):
    """Momenta scaled into the subnormal range on a uniform-pressure
    Taylor-Green box: the Riemann solver's u* numerator and the face-state
    quotients are subnormal, so the flux pass's twin runs."""
    mech, st = problems.tgv(16, seed=42)
    for n in (1, 2, 3):
        st.S[n] *= 1e-318
    cfg = problems.make_config(mech)
    ref, = oracle_lib.mol_rhs(cfg, [st])
    (gpu,), status = gpu_rhs(cuda_lib, cfg, [st])
    _same(gpu, ref, "subnormal momenta")
    assert status.exact_recomputes > 0


def _uniform_gas_with_still_block(n, seed):
    """Uniform density and temperature, seeded velocities, and an 8x8x8
    block at z in [20, 28) whose velocities are subnormal: its kinetic
    energy underflows, so its pressure is exactly uniform, and the Riemann
    solver's u* numerator there is a subnormal number."""
    mech = problems.gamma_law_single()
    rng = np.random.default_rng(seed)
    rho0, T0 = 1.17e-3, 300.0
    shape = (n, n, n)
    rho = np.full(shape, rho0)
    T = np.full(shape, T0)
    vel = [rng.normal(0.0, 3e3, shape) for _ in range(3)]
    for v in vel:
        v[20:28, 0:8, 0:8] *= 1e-318
    Sv = problems.conserved(mech, rho, *vel, T, np.ones((1,) + shape))
    ng = problems.NG
    S = np.zeros((Sv.shape[0], n + 2 * ng, n + 2 * ng, n + 2 * ng))
    S[:, ng:-ng, ng:-ng, ng:-ng] = Sv
    problems.fill_ghosts(S, ng, ("periodic",) * 3)
    dx = 2.0 * np.pi / n
    return mech, problems.BoxState(lo=(0, 0, 0), hi=(n - 1,) * 3, S=S, dx=(dx, dx, dx))


def test_exact_flux_twin_redoes_only_marked_tiles(cuda_lib, oracle_lib):
    """Only the tiles in and around the still block need IEEE divisions.
    With one CTA per tile and with the persistent grid (each CTA runs up z
    columns of tiles, carrying face and slope layers from tile to tile), the
    exact twin evaluates the marked tiles again, those that took a carried
    layer from a marked tile included, and the whole RHS equals the oracle's
    bit for bit."""
    from pelec_gb300 import abi

    mech, st = _uniform_gas_with_still_block(64, seed=45)
    cfg = problems.make_config(mech)
    ref, = oracle_lib.mol_rhs(cfg, [st])
    op = cuda_lib.MOLOperator(cfg)
    for t in (0, abi.PC_LAUNCH_PERSISTENT):
        op.set_tile(t)
        (gpu,), status = gpu_rhs(cuda_lib, cfg, [st], op=op)
        _same(gpu, ref, f"still block, launch configuration {t}")
        assert status.exact_recomputes > 0
        assert status.cells == 64 ** 3


def test_ordinary_states_need_no_exact_pass(cuda_lib, oracle_lib):
    mech, st, _ = problems.flame((16, 16, 16), seed=43)
    cfg = problems.make_config(mech)
    ref, = oracle_lib.mol_rhs(cfg, [st])
    (gpu,), status = gpu_rhs(cuda_lib, cfg, [st])
    _same(gpu, ref, "flame 16^3")
    assert status.exact_recomputes == 0


def test_subnormal_velocities_run_the_exact_face_adjoint(cuda_lib):
    """The vector-Jacobian product on the same state: its face adjoint meets
    the same subnormal quotients, so its exact twin clears the record
    cotangents and accumulates them again.  <mu, J v> from the dual-number
    tangent (IEEE quotients throughout) must equal <J^T mu, v>."""
    import torch

    from gpu_util import to_multifab

    mol = cuda_lib
    mech, st = problems.tgv(12, seed=44)
    for n in (1, 2, 3):
        st.S[n] *= 1e-318
    cfg = problems.make_config(mech)
    rng = np.random.default_rng(44)
    nx, ny, nz = st.shape
    mu = rng.normal(size=(st.S.shape[0], nz, ny, nx))
    g = st.S[:, 2:-2, 2:-2, 2:-2]
    v = rng.normal(size=g.shape) * np.sqrt((g ** 2).mean(axis=(1, 2, 3)))[:, None, None, None]
    v[5] = 0.0
    v[6] = 0.0
    op = mol.MOLOperator(cfg)
    S = to_multifab(mol, [st], st.ng)
    Rb = mol.MultiFab(S.boxes, S.ncomp, 0, fabs=[torch.from_numpy(np.ascontiguousarray(mu)).cuda()])
    Ub = mol.MultiFab(S.boxes, S.ncomp, 2)
    op.rhs_vjp(S, Rb, Ub, st.dx)
    torch.cuda.synchronize()
    assert op.status().exact_recomputes > 0
    Sd = mol.MultiFab(S.boxes, S.ncomp, 2, fabs=[torch.from_numpy(np.ascontiguousarray(v)).cuda()])
    R = mol.MultiFab(S.boxes, S.ncomp, 0)
    Rd = mol.MultiFab(S.boxes, S.ncomp, 0)
    op.rhs_jvp(S, Sd, R, Rd, st.dx)
    torch.cuda.synchronize()
    Jv = Rd.fabs[0].cpu().numpy()
    a = float((mu * Jv).sum())
    b = float((Ub.fabs[0].cpu().numpy() * v).sum())
    assert abs(a - b) <= 1e-10 * float(np.abs(mu * Jv).sum()), (a, b)
