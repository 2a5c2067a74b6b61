"""GPU test of pc_mol_rhs_box_static, the entry point that allocates no
device memory (for callers that cannot call cudaMalloc while they run, for
example code running under a memory pool that forbids other allocations, or
an application that reserved all device memory at start-up).

It must give the same right-hand side as pc_mol_rhs_level on the same box —
bit for bit, since it launches the same kernels (FP64, and the mixed forms)
— on consecutive calls
that reuse its fixed device array, and must refuse a box that does not fit
that array.  This file is collected last so that a run stopping at the first
failure has already run every other test.
"""
import ctypes
from ctypes import POINTER, c_double, c_int, c_void_p

import numpy as np
import pytest

from conftest import rel_maxnorm
from gpu_util import gpu_rhs
from pelec_gb300 import abi, mechanism, problems

pytestmark = pytest.mark.gpu

RTOL = 1e-12  # the FP64 parity bar used by the other GPU tests


def _static_fn(mol):
    fn = mol.library().pc_mol_rhs_box_static
    fn.argtypes = [POINTER(abi.PcMolConfig), POINTER(abi.PcBoxDesc), POINTER(c_double), c_void_p]
    fn.restype = c_int
    return fn


def _run_static(mol, cfg, st):
    import torch

    fn = _static_fn(mol)
    S = torch.from_numpy(np.ascontiguousarray(st.S)).cuda()
    nx, ny, nz = st.shape
    R = torch.full((st.S.shape[0], nz, ny, nx), float("nan"), dtype=torch.float64, device="cuda")
    desc = abi.box_desc(st.lo, st.hi, abi.array4(S.data_ptr(), S.shape, st.begin),
                        abi.array4(R.data_ptr(), R.shape, st.lo))
    dx = (c_double * 3)(*st.dx)
    stream = torch.cuda.current_stream().cuda_stream
    rc = fn(ctypes.byref(cfg), ctypes.byref(desc), dx, c_void_p(stream))
    torch.cuda.synchronize()
    return rc, R.cpu().numpy()


def test_static_entry_matches_level_entry_on_consecutive_calls(cuda_lib):
    mol = cuda_lib
    mech9, flameA, _ = problems.flame((20, 16, 12), seed=31)
    _, flameB, _ = problems.flame((24, 24, 24), seed=32)
    mech1, tgv = problems.tgv(32, seed=33)
    mech21, flame21, _ = problems.flame((16, 12, 20), seed=35, mech=mechanism.drm_synthetic())
    cases = [(problems.make_config(mech9), flameA), (problems.make_config(mech9), flameB),
             (problems.make_config(mech1), tgv), (problems.make_config(mech21), flame21),
             (problems.make_config(mech9), flameA)]
    outs = []
    for cfg, st in cases:  # consecutive calls share the static array
        rc, R = _run_static(mol, cfg, st)
        assert rc == abi.PC_OK, mol.error_string(rc)
        outs.append(R)
    for (cfg, st), R in zip(cases, outs):
        (ref,), _ = gpu_rhs(mol, cfg, [st])
        err = rel_maxnorm(R, ref)
        assert np.all(np.isfinite(R))
        assert err.max() <= RTOL, err
        np.testing.assert_array_equal(R, ref)  # the same kernels: the same bits
    # the repeated box gives the same answer after other boxes used the array
    np.testing.assert_array_equal(outs[0], outs[4])


@pytest.mark.parametrize("precision", [abi.PC_PRECISION_MIXED, abi.PC_PRECISION_MIXED_FP64])
def test_static_entry_mixed_matches_level_entry(cuda_lib, precision):
    """The mixed forms through the static entry: the same kernels as
    pc_mol_rhs_level, so the same bits, at 9 and 21 species and one species
    (GammaLaw), on consecutive calls."""
    mol = cuda_lib
    mech9, flame, _ = problems.flame((20, 16, 12), seed=36)
    mech1, tgv = problems.tgv(24, seed=37)
    mech21, flame21, _ = problems.flame((16, 12, 20), seed=38, mech=mechanism.drm_synthetic())
    cases = [(problems.make_config(m, precision=precision), st)
             for m, st in ((mech9, flame), (mech1, tgv), (mech21, flame21))]
    for cfg, st in cases:
        rc, R = _run_static(mol, cfg, st)
        assert rc == abi.PC_OK, mol.error_string(rc)
        (ref,), _ = gpu_rhs(mol, cfg, [st])
        assert np.all(np.isfinite(R))
        np.testing.assert_array_equal(R, ref)


def test_static_entry_rejects_a_box_that_does_not_fit(cuda_lib):
    mol = cuda_lib
    mech9, st, _ = problems.flame((64, 64, 64), seed=34)
    rc, R = _run_static(mol, problems.make_config(mech9), st)
    assert rc == abi.PC_ERR_TOO_LARGE
    assert np.all(np.isnan(R))  # nothing was launched
