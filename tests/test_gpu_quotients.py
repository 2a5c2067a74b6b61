"""GPU test of the exact shared-divisor quotient of the FP64 kernels.

The FP64 passes divide by a shared divisor b as the product with its IEEE
reciprocal, corrected in integer arithmetic to the correctly rounded
quotient.  pc_mol_check_quotients runs that routine on arbitrary operands;
its results must equal IEEE division bit for bit, NaNs aside (any NaN).
"""
import ctypes
from ctypes import c_int, c_longlong, c_void_p

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _quotients(mol, a, b):
    import torch

    fn = mol.library().pc_mol_check_quotients
    fn.argtypes = [c_void_p, c_void_p, c_void_p, c_longlong, c_void_p]
    fn.restype = c_int
    ta = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    tb = torch.from_numpy(np.ascontiguousarray(b)).cuda()
    tq = torch.empty_like(ta)
    rc = fn(ta.data_ptr(), tb.data_ptr(), tq.data_ptr(), a.size, c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    torch.cuda.synchronize()
    return tq.cpu().numpy()


def _assert_ieee(a, b, q):
    with np.errstate(all="ignore"):
        ref = a / b
    both_nan = np.isnan(ref) & np.isnan(q)
    bad = (ref.view(np.int64) != q.view(np.int64)) & ~both_nan
    idx = np.flatnonzero(bad)[:5]
    assert not idx.size, [(float.hex(float(a[i])), float.hex(float(b[i])), float.hex(float(q[i])),
                           float.hex(float(ref[i]))) for i in idx]


def _significands(rng, n, kind):
    if kind == "uniform":
        return rng.uniform(1.0, 2.0, n)
    k = rng.integers(0, 64, n).astype(np.float64)
    if kind == "low":   # just above 1: 1 + k ulp
        return 1.0 + k * 2.0 ** -52
    return 2.0 - (k + 1) * 2.0 ** -52  # just below 2


@pytest.mark.parametrize("kinds", [("uniform", "uniform"), ("low", "uniform"), ("high", "uniform"),
                                   ("uniform", "low"), ("uniform", "high"), ("low", "low"), ("high", "high"),
                                   ("low", "high"), ("high", "low")])
def test_quotients_equal_ieee_division(cuda_lib, kinds):
    rng = np.random.default_rng([ord(c) for c in "".join(kinds)])
    n = 1 << 23
    sa, sb = _significands(rng, n, kinds[0]), _significands(rng, n, kinds[1])
    ea, eb = rng.integers(-420, 420, n), rng.integers(-420, 420, n)
    a = np.ldexp(sa, ea) * rng.choice([-1.0, 1.0], n)
    b = np.ldexp(sb, eb) * rng.choice([-1.0, 1.0], n)
    _assert_ieee(a, b, _quotients(cuda_lib, a, b))


def test_quotients_of_workload_like_operands(cuda_lib):
    """Quotients within a few ulp of a power of two (either side, where the
    spacing of doubles changes), mass fractions over densities, pressure
    differences over sound speeds, exact quotients (a = b t for small
    integers t) and powers of two."""
    rng = np.random.default_rng(7)
    n = 1 << 22
    b = rng.uniform(1e-5, 1e-2, n)
    t = rng.integers(1, 1 << 20, n).astype(np.float64) * np.ldexp(1.0, rng.integers(-30, 30, n))
    near = b * (1.0 + rng.integers(-3, 4, n) * 2.0 ** -52)  # quotients within a few ulp of 1, both sides
    cases = [(np.ldexp(near, rng.integers(-40, 40, n)), b),
             (rng.uniform(0, 1e-2, n) * rng.uniform(0, 1, n), b),
             (rng.normal(0, 1e3, n), rng.uniform(3e4, 1e5, n)),
             (b * t, b), (b, b), (np.ldexp(1.0, rng.integers(-300, 300, n)), b),
             (b, np.ldexp(1.0, rng.integers(-300, 300, n)))]
    for a, bb in cases:
        _assert_ieee(a, bb, _quotients(cuda_lib, a, bb))


def test_quotients_special_operands(cuda_lib):
    tiny, huge = 2.0 ** -1074, 1.7976931348623157e308
    vals = np.array([0.0, -0.0, 1.0, -1.0, 3.0, 0.1, tiny, -tiny, 2.0 ** -1022, 2.0 ** -401, 2.0 ** -400,
                     2.0 ** 400, 2.0 ** 401, 2.0 ** 1000, huge, np.inf, -np.inf, np.nan, 1.0 + 2.0 ** -52,
                     2.0 - 2.0 ** -52, 1e-300, 1e300])
    a, b = np.meshgrid(vals, vals)
    a, b = a.ravel().copy(), b.ravel().copy()
    _assert_ieee(a, b, _quotients(cuda_lib, a, b))
