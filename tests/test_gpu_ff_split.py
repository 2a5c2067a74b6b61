"""The double-float conversions of the mixed form (pc_ff.cuh): ff_of(double)
and f2d_exact, which take the integer pipe in their fast ranges, bit for bit
against CUDA's own conversions (__double2float_rn of x and of the remainder;
float -> double), over the whole exponent range, the ends of the fast
range, rounding ties and carries, zeros, subnormals, infinities and NaNs.
The test kernel (tests/csrc/ff_check.cu) is compiled with nvcc here."""
import ctypes
import os
import subprocess
import tempfile

import numpy as np
import pytest

torch = pytest.importorskip("torch")

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    out = os.path.join(tempfile.mkdtemp(prefix="ffcheck_"), "libffcheck.so")
    subprocess.run([_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-shared",
                    "-Xcompiler", "-fPIC", "-fmad=true", "-I", os.path.join(ROOT, "pelec_gb300", "csrc"),
                    "-o", out, os.path.join(HERE, "csrc", "ff_check.cu")], check=True)
    L = ctypes.CDLL(out)
    L.ff_check.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p, ctypes.c_void_p]
    L.ff_check.restype = ctypes.c_int
    return L


def _doubles(rng):
    """Bit patterns: random over all exponents and both signs; every exponent
    at the fast range's ends; ties and carries of the 29 dropped bits; zeros,
    subnormals, infinities, NaNs."""
    parts = [rng.integers(0, 2 ** 64, size=200000, dtype=np.uint64)]
    e = np.arange(0, 2048, dtype=np.uint64)
    for low in (np.uint64(0), np.uint64(1 << 28), np.uint64((1 << 28) + 1), np.uint64((1 << 28) - 1),
                np.uint64((1 << 29) - 1), np.uint64(1 << 29 | 1 << 28), np.uint64(0xFFFFFFFFFFFFF)):
        for sign in (np.uint64(0), np.uint64(1) << np.uint64(63)):
            parts.append(sign | (e << np.uint64(52)) | low)
    # mantissa all ones (a rounding carry into the exponent) at every exponent
    parts.append((e << np.uint64(52)) | np.uint64(0xFFFFFFFFFFFFF))
    # values of the state's magnitudes (densities, energies, species densities)
    v = np.concatenate([10.0 ** rng.uniform(-40, 40, 50000), -(10.0 ** rng.uniform(-40, 40, 50000))])
    parts.append(v.view(np.uint64))
    parts.append(np.array([0, 1 << 63, 1, 0x7FF0000000000000, 0xFFF0000000000000, 0x7FF8000000000000],
                          dtype=np.uint64))
    return np.concatenate(parts)


def _floats(rng):
    parts = [rng.integers(0, 2 ** 32, size=200000, dtype=np.uint64).astype(np.uint32)]
    e = np.arange(0, 256, dtype=np.uint32)
    for low in (0, 1, 0x400000, 0x7FFFFF):
        for sign in (0, 1 << 31):
            parts.append(np.uint32(sign) | (e << np.uint32(23)) | np.uint32(low))
    parts.append(np.array([0, 1 << 31, 1, 0x7F800000, 0xFF800000, 0x7FC00000], dtype=np.uint32))
    return np.concatenate(parts)


@pytest.mark.gpu
def test_ff_of_and_f2d_bit_for_bit(lib):
    rng = np.random.default_rng(7)
    xb = _doubles(rng)
    fb = _floats(rng)
    n = max(len(xb), len(fb))
    xb = np.resize(xb, n)
    fb = np.resize(fb, n)
    x = torch.from_numpy(xb.view(np.float64).copy()).cuda()
    f = torch.from_numpy(fb.view(np.float32).copy()).cuda()
    split = torch.empty(4 * n, dtype=torch.float32, device="cuda")
    widen = torch.empty(2 * n, dtype=torch.float64, device="cuda")
    rc = lib.ff_check(x.data_ptr(), f.data_ptr(), n, split.data_ptr(), widen.data_ptr())
    assert rc == 0, rc
    s = split.cpu().numpy().view(np.uint32).reshape(n, 4)
    w = widen.cpu().numpy().view(np.uint64).reshape(n, 2)
    xs = xb.view(np.float64)
    fs = fb.view(np.float32)
    nan_x = np.isnan(xs)
    bad_hi = (s[:, 0] != s[:, 2]) & ~nan_x
    bad_lo = (s[:, 1] != s[:, 3]) & ~nan_x
    assert not bad_hi.any(), [hex(v) for v in xb[bad_hi][:5]]
    assert not bad_lo.any(), [hex(v) for v in xb[bad_lo][:5]]
    # a NaN stays a NaN
    hi = s[:, 0].view(np.float32)
    assert np.isnan(hi[nan_x]).all()
    nan_f = np.isnan(fs)
    bad_w = (w[:, 0] != w[:, 1]) & ~nan_f
    assert not bad_w.any(), [hex(v) for v in fb[bad_w][:5]]
    assert np.isnan(w[nan_f, 0].view(np.float64)).all()
    # the fast ranges were exercised: most of the state-magnitude sample takes them
    e11 = (xb >> np.uint64(52)) & np.uint64(0x7FF)
    assert ((e11 >= 951) & (e11 <= 1138)).sum() > 50000
