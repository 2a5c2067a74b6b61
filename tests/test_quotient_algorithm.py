"""CPU test of the arithmetic of the FP64 kernels' exact shared-divisor
quotient (div_fast in pelec_gb300/csrc/pc_device.cuh), restated step by step
in Python integers: y = 1/b and q0 = a y both rounded toward zero (exact
rational arithmetic here), the remainder R = A 2^k - B M of the 53-bit
significands modulo 2^64, the step s in [0, 4] counted from 2R against odd
multiples of B, and the stop at a power of two just above q0.  Every result
the fast path gives must equal IEEE division; the GPU test
(test_gpu_quotients.py) checks the compiled code the same way.
"""
import math
import struct
from fractions import Fraction

import numpy as np

M64 = (1 << 64) - 1
M32 = (1 << 32) - 1


def _bits(x: float) -> int:
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def _float(b: int) -> float:
    return struct.unpack("<d", struct.pack("<Q", b & M64))[0]


DBL_MAX = 1.7976931348623157e308


def _rz(fr: Fraction) -> float:
    if abs(fr) > DBL_MAX:  # rounding toward zero never overflows
        return DBL_MAX if fr > 0 else -DBL_MAX
    r = float(fr)  # correctly rounded to nearest
    if abs(Fraction(r)) > abs(fr):
        r = math.nextafter(r, 0.0)
    return r


def div_fast(a: float, b: float):
    """(quotient, slow) as the kernel computes them (finite a, nonzero finite b)."""
    y = _rz(Fraction(1) / Fraction(b))
    q0 = _rz(Fraction(a) * Fraction(y)) if a != 0.0 else math.copysign(0.0, a) * math.copysign(1.0, y)
    ia, ib, iq = _bits(a), _bits(b), _bits(q0)
    ah, al, bh, bl, qh, ql = ia >> 32, ia & M32, ib >> 32, ib & M32, iq >> 32, iq & M32
    ea, eb, eq = (ah >> 20) & 0x7FF, (bh >> 20) & 0x7FF, (qh >> 20) & 0x7FF
    sh = (ea - eb - eq + 1043) & 31
    Bh, Mh = (bh & 0xFFFFF) | 0x100000, (qh & 0xFFFFF) | 0x100000
    p = bl * ql
    phi = ((p >> 32) + bl * Mh + Bh * ql) & M32
    R = ((((al << sh) & M32) << 32) - ((phi << 32) | (p & M32))) & M64
    R = R - (1 << 64) if R >= 1 << 63 else R
    B = (Bh << 32) | bl
    st = sum(int(2 * R > m * B) for m in (1, 3, 5, 7))
    d = 0xFFFFFFFF - ql + 1
    if (qh & 0xFFFFF) == 0xFFFFF and ql >= 0xFFFFFFFC and st > d:
        st = d + int(R >= (d + 1) * B)
    zero = ((ah << 1) & M32 | al) == 0
    if zero:
        return q0, eb == 0
    slow = not (1 <= ea <= 2046) or not (1 <= eb <= 2044) or not (2 <= eq <= 2045) or R < 0
    return _float(iq + st), slow


def _check(pairs):
    slow_count = 0
    for a, b in pairs:
        for sa in (1.0, -1.0):
            q, slow = div_fast(sa * a, b)
            slow_count += slow
            if not slow:
                assert _bits(q) == _bits((sa * a) / b), (float.hex(sa * a), float.hex(b), float.hex(q))
    return slow_count


def test_random_operands():
    rng = np.random.default_rng(21)
    pairs = [(float(rng.uniform(1, 2) * 2.0 ** int(rng.integers(-200, 200))),
              float(rng.uniform(1, 2) * 2.0 ** int(rng.integers(-200, 200)))) for _ in range(20000)]
    assert _check(pairs) == 0


def test_quotients_next_to_powers_of_two():
    """a = b 2^k (1 + j 2^-52), |j| <= 6: quotients a few ulp either side of
    a power of two, where the spacing of doubles changes."""
    rng = np.random.default_rng(22)
    pairs = []
    for _ in range(20000):
        b = float(rng.uniform(1, 2) * 2.0 ** int(rng.integers(-30, 30)))
        j = int(rng.integers(-6, 7))
        a = float(Fraction(b) * (1 + Fraction(j, 2 ** 52)) * Fraction(2) ** int(rng.integers(-5, 5)))
        pairs.append((a, b))
    assert _check(pairs) == 0


def test_significands_near_binade_ends():
    rng = np.random.default_rng(23)

    def sig():
        k = int(rng.integers(0, 64))
        return 1 + k * 2.0 ** -52 if rng.random() < 0.5 else 2 - (k + 1) * 2.0 ** -52

    pairs = [(sig() * 2.0 ** int(rng.integers(-4, 4)), sig()) for _ in range(20000)]
    assert _check(pairs) == 0


def test_special_operands_take_the_slow_path():
    """Subnormal numerators or divisors, a divisor whose reciprocal is not
    normal, and quotients outside the normal range go to IEEE division."""
    tiny = 2.0 ** -1074
    for a, b in [(0.0, tiny), (tiny, 1.0), (1.0, tiny), (1.0, 2.0 ** 1023), (2.0 ** -1000, 2.0 ** 100),
                 (2.0 ** 1000, 2.0 ** -100)]:
        q, slow = div_fast(a, b)
        assert slow, (a, b)
    q, slow = div_fast(0.0, 3.0)
    assert not slow and q == 0.0 and math.copysign(1.0, q) == 1.0
    q, slow = div_fast(-0.0, 3.0)
    assert not slow and q == 0.0 and math.copysign(1.0, q) == -1.0
