"""The split-precision path's digit splitting, checked on the CPU.

The device routine (csrc/fast_device.cuh digits_of) cuts a double-float
v = hi + lo in [0, 1] into NS balanced base-128 digits with FP32 operations.
Here every one of those operations is replayed in exact rational arithmetic
with round-to-nearest-even to FP32, and the properties the tensor-core
contraction relies on are checked: integer digits, the first in [0, 128],
all within [-128, 128] (so digit products summed over a level stay exact in
FP32), and v - sum_s d_s 2^(-7(s+1)) within 2^(-7 NS - 1) + 2^-59.
"""
from fractions import Fraction

import numpy as np
import pytest

SHIFT = Fraction(3 * 2 ** 22)


def rn32(q: Fraction) -> Fraction:
    """q rounded to the nearest FP32 value (ties to even), as a Fraction."""
    if q == 0:
        return Fraction(0)
    sign = -1 if q < 0 else 1
    a = abs(q)
    e = a.numerator.bit_length() - a.denominator.bit_length()
    if Fraction(2) ** e > a:
        e -= 1
    e = max(e, -126)                      # subnormal spacing below 2^-126
    ulp = Fraction(2) ** (e - 23)
    m = a / ulp
    n = m.numerator // m.denominator
    rem = m - n
    if rem > Fraction(1, 2) or (rem == Fraction(1, 2) and n % 2 == 1):
        n += 1
    return sign * n * ulp


def digits(hi: Fraction, lo: Fraction, ns: int):
    """The device routine's operations, each rounded to FP32."""
    d = [Fraction(0)] * ns
    nh = min(ns, 5)
    x = hi
    for s in range(nh):
        d[s] = rn32(rn32(128 * x + SHIFT) - SHIFT)
        x = rn32(128 * x - d[s])
    w = rn32(lo * 2 ** 21)
    for s in range(3, nh):
        e = rn32(rn32(128 * w + SHIFT) - SHIFT)
        w = rn32(128 * w - e)
        d[s] = rn32(d[s] + e)
    r = rn32(x + w)
    for s in range(5, ns):
        d[s] = rn32(rn32(128 * r + SHIFT) - SHIFT)
        if s + 1 < ns:
            r = rn32(128 * r - d[s])
    return d


def ulp32(x: Fraction) -> Fraction:
    if x == 0:
        return Fraction(2) ** -149
    e = x.numerator.bit_length() - x.denominator.bit_length()
    if Fraction(2) ** e > x:
        e -= 1
    return Fraction(2) ** (max(e, -126) - 23)


def cases(seed=7, n=400):
    rng = np.random.default_rng(seed)
    out = [(Fraction(0), Fraction(0)), (Fraction(1), Fraction(0)),
           (1 - Fraction(2) ** -24, Fraction(2) ** -25),
           (1 - Fraction(2) ** -24, -Fraction(2) ** -25),
           (Fraction(1, 2), -Fraction(2) ** -26), (Fraction(1, 2), Fraction(2) ** -25),
           (Fraction(2) ** -30, Fraction(2) ** -54), (Fraction(2) ** -60, -Fraction(2) ** -84),
           (Fraction(127, 128), Fraction(0)), (Fraction(255, 256), Fraction(2) ** -33)]
    for _ in range(n):
        k = int(rng.integers(1, 64))
        hi = Fraction(int(rng.integers(2 ** 23, 2 ** 24)), 2 ** (23 + k))
        u = ulp32(hi)
        m = int(rng.integers(2 ** 23, 2 ** 24))
        lo = rn32(Fraction(m, 2 ** 24) * u / 2 * Fraction(int(rng.integers(1, 2 ** 10)), 2 ** 10))
        if rng.random() < 0.5:
            lo = -lo
        if rng.random() < 0.1:
            lo = Fraction(0)
        out.append((hi, lo))
    return out


@pytest.mark.parametrize("ns", [4, 5, 6, 7, 8])
def test_digits_bounds_and_error(ns):
    bound = Fraction(2) ** (-7 * ns - 1) + Fraction(2) ** -59
    if ns <= 5:
        bound = Fraction(2) ** (-7 * ns)
    for hi, lo in cases(seed=ns):
        d = digits(hi, lo, ns)
        assert all(x.denominator == 1 for x in d), (hi, lo, d)
        assert 0 <= d[0] <= 128
        assert all(-128 <= x <= 128 for x in d), (hi, lo, d)
        approx = sum(x * Fraction(2) ** (-7 * (s + 1)) for s, x in enumerate(d))
        assert abs(hi + lo - approx) <= bound, (hi, lo, float(hi + lo - approx))


def test_level_sums_stay_exact_in_fp32():
    # the worst level of an NS = 8 contraction over K = 64 (forward) and of an
    # NB = 7 one over K = 128 (dlnL/dP): every partial sum is an integer <= 2^24
    assert 8 * 64 * 128 * 128 <= 2 ** 23
    assert 7 * 128 * 128 * 128 <= 2 ** 24


def p_fixed_bits(v: float, ns: int) -> int:
    """The digit-plane kernel's floor(v 2^(7 ns)) from the bit fields of a double
    in [0, 1] (k_fast.cu p_fixed_bits), restated."""
    import struct
    u = struct.unpack("<Q", struct.pack("<d", v))[0]
    e = (u >> 52) & 0x7FF
    if (u >> 63) or e == 0:
        return 0
    m = (u & ((1 << 52) - 1)) | (1 << 52)
    sh = e - 1075 + 7 * ns
    if sh >= 0:
        return m << sh
    return 0 if sh <= -64 else m >> -sh


@pytest.mark.parametrize("ns", [5, 6, 7, 8])
def test_p_fixed_bits_equals_floor(ns):
    import math
    rng = np.random.default_rng(ns)
    vals = [0.0, 1.0, 0.5, 2.0 ** -56, 2.0 ** -57, 2.0 ** -1000, 5e-324, 1.0 - 2.0 ** -53, -0.0, -1e-300]
    vals += list(rng.random(2000)) + list(rng.random(500) * 2.0 ** -30) + list(2.0 ** -rng.integers(1, 70, 500))
    for v in vals:
        want = math.floor(v * 2.0 ** (7 * ns)) if v > 0 else 0
        assert p_fixed_bits(float(v), ns) == want, v
