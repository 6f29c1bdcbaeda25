"""The host FP32 fma emulation used by the FP32 kernel tests: equal to the
correctly rounded value of the exact a*b + c on random operands and on
products that land on an FP32 midpoint with a tiny addend (where rounding
through FP64 first would round the wrong way)."""
from fractions import Fraction

import numpy as np

from fp32_emul import fma32


def _exact(a, b, c):
    """correct FP32 rounding (ties to even) of the exact a*b + c"""
    ex = Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c))
    lo = np.float32(float(ex))                 # within one FP32 step of ex
    while Fraction(float(lo)) > ex:
        lo = np.nextafter(lo, np.float32(-np.inf))
    while Fraction(float(np.nextafter(lo, np.float32(np.inf)))) <= ex:
        lo = np.nextafter(lo, np.float32(np.inf))
    hi = np.nextafter(lo, np.float32(np.inf))
    if Fraction(float(lo)) == ex:
        return lo
    m = (Fraction(float(lo)) + Fraction(float(hi))) / 2
    if ex < m:
        return lo
    if ex > m:
        return hi
    return lo if (np.array([lo]).view(np.int32)[0] & 1) == 0 else hi


def test_fma32_random():
    rng = np.random.default_rng(3)
    a, b, c = [(rng.normal(size=1000) * 10.0 ** rng.integers(-6, 6, 1000)).astype(np.float32) for _ in range(3)]
    got = fma32(a, b, c)
    want = np.array([_exact(x, y, z) for x, y, z in zip(a, b, c)], np.float32)
    assert np.array_equal(got.view(np.int32), want.view(np.int32))


def test_fma32_midpoint_products():
    # (1 + 2^-12)^2 = 1 + 2^-11 + 2^-24 lies halfway between two FP32 numbers;
    # a tiny addend decides the rounding, which FP64 alone would lose
    a = np.float32(1 + 2.0 ** -12)
    for c in (2.0 ** -80, -(2.0 ** -80), 0.0, 2.0 ** -60):
        c32 = np.float32(c)
        got = fma32(a, a, c32)
        assert got.view(np.int32) == np.array([_exact(a, a, c32)], np.float32).view(np.int32)[0]
    assert fma32(a, a, np.float32(2.0 ** -80)) == np.float32(1 + 2.0 ** -11 + 2.0 ** -23)
    assert fma32(a, a, np.float32(-(2.0 ** -80))) == np.float32(1 + 2.0 ** -11)
