"""The division the mixed form's right-hand side uses, restated on the CPU: x / y from a
precomputed ry = RN(1/y) by Markstein's correction step (q = RN(x ry), rem = RN(x - q y)
exact under an FMA, RN(q + rem ry)). The FMA is emulated exactly with rationals (the
product and sum are exact Fractions, `float()` rounds them correctly), so this pins the
method itself, independently of the device: it must equal the correctly rounded quotient
on the numerator families the device check uses (random significands over the exponent
range the kernel takes the step on, quotients next to a double, quotients next to a
midpoint between two doubles) for the same divisors."""
import random
import struct
from fractions import Fraction

import pytest


def fma(a, b, c):
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def div_rdt(x, y, ry):
    q = x * ry
    rem = fma(-q, y, x)
    return fma(rem, ry, q)


def bits(v):
    return struct.unpack("<Q", struct.pack("<d", v))[0]


def from_bits(b):
    return struct.unpack("<d", struct.pack("<Q", b))[0]


DIVISORS = [0.1, 0.05, 0.3, 1.0 / 3.0, 0.7, 0.037, 1.0 - 2.0 ** -53, 1.0 + 2.0 ** -52, 2.0 - 2.0 ** -51, 0.25,
            2.0 ** -60, 2.0 ** 60, 12345.678, 9.87e-15]


@pytest.mark.parametrize("y", DIVISORS)
def test_markstein_step_is_correctly_rounded(y):
    rng = random.Random(hash(y) & 0xffff)
    ry = 1.0 / y
    for mode in range(3):
        for _ in range(1500):
            mant = rng.getrandbits(52)
            sign = rng.getrandbits(1) << 63
            if mode == 0:
                e = 123 + rng.randrange(1801)  # the exponents the kernel takes the step on
                x = from_bits(sign | (e << 52) | mant)
            else:
                m = from_bits(sign | (1023 << 52) | mant)
                x = y * m if mode == 1 else fma(y, m, y * (m * 2.0 ** -53))
            assert bits(div_rdt(x, y, ry)) == bits(x / y), (y, mode, x)
