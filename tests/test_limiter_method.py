"""The device's MUSCL limiter arithmetic (k_scalar_pass with MUSCL) restated on the CPU and
compared with the reference's definitions on special values: minmod (transport.rs:510-516)
is 0 where the FP64 product a b is <= 0 (an underflow to zero included), else
f64::signum(a) * f64::min(|a|, |b|); the device keeps the product and the test, and takes
the minimum as the smaller magnitude bit pattern with a's sign bit (a NaN a passes
through). The products by 0.5 and 2 of the monotonized-central slope (transport.rs:517-526)
are exponent shifts on the device, exact while operand and result are normal; the FP64
product otherwise, so only the shift is restated here."""
import itertools

import numpy as np

SPECIAL = np.array([0.0, -0.0, 5e-324, -5e-324, 1e-310, -3e-310, 2.2250738585072014e-308, 1e-200, -1e-200,
                    1e-160, 3e-155, 0.5, -1.0, 1.0, 2.0, -7.25, 1e150, 1e300, -1.7e308, np.inf, -np.inf, np.nan],
                   dtype=np.float64)
MAG = np.uint64(0x7FFFFFFFFFFFFFFF)
SIGN = np.uint64(0x8000000000000000)


def u64(x):
    return np.array([x], dtype=np.float64).view(np.uint64)[0]


def f64(b):
    return np.array([b], dtype=np.uint64).view(np.float64)[0]


def minmod_reference(a, b):
    """transport.rs:510-516 with Rust's f64 semantics (signum of NaN is NaN; min returns
    the other operand of a NaN)."""
    with np.errstate(all="ignore"):
        if np.float64(a) * np.float64(b) <= 0.0:
            return 0.0
        signum = a if np.isnan(a) else (-1.0 if np.signbit(a) else 1.0)
        m = abs(b) if np.isnan(a) else (abs(a) if np.isnan(b) else min(abs(a), abs(b)))
        return np.float64(signum) * np.float64(m)


def minmod_device(a, b):
    """The device's form (minmod_bits): the FP64 product test, then the minimum of the
    magnitude bit patterns with a's sign bit."""
    with np.errstate(all="ignore"):
        if np.float64(a) * np.float64(b) <= 0.0:
            return 0.0
    if np.isnan(a):
        return a
    ma, mb = u64(a) & MAG, u64(b) & MAG
    return f64(min(ma, mb) | (u64(a) & SIGN))


def same(x, y):
    return (np.isnan(x) and np.isnan(y)) or u64(x) == u64(y)


def test_minmod_bits_equal_reference_on_special_values():
    for a, b in itertools.product(SPECIAL, SPECIAL):
        assert same(minmod_device(a, b), minmod_reference(a, b)), (a, b)


def test_minmod_bits_equal_reference_on_random_values():
    rng = np.random.default_rng(4)
    mant = rng.uniform(-1.0, 1.0, (20000, 2))
    expo = rng.integers(-1074, 1023, (20000, 2)).astype(np.float64)
    vals = np.ldexp(mant, expo.astype(np.int64))
    for a, b in vals:
        assert same(minmod_device(a, b), minmod_reference(a, b)), (a, b)


def mul_pow2_shift(x, e):
    """The exponent shift of mul_pow2: x * 2^e by moving the exponent field when x and the
    result are normal, else the FP64 product."""
    b = int(u64(x))
    ex = (b >> 52) & 0x7FF
    r = ex + e
    if ex != 0 and ex != 0x7FF and 1 <= r <= 2046:
        return f64(np.uint64((b + (e << 52)) & 0xFFFFFFFFFFFFFFFF))
    if b & 0x7FFFFFFFFFFFFFFF == 0:
        return x
    with np.errstate(all="ignore"):
        return np.float64(x) * np.float64(2.0 ** e)


def test_half_and_twice_equal_fp64_products():
    rng = np.random.default_rng(9)
    vals = list(SPECIAL) + list(np.ldexp(rng.uniform(-1.0, 1.0, 20000), rng.integers(-1074, 1024, 20000)))
    with np.errstate(all="ignore"):
        for x in vals:
            assert same(mul_pow2_shift(x, -1), np.float64(0.5) * np.float64(x)), x
            assert same(mul_pow2_shift(x, 1), np.float64(2.0) * np.float64(x)), x


def prod_le_zero_device(a, b):
    """The device's `a * b <= 0.0` (prod_le_zero) on the bits: NaN operands and 0 * inf give
    NaN (false); a zero operand gives a zero product (true); different signs a negative
    product (true); an infinite operand of the same sign +inf (false). Same-sign finite
    nonzero operands |a| = ma 2^qa, |b| = mb 2^qb (ma, mb in [1, 2)): the product is at
    least 2^-1074, the smallest subnormal, when qa + qb >= -1074 (false) and below 2^-1075,
    half of it, so rounding to zero, when qa + qb <= -1077 (true); in between the FP64
    product decides."""
    ua, ub = int(u64(a)), int(u64(b))
    ma, mb = ua & 0x7FFFFFFFFFFFFFFF, ub & 0x7FFFFFFFFFFFFFFF
    inf = 0x7FF0000000000000
    if ma > inf or mb > inf:
        return False
    if ma == 0 or mb == 0:
        return not (ma == inf or mb == inf)
    if (ua ^ ub) >> 63:
        return True
    if ma == inf or mb == inf:
        return False

    def q(m):
        e = m >> 52
        return e - 1023 if e else -1074 + (m.bit_length() - 1)

    s = q(ma) + q(mb)
    if s >= -1074:
        return False
    if s <= -1077:
        return True
    with np.errstate(all="ignore"):
        return bool(np.float64(a) * np.float64(b) <= 0.0)


def test_product_sign_test_on_bits_equals_fp64():
    rng = np.random.default_rng(12)
    edge = [np.ldexp(1.0, e) for e in range(-1076, -1070)] + [np.ldexp(1.5, e) for e in range(-540, -530)]
    vals = list(SPECIAL) + edge + [np.nextafter(np.ldexp(1.0, -537), 1.0), np.ldexp(1.0, -537), 2.0 ** -538]
    vals += list(np.ldexp(rng.uniform(-2.0, 2.0, 3000), rng.integers(-1074, 1024, 3000)))
    vals += list(np.ldexp(rng.uniform(0.5, 2.0, 3000), rng.integers(-545, -530, 3000)))
    vals = np.array(vals, dtype=np.float64)
    with np.errstate(all="ignore"):
        for a in vals[rng.permutation(vals.size)[:400]]:
            want = (np.float64(a) * vals) <= 0.0
            got = np.array([prod_le_zero_device(a, b) for b in vals])
            bad = np.nonzero(want != got)[0]
            assert bad.size == 0, (a, vals[bad[:3]])
        for a, b in itertools.product(SPECIAL, SPECIAL):
            assert prod_le_zero_device(a, b) == bool(np.float64(a) * np.float64(b) <= 0.0), (a, b)
