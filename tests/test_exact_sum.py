"""The tridiagonalisation's exact warp and group sums (sum_exact in
csrc/lg_eig2.cu), restated step for step in Python integers: each value is
aligned at the largest exponent of its lane group into a 128-bit fixed-point
number (bits below 2^-64 of that exponent's unit truncated), the numbers are
added exactly, and the total is rounded once to nearest-even.  Checked here
against exact rational sums: the sum is correctly rounded when the exponents
span at most 64 binades (nothing is truncated); otherwise its error is below
n units of 2^-116 of the largest term's binade plus one ulp of the result
(an FP64 addition tree's bound is about log2(n) 2^-53 of the largest term).
The GPU parity tests cover the device code itself."""
import math
import random
import struct
from fractions import Fraction

import pytest


def _bits(v):
    return struct.unpack("<Q", struct.pack("<d", v))[0]


def _float(b):
    return struct.unpack("<d", struct.pack("<Q", b))[0]


def sum_exact(vals):
    """One group's sum, as the device computes it."""
    bs = [_bits(v) for v in vals]
    es = [(b >> 52) & 0x7FF for b in bs]
    emax = max(es)
    total = 0
    for b, e in zip(bs, es):
        if e == 0:  # zero (subnormals count as zero)
            continue
        m = (b & ((1 << 52) - 1)) | (1 << 52)
        sh = emax - e
        x = (m << 64) >> sh if sh < 128 else 0  # hi:lo, truncated magnitude
        total += -x if b >> 63 else x
    if total == 0:
        return 0.0
    neg, mag = total < 0, abs(total)
    p = mag.bit_length() - 1
    drop = p - 52
    if drop <= 0:
        mant = mag << -drop
    else:
        mant = mag >> drop
        half = (mag >> (drop - 1)) & 1
        sticky = (mag & ((1 << (drop - 1)) - 1)) != 0
        mant += 1 if half and (sticky or (mant & 1)) else 0
    r = _float(((p + emax - 116 - 1) << 52) + mant)
    return -r if neg else r


def _ulp(x):
    x = abs(x)
    if x == 0.0:
        return 2.0 ** -1074
    _, e = math.frexp(x)
    return 2.0 ** (e - 53)


def _cases(rng, n_cases):
    for _ in range(n_cases):
        n = rng.choice([1, 2, 3, 4, 8, 16, 31, 32])
        spread = rng.choice([0, 4, 30, 60, 120])
        base = rng.randint(-200, 200)
        vals = [rng.choice([-1.0, 1.0]) * rng.random() * 2.0 ** (base + rng.randint(0, spread))
                for _ in range(n)]
        if rng.random() < 0.2 and n > 1:  # cancellation
            vals[-1] = -sum(vals[:-1])
        if rng.random() < 0.1:
            vals[rng.randrange(n)] = 0.0
        yield vals


@pytest.mark.parametrize("seed", [1, 2])
def test_sum_error_is_within_the_truncation_bound(seed):
    rng = random.Random(seed)
    for vals in _cases(rng, 4000):
        exact = sum(Fraction(v) for v in vals)
        r = sum_exact(vals)
        emax = max((_bits(v) >> 52) & 0x7FF for v in vals)
        unit = Fraction(2) ** (emax - 1139) if emax else Fraction(0)
        err = abs(Fraction(r) - exact)
        assert err <= len(vals) * unit + Fraction(_ulp(r)), (vals, r, float(exact))
        # never worse than a left-to-right FP64 sum's error bound
        assert err <= len(vals) * Fraction(2) ** -53 * sum(abs(Fraction(v)) for v in vals) + \
            Fraction(_ulp(r))


def test_sum_is_correctly_rounded_without_truncation():
    """With exponents within 64 of each other nothing is truncated, and the
    single rounding gives the correctly rounded sum (Python's float of the
    exact rational sum)."""
    rng = random.Random(7)
    for _ in range(4000):
        n = rng.randint(1, 32)
        base = rng.randint(-100, 100)
        vals = [rng.choice([-1.0, 1.0]) * (1.0 + rng.random()) * 2.0 ** (base + rng.randint(0, 10))
                for _ in range(n)]
        assert sum_exact(vals) == float(sum(Fraction(v) for v in vals))


def test_group_sums_are_independent_sums_of_each_group():
    """The grouped form gives every aligned group of f lanes the sum of its
    own values (the maximum exponent is taken within the group)."""
    rng = random.Random(3)
    lanes = [rng.choice([-1.0, 1.0]) * rng.random() * 2.0 ** rng.randint(-60, 60) for _ in range(32)]
    for f in (1, 2, 4, 8, 16, 32):
        for g0 in range(0, 32, f):
            grp = lanes[g0:g0 + f]
            exact = sum(Fraction(v) for v in grp)
            assert abs(Fraction(sum_exact(grp)) - exact) <= Fraction(_ulp(float(exact)))
