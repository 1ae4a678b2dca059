"""The mixed path's float/double conversions by integer operations (d2f_bits,
f2d_bits in csrc/lg_device.cuh), restated step for step in Python integers and
checked against IEEE conversions (numpy): double -> float rounds to nearest,
ties to even, overflows to infinity, and gives a signed zero below the float
normal range (where IEEE would give a float subnormal); float -> double is
exact for normal floats and gives a signed zero for float subnormals.  The
GPU parity tests of the mixed path cover the device code itself."""
import struct

import numpy as np


def d2f_bits(x):
    hi = (struct.unpack("<Q", struct.pack("<d", x))[0] >> 32) & 0xFFFFFFFF
    lo = struct.unpack("<Q", struct.pack("<d", x))[0] & 0xFFFFFFFF
    sign = hi & 0x80000000
    e = ((hi >> 20) & 0x7FF) - 1023 + 127
    if e <= 0:
        return struct.unpack("<f", struct.pack("<I", sign))[0]
    if e >= 255:
        return struct.unpack("<f", struct.pack("<I", sign | 0x7F800000))[0]
    m = ((hi & 0xFFFFF) << 3) | (lo >> 29)
    rest = lo & 0x1FFFFFFF
    bits = (e << 23) | m
    bits += 1 if (rest > 0x10000000 or (rest == 0x10000000 and (m & 1))) else 0
    return struct.unpack("<f", struct.pack("<I", sign | bits))[0]


def f2d_bits(f):
    u = struct.unpack("<I", struct.pack("<f", f))[0]
    sign = u & 0x80000000
    ef = (u >> 23) & 0xFF
    if ef == 0:
        return struct.unpack("<d", struct.pack("<Q", sign << 32))[0]
    hi = sign | ((ef + (1023 - 127)) << 20) | ((u & 0x7FFFFF) >> 3)
    lo = (u & 7) << 29
    return struct.unpack("<d", struct.pack("<Q", (hi << 32) | lo))[0]


def _same(a, b):
    return struct.pack("<f", a) == struct.pack("<f", b)


def test_double_to_float_rounds_to_nearest_even_in_the_normal_range():
    rng = np.random.default_rng(5)
    xs = rng.standard_normal(20000) * 2.0 ** rng.integers(-120, 120, 20000)
    # ties: doubles exactly halfway between two floats, both parities
    base = rng.standard_normal(2000).astype(np.float32).astype(np.float64)
    ties = base + np.spacing(base.astype(np.float32)).astype(np.float64) / 2
    for x in np.concatenate([xs, ties, -ties]):
        ref = np.float32(x)
        if not np.isfinite(ref) or abs(ref) < np.finfo(np.float32).tiny:
            continue
        assert _same(d2f_bits(float(x)), float(ref)), x


def test_double_to_float_edges():
    big = float(np.finfo(np.float32).max)
    assert d2f_bits(big) == big
    assert d2f_bits(2.0 ** 128) == float("inf") and d2f_bits(-(2.0 ** 128)) == float("-inf")
    # just below the halfway point to 2^128: down to the largest float; above
    # it: the rounding carries into the exponent, infinity
    assert d2f_bits(big * (1 + 2.0 ** -25)) == big
    assert d2f_bits(big * (1 + 2.0 ** -24)) == float("inf")
    tiny = float(np.finfo(np.float32).tiny)
    assert d2f_bits(tiny) == tiny
    for sub in (tiny / 2, 1e-45, -1e-40):  # float subnormal range: signed zero
        z = d2f_bits(sub)
        assert z == 0.0 and np.signbit(z) == np.signbit(sub)
    assert d2f_bits(0.0) == 0.0 and np.signbit(d2f_bits(-0.0))


def test_float_to_double_is_exact_for_normal_floats():
    rng = np.random.default_rng(6)
    fs = (rng.standard_normal(20000) * 2.0 ** rng.integers(-125, 127, 20000)).astype(np.float32)
    for f in fs:
        if abs(f) < np.finfo(np.float32).tiny or not np.isfinite(f):
            continue
        assert f2d_bits(float(f)) == float(np.float64(f))
    sub = float(np.float32(1e-40))
    assert f2d_bits(sub) == 0.0 and f2d_bits(-sub) == 0.0 and np.signbit(f2d_bits(-sub))
