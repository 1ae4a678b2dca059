"""The mixed path's float/double conversions by integer operations (d2f_bits,
f2d_bits in csrc/lg_device.cuh), restated step for step in Python integers and
checked against IEEE conversions (numpy): double -> float rounds to nearest,
ties to even, overflows to infinity, and gives a signed zero below the float
normal range (where IEEE would give a float subnormal); float -> double is
exact for normal floats and gives a signed zero for float subnormals.  The
exact doubling of the QL rotations (twice_bits in csrc/lg_eig2.cu) equals IEEE
2 x for every double, subnormals, the largest binade, zero, infinity and NaN
included, and the selection prefilter's argument reduction keeps its cosine
within 3e-7.  The GPU parity tests cover the device code itself."""
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


def twice_bits(x):
    u = struct.unpack("<Q", struct.pack("<d", x))[0]
    sign = u & 0x8000000000000000
    mag = u ^ sign
    e = mag >> 52
    if e == 0:
        mag <<= 1
    elif e < 2046:
        mag += 1 << 52
    elif e == 2046:
        mag = 0x7FF0000000000000
    return struct.unpack("<d", struct.pack("<Q", sign | mag))[0]


def test_doubling_on_the_bit_pattern_equals_ieee_doubling():
    rng = np.random.default_rng(7)
    xs = rng.standard_normal(20000) * 2.0 ** rng.integers(-1074, 1024, 20000).astype(float)
    sub = np.array([5e-324, -5e-324, 2.0 ** -1023, 2.0 ** -1022 - 5e-324, -(2.0 ** -1030) * 3])
    big = np.finfo(np.float64).max
    edges = np.array([0.0, -0.0, big, -big, big / 2, 2.0 ** 1023, np.inf, -np.inf, 1.0, -3.5])
    with np.errstate(over="ignore"):
        for x in np.concatenate([xs, sub, edges]):
            got = twice_bits(float(x))
            ref = float(np.float64(x) * 2.0)
            assert struct.pack("<d", got) == struct.pack("<d", ref), x
    assert np.isnan(twice_bits(float("nan")))


def test_prefilter_argument_reduction_error():
    """The selection prefilter's cosine (cos_prefilter in csrc/lg_search.cu)
    reduces a longitude difference x in (-3 pi, 3 pi) to [-pi, pi] by the
    nearest multiple of the FP32 2 pi, in FP32 without contraction (the file is
    built with -fmad=false): restated in numpy float32, the cosine of the
    reduced argument is within 3e-7 of the cosine of x, and the argument lies
    in [-pi, pi] up to rounding, where the hardware cosine's documented error
    bound holds; both stay far inside the 1e-5 band that goes to the exact
    FP64 test."""
    k2pi = np.float32(6.28318530717958648)
    inv = np.float32(1.0) / k2pi
    rng = np.random.default_rng(11)
    x = rng.uniform(-3 * np.pi, 3 * np.pi, 200000).astype(np.float32)
    x = np.concatenate([x, np.float32([0.0, np.pi, -np.pi, 2 * np.pi, -2 * np.pi, 3 * np.pi - 1e-3])])
    n = np.rint(x * inv).astype(np.float32)
    r = (x - (k2pi * n).astype(np.float32)).astype(np.float32)
    exact = np.remainder(x.astype(np.float64) + np.pi, 2 * np.pi) - np.pi
    err = np.abs(np.cos(r.astype(np.float64)) - np.cos(exact))
    assert err.max() < 3e-7, err.max()
    assert np.all(np.abs(r) <= np.float32(np.pi) * (1 + 1e-6))
