"""The exactness argument of the mixed-precision traversal (pn_traverse.cuh: two_sum,
diff_f32), restated with numpy Float32 arithmetic (IEEE round to nearest, no contraction)
and checked on the CPU: whenever the Float32-only difference of the hi/lo split decides,
it equals the reference's Float32(Float64(x - y)), including for pairs placed within 1e-9
of a Float32 rounding boundary, at powers of two and for tiny differences; the cases it
cannot decide are left to Float64 (and are rare for ordinary pairs)."""
import struct

import numpy as np

f32 = np.float32


def two_sum(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    return s, f32(f32(a - f32(s - bb)) + f32(b - bb))


def _bits(x):
    return struct.unpack("<i", struct.pack("<f", x))[0]


def _from_bits(i):
    return f32(struct.unpack("<f", struct.pack("<i", i))[0])


def diff_f32(xh, xl, yh, yl, eb):
    s, t = two_sum(xh, f32(-yh))
    p, q = two_sum(xl, f32(-yl))
    w = f32(f32(t + p) + q)
    zh, zl = two_sum(s, w)
    az = abs(zh)
    if not az >= f32(1e-30):
        return None
    bits = _bits(az)
    half_ulp = _from_bits((bits & 0x7F800000) - (24 << 23))
    if bits & 0x007FFFFF == 0:
        half_ulp = f32(half_ulp * f32(0.5))
    if not f32(half_ulp - abs(zl)) > f32(eb + f32(az * f32(2.3e-16))):
        return None
    return zh


def split(x):
    h = f32(x)
    return h, f32(x - float(h))


def check(pairs, ext):
    eb = f32(2.0 ** -44 * (ext + 3.0))
    decided = 0
    for x, y in pairs:
        got = diff_f32(*split(x), *split(y), eb)
        if got is not None:
            decided += 1
            assert got == f32(x - y), (x, y)
    return decided


def test_ordinary_pairs_decide_and_are_exact():
    rng = np.random.default_rng(5)
    ext = 200.0
    x = rng.uniform(-ext, ext, 20000)
    y = x + rng.uniform(-6.0, 6.0, x.size)
    decided = check(zip(x.tolist(), y.tolist()), ext)
    assert decided >= 0.995 * x.size  # Float64 is needed for a tiny fraction only


def test_pairs_at_rounding_boundaries_are_never_wrong():
    rng = np.random.default_rng(6)
    ext = 200.0
    pairs = []
    for _ in range(20000):
        x = float(rng.uniform(-ext, ext))
        d = f32(rng.uniform(-6.0, 6.0))
        half = float(np.spacing(abs(d))) / 2
        y = x - (float(d) + half * rng.choice([-1.0, 1.0]) * (1 + rng.uniform(-1e-9, 1e-9)))
        pairs.append((x, y))
    for k in range(-20, 4):  # differences at powers of two and just around them
        p2 = 2.0 ** k
        for sgn in (1.0, -1.0):
            for e in (0.0, 1e-12, -1e-12):
                pairs.append((50.0, 50.0 - sgn * p2 * (1 + e)))
    check(pairs, ext)


def test_tiny_and_zero_differences_fall_back():
    eb = f32(2.0 ** -44 * 203.0)
    assert diff_f32(*split(7.25), *split(7.25), eb) is None  # zero: the caller's self pair
    x = 123.456789
    got = diff_f32(*split(x), *split(x + 1e-13), eb)
    assert got is None or got == f32(x - (x + 1e-13))
