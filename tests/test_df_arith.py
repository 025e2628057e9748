"""The double-float arithmetic of the Float64 WCSPH sweeps (csrc/pn_df.cuh), restated in
numpy Float32 and checked on the CPU against exact rational arithmetic.

numpy's float32 operations are IEEE round-to-nearest, like the device's explicitly rounded
__fadd_rn / __fsub_rn / __fmul_rn; the device's two_prod uses a fused multiply-add, which
is restated here as Dekker's exact product (the same p + e = a b).  Checked:
* the three-part split of k_to_pos32 is exact: x = xa + xb + xc for coordinates up to 1e9;
* df_diff3 gives the exact difference of two Float64 values to 2^-46 of it;
* d^2 formed from those differences is within 1e-13 of the exact d^2 -- far inside the
  1e-12 band outside which the double-float d^2 decides the neighbour test, so that the
  decision always equals the Float64 one;
* df_mul / df_add / df_add_pos (non-negative operands) / df_sqr keep 2^-44 relative
  accuracy on WCSPH-sized operands.
"""
from fractions import Fraction

import numpy as np

f32 = np.float32


def two_sum(a, b):
    s = f32(a + b)
    bb = f32(s - a)
    e = f32(f32(a - f32(s - bb)) + f32(b - bb))
    return s, e


def fast_two_sum(a, b):
    s = f32(a + b)
    return s, f32(b - f32(s - a))


def _split(a):  # Veltkamp split of a Float32 into two 12-bit halves
    c = f32(f32(4097.0) * a)
    hi = f32(c - f32(c - a))
    return hi, f32(a - hi)


def two_prod(a, b):
    p = f32(a * b)
    ah, al = _split(a)
    bh, bl = _split(b)
    e = f32(f32(f32(f32(ah * bh) - p) + f32(ah * bl)) + f32(al * bh))
    e = f32(e + f32(al * bl))
    return p, e


def df_add(a, b):
    s, se = two_sum(a[0], b[0])
    t, te = two_sum(a[1], b[1])
    se = f32(se + t)
    s, se = fast_two_sum(s, se)
    se = f32(se + te)
    return fast_two_sum(s, se)


def df_add_pos(a, b):
    """the sum of two non-negative values (d^2, the density): no cancellation"""
    s, e = two_sum(a[0], b[0])
    e = f32(e + f32(a[1] + b[1]))
    return fast_two_sum(s, e)


def df_add_f(a, b):
    s, se = two_sum(a[0], b)
    se = f32(se + a[1])
    return fast_two_sum(s, se)


def df_mul(a, b):
    p, e = two_prod(a[0], b[0])
    e = f32(e + f32(a[0] * b[1]))   # the device forms these two with fused multiply-adds
    e = f32(e + f32(a[1] * b[0]))
    return fast_two_sum(p, e)


def df_sqr(a):
    p, e = two_prod(a[0], a[0])
    e = f32(e + f32(f32(f32(2.0) * a[0]) * a[1]))
    return fast_two_sum(p, e)


def split3(x):
    """k_to_pos32: xa = fl32(x), xb = fl32(x - xa), xc = fl32(x - xa - xb) (Float64 diffs)."""
    xa = f32(x)
    r = float(x) - float(xa)
    xb = f32(r)
    xc = f32(r - float(xb))
    return xa, xb, xc


def df_diff3(x, y):
    xa, xb, xc = split3(x)
    ya, yb, yc = split3(y)
    s1, e1 = two_sum(xa, f32(-ya))
    s2, e2 = two_sum(xb, f32(-yb))
    s, e = two_sum(s1, s2)
    low = f32(f32(f32(e1 + e2) + f32(xc - yc)) + e)
    return fast_two_sum(s, low)


def val(d):
    return Fraction(float(d[0])) + Fraction(float(d[1]))


def _points(rng, n, scale, reach=3.0):
    x = rng.uniform(-scale, scale, size=(n, 3))
    y = x + rng.uniform(-reach, reach, size=(n, 3))
    return x, y


def test_split3_is_exact():
    rng = np.random.default_rng(1)
    xs = np.concatenate([rng.uniform(-1e9, 1e9, 2000), rng.uniform(-1.0, 1.0, 2000),
                         rng.uniform(-201.0, 201.0, 2000), [0.0, 1e-300, -3.5, 2.0**60]])
    for x in xs:
        xa, xb, xc = split3(x)
        assert Fraction(float(xa)) + Fraction(float(xb)) + Fraction(float(xc)) == \
            Fraction(float(x)) or abs(x) < 1e-30  # tiny values: the last part underflows


def test_diff3_and_d2_accuracy():
    rng = np.random.default_rng(2)
    # lattice-sized coordinates, large offsets, coordinates on both sides of zero, and
    # nearly coincident points far from the origin (the difference a few ulp of x)
    for scale, reach in ((200.0, 3.0), (1e6, 3.0), (1.0, 3.0), (1e6, 1e-9)):
        x, y = _points(rng, 400, scale, reach)
        for xi, yi in zip(x, y):
            pd = [df_diff3(xi[k], yi[k]) for k in range(3)]
            for k in range(3):
                exact = Fraction(float(xi[k])) - Fraction(float(yi[k]))
                if exact != 0:
                    assert abs(val(pd[k]) - exact) <= abs(exact) * Fraction(1, 2**46)
            d2 = df_add_pos(df_add_pos(df_sqr(pd[0]), df_sqr(pd[1])), df_sqr(pd[2]))
            exact = sum((Fraction(float(xi[k])) - Fraction(float(yi[k])))**2 for k in range(3))
            # the Float64 d^2 is within ~4 ulp (1e-15) of the exact one; the band is 1e-12
            assert abs(val(d2) - exact) <= exact * Fraction(1, 10**13)


def test_mul_add_accuracy():
    rng = np.random.default_rng(3)
    for _ in range(2000):
        u, v = rng.uniform(0.01, 100.0, 2)
        a = (f32(u), f32(u - float(f32(u))))
        b = (f32(v), f32(v - float(f32(v))))
        exact_a, exact_b = val(a), val(b)
        for got, exact in ((df_mul(a, b), exact_a * exact_b), (df_add(a, b), exact_a + exact_b),
                           (df_add_pos(a, b), exact_a + exact_b), (df_sqr(a), exact_a * exact_a)):
            assert abs(val(got) - exact) <= abs(exact) * Fraction(1, 2**44)
