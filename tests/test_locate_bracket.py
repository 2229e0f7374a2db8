"""The cell-floor argument of the weighting kernels, checked in exact arithmetic on the
CPU.  The kernels bracket 1/res by two floats inv_lo <= 1/res <= inv_hi (each found from
fl32(1/res) by stepping at least 2^-50 relative away, as grid.cu does) and take
floor(X * inv_lo) and floor(X * inv_hi) with round-down fused multiply-adds; when the two
agree they must equal the reference's floor(fl64(X / res)) (Grid3d.cpp:181-183).  Here the
products are exact rationals, X runs over random coordinates and over the floats around
every cell boundary k * res, and the share of coordinates that need the threshold table
(the floors disagree) stays near q * 2^-22."""

import math
from fractions import Fraction

import numpy as np
import pytest


def bracket(res: float):
    ir = 1.0 / res
    lo = hi = np.float32(ir)
    while float(lo) > ir * (1.0 - 2.0**-50):
        lo = np.nextafter(lo, np.float32(0.0))
    while float(hi) < ir * (1.0 + 2.0**-50):
        hi = np.nextafter(hi, np.float32(np.inf))
    return lo, hi


def coordinates(res: float, size: int, rng):
    xs = list(rng.uniform(0.0, size * res, 4000).astype(np.float32))
    for k in rng.integers(1, size, 300):
        x = np.float32(k * res)
        for _ in range(3):
            x = np.nextafter(x, np.float32(0.0))
        for _ in range(7):
            xs.append(x)
            x = np.nextafter(x, np.float32(np.inf))
    return xs


@pytest.mark.parametrize("res", [0.05, 0.1, 0.02, 0.3, 0.07, 0.125, 1.0 / 3.0, 0.2])
def test_agreeing_floors_are_the_reference_cell(res):
    rng = np.random.default_rng(int(res * 1e6))
    lo, hi = bracket(res)
    assert float(lo) < 1.0 / res < float(hi)
    flo, fhi = Fraction(float(lo)), Fraction(float(hi))
    size = 2000
    near = 0
    xs = coordinates(res, size, rng)
    for X in xs:
        xf = Fraction(float(X))
        a, b = math.floor(xf * flo), math.floor(xf * fhi)
        ref = math.floor(float(X) / res)  # the reference's double divide, then floor
        assert a <= ref <= b
        if a == b:
            assert a == ref, (res, float(X))
        else:
            near += 1
    # the boundary points (2,100 of the coordinates) dominate; random ones rarely need the table
    assert near < 0.5 * len(xs)


def test_random_coordinates_rarely_need_the_table():
    rng = np.random.default_rng(3)
    res = 0.05
    lo, hi = bracket(res)
    flo, fhi = Fraction(float(lo)), Fraction(float(hi))
    xs = rng.uniform(0.0, 100.0, 20000).astype(np.float32)
    near = sum(1 for X in xs if math.floor(Fraction(float(X)) * flo) != math.floor(Fraction(float(X)) * fhi))
    # expected about mean(q) * (hi - lo) / (1/res) ~ 1000 * 2^-22.3 ~ 2e-4 of the coordinates
    assert near <= 20


def test_round_down_fma_floor_range():
    """X * inv + 1.5 * 2^23 stays in [2^23, 2^24) for 0 <= X * inv < 2^22, where the floats
    are the integers, so rounding the exact sum down gives 1.5 * 2^23 + floor(X * inv); the
    kernels use it for axes below 2^21 cells (a valid X keeps X * inv_hi below size + 1)."""
    c = Fraction(3 * 2**22)
    for q in [Fraction(0), Fraction(1, 3), Fraction(2**21) + Fraction(1, 7), Fraction(2**22) - Fraction(1, 2**20)]:
        s = c + q
        assert 2**23 <= s < 2**24
        assert math.floor(s) - c == math.floor(q)


def floor_constants(size):
    """The grid's floor constants m[a] (grid.cu, restated): sum_a (bits(2^23) + m[a]) * stride[a]
    = 0 mod 2^32 with strides (1, sx, sx * sy), or None where an offset leaves no room for
    size[a] + 2 floors below 2^24."""
    sx, sy, sz = size
    two32, b = 1 << 32, 0x4B000000
    s1, s2 = sx, sx * sy
    r = (two32 - (b * ((1 + s1 + s2) % two32)) % two32) % two32
    m2, r2 = divmod(r, s2)
    m1, m0 = divmod(r2, s1)
    m = (m0, m1, m2)
    if any(mi + n + 2 > (1 << 23) for mi, n in zip(m, size)):
        return None
    return m


@pytest.mark.parametrize("size", [(2000, 2000, 400), (800, 800, 160), (400, 400, 100), (200, 200, 200),
                                  (1000, 1000, 200), (44, 40, 16), (120, 100, 60), (522, 384, 153),
                                  (2097151, 2, 2), (3, 5, 7), (10, 11, 10)])
def test_floor_bits_are_the_cell_index(size):
    """The zero-minimum and real-map yaw loops read the cell index off the bit patterns of
    the three round-down floors fma_rd(X, inv, 2^23 + m[a]) = 2^23 + m[a] + k[a] (floats in
    [2^23, 2^24) are the integers): weighted by the strides they sum, mod 2^32, to the
    reference's ix + iy * sx + iz * sx * sy (Grid3d.cpp:187) for every cell, the one-past
    floors included."""
    m = floor_constants(size)
    if size in ((3, 5, 7), (10, 11, 10)):
        assert m is None  # too small for the constants: the general loop takes such grids
        return
    assert m is not None
    sx, sy, sz = size
    rng = np.random.default_rng(sum(size))
    k = np.stack([rng.integers(0, n + 2, 20000) for n in size], 1)
    k[:3] = [[0, 0, 0], [sx - 1, sy - 1, sz - 1], [sx + 1, sy + 1, sz + 1]]
    bits = np.stack([(np.float32(2.0**23) + np.float32(m[a]) + k[:, a].astype(np.float32)).view(np.uint32)
                     for a in range(3)], 1).astype(np.uint64)
    stride = np.array([1, sx, sx * sy], np.uint64)
    idx = (bits * stride).sum(1) % (1 << 32)
    want = (k[:, 0] + k[:, 1] * sx + k[:, 2] * sx * sy).astype(np.uint64) % (1 << 32)
    np.testing.assert_array_equal(idx, want)
