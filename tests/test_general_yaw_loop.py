"""The arithmetic of the general yaw loop (maps whose minimum makes the particle offsets
non-floats, as a real octomap map's does), checked on the CPU in IEEE float32/float64
against the reference's X = fl32(fl64(f + (double(t) - min))) (Grid3d.cpp:155-157) and
its cell floor(fl64(X / res)) (Grid3d.cpp:181-183).

The loop splits off = double(t) - min as H + L (H = fl32(off), L = fl32(off - H)) and
takes v = (f + H) + L in float.  Claim 1: wherever |v| >= 2^-20 max|H| and the floors of
v against 1/res bracketed 2^-22 relative below and above agree, X has v's sign and the
floor is the reference's cell.  Claim 2 (the open points): Knuth's two-sum estimate of X
with its residual test is the reference's X wherever the test does not call the rounding
undecided.  f runs over uniform coordinates, over the floats around every cell boundary
and around the map's minimum plane (X near 0)."""

import numpy as np
import pytest

F32 = np.float32


def widened(res: float):
    """inv_lo2 / inv_hi2 as the grid's host code builds them."""
    ir = 1.0 / res
    lo = hi = F32(ir)
    while float(lo) > ir * (1.0 - 2.0**-22):
        lo = np.nextafter(lo, F32(0.0))
    while float(hi) < ir * (1.0 + 2.0**-22):
        hi = np.nextafter(hi, F32(np.inf))
    return lo, hi


def split(off: np.ndarray):
    """H, L as the kernels' per-particle set-up makes them: L = 0 only where off == H."""
    H = off.astype(F32) + F32(0.0)
    rest = off - H.astype(np.float64)
    L = rest.astype(F32)
    tiny = (L == 0) & (rest != 0)
    L[tiny] = np.copysign(F32(1.401298464324817e-45), rest[tiny]).astype(F32)
    return H, L


def two_sum_x(s, H, L):
    """The open-point estimate of X and whether its rounding is undecided (the kernel's
    gen_exact_x, restated in float32)."""
    a = s + H
    bv = a - s
    av = a - bv
    e = (s - av) + (H - bv)
    t = e + L
    X = a + t
    w = (a - X) + t
    xb = X.view(np.uint32) & np.uint32(0x7FFFFFFF)
    half_ulp = ((xb & np.uint32(0x7F800000)) - np.uint32(24 << 23)).view(F32)
    margin = (np.abs(w) + np.abs(t)) * F32(2.0**-23) + np.abs(H) * F32(2.0**-47)
    amb = (~(np.abs(np.abs(w) - half_ulp) > margin)) | ((xb & np.uint32(0x7FFFFF)) == 0) | (xb < 0x0D000000) | \
        ~(np.abs(a) >= np.abs(H) * F32(2.0**-20))
    return X, amb & (L != 0)


def cases(res, mn, extent, n, rng):
    """Particle coordinates t inside the map and transformed point coordinates f: uniform,
    around cell boundaries (X = k * res) and around the minimum plane (X = 0)."""
    t = (mn + rng.uniform(0.0, extent, n)).astype(F32)
    off = t.astype(np.float64) - mn
    f = rng.uniform(-40.0, 40.0, n).astype(F32)
    third = n // 3
    k = rng.integers(0, int(extent / res), third)
    f[:third] = (k * res - off[:third]).astype(F32)
    f[third:2 * third] = (-off[third:2 * third]).astype(F32)
    steps = rng.integers(-6, 7, 2 * third).astype(np.int32)
    bits = f[:2 * third].view(np.int32) + steps
    f[:2 * third] = bits.view(F32)
    return t, off, f


@pytest.mark.parametrize("res,mn", [(0.05, -17.35), (0.05, -9.5), (0.1, -1.4), (0.05, -0.35),
                                    (0.2, -123.456), (0.07, 3.3), (0.05, -2.7)])
def test_general_yaw_floors_and_open_points(res, mn):
    rng = np.random.default_rng(int(res * 1000) + int(abs(mn) * 100))
    extent = 100.0
    n = 600_000
    t, off, f = cases(res, mn, extent, n, rng)
    H, L = split(off)
    v = (f + H) + L
    X = (f.astype(np.float64) + off).astype(F32)  # the reference
    lo2, hi2 = widened(res)
    flo = np.floor(v.astype(np.float64) * float(lo2))  # exact products: 24 x 24 bits
    fhi = np.floor(v.astype(np.float64) * float(hi2))
    zb = F32(2.0**-20) * np.abs(H)
    # the estimate's error bound behind the bracket: |v - X| <= 3.125 * 2^-24 |v| + 2^-47 |H|
    # (below the bracket's 4 * 2^-24) wherever |v| >= 2^-20 |H|
    far = np.abs(v) >= zb
    err = np.abs(v[far].astype(np.float64) - X[far].astype(np.float64))
    bound = 3.125 * 2.0**-24 * np.abs(v[far].astype(np.float64)) + 2.0**-47 * np.abs(H[far].astype(np.float64))
    assert (err <= bound).all()
    settled = far & (flo == fhi)
    # claim 1: settled points have X's sign and, inside the map, the reference's cell
    assert np.array_equal(X[settled] < 0, v[settled] < 0)
    inside = settled & (X >= 0)
    ref_cell = np.floor(X[inside].astype(np.float64) / res)
    np.testing.assert_array_equal(flo[inside], ref_cell)
    # the uniform third rarely needs the exact path
    uni = slice(2 * (n // 3), n)
    assert (~settled[uni]).mean() < 2e-3
    # claim 2: the open points' two-sum estimate is the reference's X where decided
    Xe, amb = two_sum_x(f, H, L)
    ok = ~amb
    np.testing.assert_array_equal(Xe[ok].view(np.uint32), X[ok].view(np.uint32))
    # undecided: the points on the minimum plane (a = f + H cancels) where off is no
    # float, and sums at or next to a tie (common where a float minimum such as -9.5
    # leaves L a few bits); an offset that is a float (L = 0) never
    third = n // 3
    assert amb[:third].mean() < 0.05 and amb[uni].mean() < 0.05
    assert not amb[L == 0].any()
