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
and around the map's minimum plane (X near 0).  Then the loop's whole cell decision
(floors, bounds, the near-zero bound, open points), restated, against the oracle's cell
for every particle x point pair."""

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


def floor_threshold(res: float, k: int) -> np.float32:
    """The smallest float X >= 0 with floor(fl64(X) / res) >= k (the grid's threshold table)."""
    if k == 0:
        return F32(0.0)
    x = F32(k * res)
    while not np.floor(float(x) / res) >= k:
        x = np.nextafter(x, F32(np.inf))
    while True:
        d = np.nextafter(x, F32(-np.inf))
        if d >= 0 and np.floor(float(d) / res) >= k:
            x = d
        else:
            return x


def general_loop_cells(poses, scan, mn, res, size):
    """The cell of every (particle, point) pair as the general yaw loop decides it
    (weigh_chunk_yaw2_gen, open_cell), restated in numpy; -1 where it gathers the pad."""
    yaw = poses[:, 3].astype(np.float64)
    cy = np.cos(yaw).astype(F32)[:, None]
    sy = np.sin(yaw).astype(F32)[:, None]
    x, y, z = (scan[None, :, a].astype(F32) for a in range(3))
    s = [(x * cy) + (-(y * sy)), (x * sy) + (y * cy), np.broadcast_to(z, (poses.shape[0], scan.shape[0]))]
    V = [floor_threshold(res, n) for n in size]
    k = []
    near = np.zeros(s[0].shape, bool)
    valid = np.ones(s[0].shape, bool)
    X, Hs, vs = [], [], []
    for a in range(3):
        off = poses[:, a].astype(np.float64) - mn[a]
        H, L = split(off)
        H, L = H[:, None], L[:, None]
        Hs.append(H)
        v = (s[a] + H) + L
        vs.append(v)
        lo2, hi2 = widened(res)
        flo = np.floor(v.astype(np.float64) * float(lo2))
        fhi = np.floor(v.astype(np.float64) * float(hi2))
        near |= flo != fhi
        valid &= (v >= 0) & (v < V[a]) & ~np.signbit(v)
        k.append(flo)
        Xe, amb = two_sum_x(s[a], np.broadcast_to(H, s[a].shape), np.broadcast_to(L, s[a].shape))
        Xr = (s[a].astype(np.float64) + off[:, None]).astype(F32)
        X.append(np.where(amb, Xr, Xe))
    zb = F32(2.0**-20) * np.maximum(np.maximum(np.abs(Hs[0]), np.abs(Hs[1])), np.abs(Hs[2]))
    for v in vs:
        near |= np.abs(v) < zb
    sx_, sy_ = size[0], size[1]
    cell = np.where(valid & ~near, k[0] + k[1] * sx_ + k[2] * sx_ * sy_, -1).astype(np.int64)
    # open points: the reference's cell of the two-sum (or double-add) X
    ok = np.ones(s[0].shape, bool)
    kk = []
    for a in range(3):
        ok &= (X[a] >= 0) & (X[a] < V[a])
        kk.append(np.floor(X[a].astype(np.float64) / res))
    open_cell = np.where(ok, kk[0] + kk[1] * sx_ + kk[2] * sx_ * sy_, -1).astype(np.int64)
    return np.where(near, open_cell, cell), near


@pytest.mark.parametrize("mn", [(-17.35, -9.5, -1.4), (-9.5, -4.25, -1.5), (-0.35, -2.7, -0.15)])
def test_general_loop_cells_equal_the_reference(mn):
    """Every (particle, point) cell of the general yaw loop, restated, equals the
    reference's (the oracle's cells): random poses and points over a 44 x 40 x 16 grid,
    plus points placed for yaw-0 particles within a few ulps of cell boundaries and of
    the minimum plane."""
    import oracle as O

    res = 0.05
    size = (44, 40, 16)
    mx = tuple(mn[a] + size[a] * res for a in range(3))
    assert tuple(int(v) for v in O.grid_sizes(mn, mx, res)) == size
    rng = np.random.default_rng(int(abs(mn[0]) * 100))
    P = 400
    centre = (np.array(mn) + np.array(mx)) / 2
    poses = np.zeros((P, 4), F32)
    poses[:, :3] = centre + rng.uniform(-0.3, 0.3, (P, 3))
    poses[:, 3] = rng.uniform(-3.2, 3.2, P)
    poses[:64, 3] = 0.0
    ext = np.array(mx) - np.array(mn)
    pts = [rng.uniform(-0.6, 0.6, (1500, 3)) * ext / ext.max()]
    for p in range(64):  # yaw 0: s is the point itself
        off = poses[p, :3].astype(np.float64) - np.array(mn)
        q = np.zeros((12, 3))
        for j in range(12):
            for a in range(3):
                kcell = rng.integers(0, size[a] + 1) if j < 9 else 0
                q[j, a] = F32(kcell * res - off[a])
        pts.append(q)
    cloud = np.zeros((sum(c.shape[0] for c in pts), 4), F32)
    cloud[:, :3] = np.concatenate(pts).astype(F32)
    nb = cloud.shape[0] - 1500
    bits = cloud[1500:, :3].view(np.int32) + rng.integers(-3, 4, (nb, 3)).astype(np.int32)
    cloud[1500:, :3] = bits.view(F32)
    prob = rng.uniform(0.0, 8.0, int(np.prod(size))).astype(F32)
    g = O.GridData(mn, mx, res, size, prob, np.zeros_like(prob))
    _, want = O.cloud_weights(g, poses, cloud, 0.0, 0.0, yaw_trig=1, cells=True)
    got, near = general_loop_cells(poses, cloud, mn, res, size)
    np.testing.assert_array_equal(got, want)
    assert near.sum() > 100  # the placed points reach the open-point path
