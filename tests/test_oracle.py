"""The CPU oracle, pinned: against the reference's own fixtures (nav_msg.bin slice),
against outputs of the reference compiled verbatim (committed in
tests/golden/ref_small.npz, and live when oracle/_ref exists), and against
published known answers (Philox)."""

import hashlib
import math
from fractions import Fraction

import numpy as np
import pytest

import oracle as O
from amcl3d_gb300 import synth as S


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


# ---- Philox4x32-10 known-answer vectors (Random123 kat_vectors) ---------------------------------

@pytest.mark.parametrize("ctr,key,expect", [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
])
def test_philox_kat(ctr, key, expect):
    assert O.philox4x32_10(ctr, key) == expect


# ---- restatement vs the committed outputs of the verbatim reference ------------------------------

def small_grid_ref_mode(ref_small):
    b = ref_small["bounds"]
    mn, mx, res = tuple(b[:3]), tuple(b[3:6]), float(b[6])
    d, p = O.compute_grid(ref_small["points"], mn, mx, res, 0.05, exp_mode=0)
    return O.GridData(mn, mx, res, tuple(int(v) for v in ref_small["dims"]), p.ravel(), d.ravel())


def test_compute_grid_matches_reference(ref_small, ref_kat):
    g = small_grid_ref_mode(ref_small)
    assert sha(g.dist) == ref_kat["dist_sha256"]
    assert sha(g.prob) == ref_kat["prob_sha256"]
    z0, z1, y0, y1, x0, x1 = ref_small["sub"]
    dims = tuple(int(v) for v in ref_small["dims"])
    np.testing.assert_array_equal(g.dist.reshape(dims[::-1])[z0:z1, y0:y1, x0:x1], ref_small["dist_sub"])
    np.testing.assert_array_equal(g.prob.reshape(dims[::-1])[z0:z1, y0:y1, x0:x1], ref_small["prob_sub"])


@pytest.mark.parametrize("tag,roll,pitch", [("rp0", 0.0, 0.0), ("rp1", 0.02, -0.03)])
def test_cloud_weight_matches_reference(ref_small, tag, roll, pitch):
    g = small_grid_ref_mode(ref_small)
    w = O.cloud_weights(g, ref_small["particles"][:, :4], ref_small["scan"], roll, pitch, yaw_trig=0)
    np.testing.assert_array_equal(w, ref_small["w_" + tag])


def test_update_and_resample_match_reference(ref_small):
    g = small_grid_ref_mode(ref_small)
    p, mean = O.update_f32(ref_small["particles"], g, ref_small["scan"], ref_small["ranges"], 0.5, 0.1, 0.0, 0.0,
                           yaw_trig=0, exp_mode=0)
    np.testing.assert_array_equal(p, ref_small["updated"])
    np.testing.assert_array_equal(mean, ref_small["mean"][:4])
    idx, over = O.resample_f32(p[:, 4], float(ref_small["u"]))
    assert not over
    np.testing.assert_array_equal(p[idx, :4], ref_small["resampled"][:, :4])
    assert np.all(ref_small["resampled"][:, 4] == np.float32(1.0) / np.float32(p.shape[0]))


# ---- restatement vs the reference's own fixtures ------------------------------------------------

def test_fixture_slice_golden(refdata, ref_kat):
    """nav_msg.bin (Grid3dTest.cpp:45-84's fixture): the z = 1.0 slice of the grid
    built from mappointcloud_msg.bin, bounds [0, 26.1]x[0, 19.2]x[0, 7.65]
    (Grid3dTest.cpp:247), res 0.05, sensor_dev 0.05."""
    mn, mx, res = (0.0, 0.0, 0.0), (26.1, 19.2, 7.65), 0.05
    size = O.grid_sizes(mn, mx, res)
    assert list(size) == ref_kat["fixture_grid_size"]
    iz = int((1.0 - mn[2]) / res)
    _, p = O.compute_grid(refdata["map_points"], mn, mx, res, 0.05, lo=(0, 0, iz), hi=(size[0], size[1], iz + 1),
                          exp_mode=0)
    layer = p.ravel()
    mxp = max(np.float32(layer.max()), np.float32(1e-6))
    sl = (layer * (np.float32(100.0) / mxp)).astype(np.float32).astype(np.int8)
    nav = refdata["nav_slice"]
    assert sl.shape == nav.shape
    assert int((sl != nav).sum()) == ref_kat["slice_mismatch"] == 33
    # With the d^2 (instead of the reference's d^4) Gaussian the agreement drops to ~87 %.


@pytest.mark.slow
def test_fixture_kat_on_rebuilt_grid(refdata, ref_kat):
    """computeCloudWeightTest (Grid3dTest.cpp:120-169) needs data/map/mapfile_complete.bt,
    which the reference does not ship; on the grid rebuilt from its map-cloud fixture
    the reference's arithmetic gives 3.7352 (expected 3.8109): this KAT stays unpinned,
    the value on the rebuilt grid is pinned instead."""
    mn, mx, res = (0.0, 0.0, 0.0), (26.1, 19.2, 7.65), 0.05
    size = O.grid_sizes(mn, mx, res)
    d, p = O.compute_grid(refdata["map_points"], mn, mx, res, 0.05, exp_mode=0)
    assert sha(d.ravel()) == ref_kat["fixture_dist_sha256"]
    g = O.GridData(mn, mx, res, size, p.ravel(), d.ravel())
    w = O.cloud_weights(g, [[20.017967, 10.140815, 3.372801, 0.166781]], refdata["scan"], 0.0, 0.0, yaw_trig=0)
    assert float(w[0]) == ref_kat["kat_on_rebuilt_grid"]
    assert abs(float(w[0]) - ref_kat["kat_expected"]) > 1e-4  # documents the unpinned KAT


# ---- live comparison with the verbatim reference (only where it was built) ------------------------

needs_ref = pytest.mark.skipif(not O.ref_available(), reason="oracle/_ref not built (reference tree absent)")


@needs_ref
@pytest.mark.parametrize("seed", [11, 12])
def test_restatement_vs_reference_live(seed):
    m = S.make_map(seed, size_m=(5.0, 4.0, 2.5), res=0.05, n_boxes=5, box_range=(0.3, 1.5))
    rg = O.RefGrid(m.points, m.min, m.max, m.res, 0.05)
    d_ref, p_ref = rg.cells()
    d, p = O.compute_grid(m.points, m.min, m.max, m.res, 0.05, exp_mode=0)
    np.testing.assert_array_equal(d.ravel(), d_ref)
    np.testing.assert_array_equal(p.ravel(), p_ref)
    g = O.GridData(m.min, m.max, m.res, m.dims, p_ref, d_ref)
    pose = S.free_pose(m, seed, height=1.2, clearance=0.4)
    scan = S.ray_cast(m, pose, n_max=700, max_range=6.0, seed=seed)
    parts = S.particles_around(pose, 40, seed + 1, dxy=1.0, da=0.5)
    for roll, pitch in ((0.0, 0.0), (-0.05, 0.04)):
        w_ref = np.array([rg.cloud_weight(scan, *parts[i, :3], roll, pitch, parts[i, 3]) for i in range(40)],
                         np.float32)
        np.testing.assert_array_equal(O.cloud_weights(g, parts[:, :4], scan, roll, pitch, yaw_trig=0), w_ref)
    ranges = S.beacons(m, pose, 4, seed=seed)
    rf = O.RefFilter(seed)
    rf.set_particles(parts)
    rf.update(rg, scan, ranges, 0.3, 0.2, 0.01, -0.02)
    p_ref_upd = rf.particles()
    p_or, mean = O.update_f32(parts, g, scan, ranges, 0.3, 0.2, 0.01, -0.02, yaw_trig=0, exp_mode=0)
    np.testing.assert_array_equal(p_or, p_ref_upd)
    np.testing.assert_array_equal(mean, rf.mean()[:4])
    u = rf.peek_uniform()
    rf.resample()
    idx, _ = O.resample_f32(p_or[:, 4], u)
    np.testing.assert_array_equal(rf.particles()[:, :4], p_or[idx, :4])
    for i in range(5):
        assert bool(O.ref().ref_grid_is_into_map(rg.h, *parts[i, :3])) == O.is_into_map(g, *parts[i, :3])
    rf.close()
    rg.close()


@needs_ref
def test_resample_overrun_matches_reference():
    """Weights summing (in float) below the last u: the reference runs past p_[N-1]."""
    P = 50
    w = np.full(P, np.float32(0.9) / P, np.float32)
    p = np.zeros((P, 7), np.float32)
    p[:, 0] = np.arange(P)
    p[:, 4] = w
    rf = O.RefFilter(3)
    rf.set_particles(p)
    u = rf.peek_uniform()
    over = rf.resample()
    idx, over2 = O.resample_f32(w, u)
    assert over and over2
    got = rf.particles()
    ok = idx < P
    np.testing.assert_array_equal(got[ok, 0], p[idx[ok], 0])
    assert np.all(got[~ok, 0] == 0)  # the padding the harness puts past the end
    rf.close()


@needs_ref
def test_range_weight_matches_reference():
    rf = O.RefFilter(1)
    rng = np.random.default_rng(0)
    ranges = np.array([[3.0, 0.0, 0.0, 2.0], [4.5, 5.0, 0.0, 2.0], [2.0, 0.0, 4.0, 2.0]], np.float32)
    for _ in range(50):
        x, y, z = rng.uniform(0, 5, 3).astype(np.float32)
        r = float(O.ref().ref_pf_range_weight(rf.h, x, y, z, ranges.ctypes.data_as(O._fp), 3, 0.1))
        assert r == O.range_weight(x, y, z, ranges, 0.1, exp_mode=0)
    assert O.range_weight(1, 1, 1, np.zeros((0, 4), np.float32), 0.1) == 0.0
    rf.close()


# ---- the exact-sum restatement -------------------------------------------------------------------

def test_fsum_is_exact_rounding():
    rng = np.random.default_rng(5)
    v = (rng.random(5000) * 10.0 ** rng.integers(-30, 5, 5000)).astype(np.float32)
    exact = sum(Fraction(float(x)) for x in v)
    assert O.fsum32(v) == float(exact)


def test_resample_exact_matches_fraction_prefix():
    rng = np.random.default_rng(9)
    w = rng.random(300).astype(np.float32)
    w /= w.sum()
    w = w.astype(np.float32)
    u = 0.37
    idx = O.resample_exact(w, u)
    P = len(w)
    factor = np.float32(1) / np.float32(P)
    r = np.float32(factor * np.float32(u))
    pref = np.cumsum([Fraction(float(x)) for x in w])
    for m in range(P):
        um = Fraction(float(np.float32(r + np.float32(factor * np.float32(m)))))
        first = next((i for i in range(P) if pref[i] >= um), P - 1)
        assert idx[m] == first


def test_two_prod32_exact():
    rng = np.random.default_rng(2)
    a = rng.normal(size=1000).astype(np.float32)
    b = (rng.normal(size=1000) * 50).astype(np.float32)
    p, e = O.two_prod32(a, b)
    for i in range(1000):
        assert Fraction(float(p[i])) + Fraction(float(e[i])) == Fraction(float(a[i])) * Fraction(float(b[i]))


def test_synth_is_deterministic():
    m1 = S.make_map(3, size_m=(4.0, 4.0, 2.0), n_boxes=3)
    m2 = S.make_map(3, size_m=(4.0, 4.0, 2.0), n_boxes=3)
    np.testing.assert_array_equal(m1.points, m2.points)
    p = S.free_pose(m1, 1)
    np.testing.assert_array_equal(S.ray_cast(m1, p, seed=4, n_max=200), S.ray_cast(m2, p, seed=4, n_max=200))
    assert math.isclose(S.free_pose(m1, 1)[0], p[0])


def _voxel_numpy(cloud, leaf):
    """Second, independent restatement of pcl::VoxelGrid (numpy float32 keys, a stable
    argsort, per-leaf sums in input order in a Python loop) for the oracle's C version."""
    c = np.asarray(cloud, np.float32)[:, :3]
    fin = np.isfinite(c).all(axis=1)
    p = c[fin]
    inv = np.float32(1.0) / np.asarray(leaf, np.float32) * np.ones(3, np.float32)
    mn, mx = p.min(axis=0), p.max(axis=0)
    span = (mx - mn) * inv
    d = span.astype(np.int64) + 1
    if float(d[0]) * float(d[1]) * float(d[2]) > 2**31 - 1:
        return None
    min_b = np.floor(mn * inv).astype(np.int64)
    div_b = np.floor(mx * inv).astype(np.int64) - min_b + 1
    ijk = (np.floor(p * inv) - min_b.astype(np.float32)).astype(np.int64)
    key = ijk[:, 0] + ijk[:, 1] * div_b[0] + ijk[:, 2] * div_b[0] * div_b[1]
    order = np.argsort(key, kind="stable")
    out = []
    i = 0
    while i < order.size:
        j = i
        s = p[order[i]].copy()
        while j + 1 < order.size and key[order[j + 1]] == key[order[i]]:
            j += 1
            s = (s + p[order[j]]).astype(np.float32)
        out.append(np.append(s / np.float32(j - i + 1), np.float32(1.0)))
        i = j + 1
    return np.array(out, np.float32).reshape(-1, 4)


@pytest.mark.parametrize("leaf", [0.1, 0.5, (0.05, 0.2, 0.3)])
def test_voxel_oracle_two_restatements(leaf):
    rng = np.random.default_rng(3)
    centers = rng.uniform(-4, 4, (150, 3))
    cloud = (centers[rng.integers(0, 150, 3000)] + rng.normal(0, 0.05, (3000, 3))).astype(np.float32)
    cloud[rng.integers(0, 3000, 30), 1] = np.nan
    got, ovf = O.voxel_downsample(cloud, leaf)
    assert not ovf
    np.testing.assert_array_equal(got, _voxel_numpy(cloud, leaf))


def test_voxel_oracle_properties():
    """Size-independent properties: one centroid per distinct leaf, all inside the cloud's
    bounding box, w = 1; the int32 overflow returns the input; empty in, empty out."""
    rng = np.random.default_rng(4)
    cloud = rng.uniform(-10, 10, (20000, 4)).astype(np.float32)
    out, ovf = O.voxel_downsample(cloud, 0.7)
    inv = np.float32(1.0) / np.float32(0.7)
    leaves = np.unique(np.floor(cloud[:, :3] * inv), axis=0)
    assert out.shape[0] == leaves.shape[0] and not ovf
    assert (out[:, 3] == 1.0).all()
    assert (out[:, :3] >= cloud[:, :3].min(axis=0)).all() and (out[:, :3] <= cloud[:, :3].max(axis=0)).all()
    same, ovf = O.voxel_downsample(cloud, 1e-4)
    assert ovf and same.shape[0] == cloud.shape[0]
    np.testing.assert_array_equal(same[:, :3], cloud[:, :3])
    empty, ovf = O.voxel_downsample(np.zeros((0, 4), np.float32), 0.1)
    assert empty.shape == (0, 4) and not ovf
