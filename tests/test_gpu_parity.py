"""GPU parity: every hot-path function of the CUDA library against the oracle on the
same seeded inputs, bit-exact where the arithmetic is the same, within the stated
tolerance where it differs by design (the GPU's exact sums vs the reference's float
running sums; double sin/exp rounded to float vs libm's sinf/expf)."""

import hashlib

import numpy as np
import pytest

import oracle as O
from amcl3d_gb300 import synth as S
from conftest import small_grid_data

pytestmark = pytest.mark.gpu

REL_REF = 1e-5  # per-particle weights vs the reference's float arithmetic


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def ulps(a, b):
    a = np.asarray(a, np.float32).view(np.int32).astype(np.int64)
    b = np.asarray(b, np.float32).view(np.int32).astype(np.int64)
    return np.abs(a - b)


def gpu_grid_from(amcl, g: "O.GridData"):
    G = amcl.Grid3d()
    G.load_cells({"min": g.min, "max": g.max, "size": g.size, "resolution": g.res, "sensor_dev": 0.05}, g.dist,
                 g.prob)
    return G


@pytest.fixture(scope="module")
def small(amcl, ref_small):
    g = small_grid_data(ref_small)
    return g, gpu_grid_from(amcl, g)


# ---- distance field ---------------------------------------------------------------------------

def test_distance_field_exact(amcl, ref_small, ref_kat):
    b = ref_small["bounds"]
    G = amcl.Grid3d()
    assert G.buildGridMap(ref_small["points"], b[:3], b[3:6], float(b[6]), 0.05)
    d, p = G.read_cells()
    assert sha(d) == ref_kat["dist_sha256"]  # the reference's squared distances, bit for bit
    g = small_grid_data(ref_small)  # oracle with exp in double rounded to float
    u = ulps(p, g.prob)
    assert u.max() <= 1 and (u > 0).mean() < 1e-4
    _, p_ref = O.compute_grid(ref_small["points"], b[:3], b[3:6], float(b[6]), 0.05, exp_mode=0)
    assert ulps(p, p_ref.ravel()).max() <= 2  # vs libm expf
    assert G.info()["size"] == tuple(int(v) for v in ref_small["dims"])


def test_distance_field_fixture_and_slice(amcl, refdata, ref_kat):
    """The reference's map-cloud fixture (179,551 points, 522x384x153 cells): squared
    distances equal the reference's everywhere, and the z = 1.0 slice reproduces
    nav_msg.bin with the reference's own 33 mismatches.  This snapshot's
    buildGridSliceMsg sizes the slice point2grid(max) - point2grid(min) =
    522 + 384*522 = 200970 values (the verbatim reference gives the same); the
    fixture, from an older version, holds the 522x384 layer, i.e. the first 200448."""
    G = amcl.Grid3d()
    G.buildGridMap(refdata["map_points"], (0.0, 0.0, 0.0), (26.1, 19.2, 7.65), 0.05, 0.05)
    d, _ = G.read_cells()
    assert sha(d) == ref_kat["fixture_dist_sha256"]
    out = G.buildGridSliceMsg(1.0)
    assert out is not None
    sl, w, h = out
    assert (w, h) == (522, 384)
    assert sl.size == 522 + 384 * 522
    nav = refdata["nav_slice"]
    assert int((sl[: nav.size] != nav).sum()) == ref_kat["slice_mismatch"]
    assert G.buildGridSliceMsg(-100.0) is None  # Grid3dTest.cpp:77-79
    # KAT pose of Grid3dTest.cpp:128-168 on the rebuilt grid (unpinned against 3.8109)
    kat = G.computeCloudWeight(refdata["scan"], 20.017967, 10.140815, 3.372801, 0.0, 0.0, 0.166781)
    assert abs(kat - ref_kat["kat_on_rebuilt_grid"]) <= 1e-5 * ref_kat["kat_on_rebuilt_grid"]
    assert G.isIntoMap(1, 1, 1) and not G.isIntoMap(-100, -100, -100)  # Grid3dTest.cpp:245-266


def test_empty_grid_semantics(amcl):
    G = amcl.Grid3d()
    assert G.computeCloudWeight(np.zeros((20, 3), np.float32), 1, 1, 1, 0, 0, 0) == 0.0  # Grid3dTest.cpp:160-161
    assert not G.isIntoMap(1, 1, 1)
    assert G.buildGridSliceMsg(0.0) is None


def test_distance_field_no_points(amcl):
    G = amcl.Grid3d()
    G.buildGridMap(np.zeros((0, 3), np.float32), (0, 0, 0), (1.0, 1.0, 1.0), 0.05, 0.05)
    d, p = G.read_cells()
    assert np.all(d == -1.0) and np.all(p == 0.0)  # PointCloudTools.cpp:142-143


def test_distance_field_negative_origin_offlattice(amcl):
    """Bounds not on a lattice through 0 (the reference test map's min is -17.35)."""
    rng = np.random.default_rng(4)
    pts = np.column_stack([rng.uniform(-17.35, -15.0, 3000), rng.uniform(-9.5, -8.0, 3000),
                           rng.uniform(-1.4, 0.3, 3000)]).astype(np.float32)
    mn, mx = (-17.35, -9.5, -1.4), (-14.9, -7.9, 0.35)
    G = amcl.Grid3d()
    G.buildGridMap(pts, mn, mx, 0.05, 0.05)
    d, p = G.read_cells()
    d_o, p_o = O.compute_grid(pts, mn, mx, 0.05, 0.05, exp_mode=1)
    np.testing.assert_array_equal(d, d_o.ravel())
    assert ulps(p, p_o.ravel()).max() <= 1


def test_grid_file_roundtrip(amcl, small, tmp_path):
    g, G = small
    path = tmp_path / "map.grid"
    assert G.saveGrid(str(path))
    raw = path.read_bytes()
    sx, sy, sz = np.frombuffer(raw[:12], np.uint32)
    dev = np.frombuffer(raw[12:20], np.float64)[0]
    assert (sx, sy, sz) == g.size and dev == 0.05
    cells = np.frombuffer(raw[20:], np.float32).reshape(-1, 2)
    np.testing.assert_array_equal(cells[:, 0], g.dist)
    np.testing.assert_array_equal(cells[:, 1], g.prob)
    H = amcl.Grid3d()
    assert H.loadGrid(str(path), g.min, g.max, g.res, 0.05)
    np.testing.assert_array_equal(H.read_cells()[1], g.prob)
    assert not H.loadGrid(str(path), g.min, g.max, g.res, 0.06)  # Grid3d.cpp:256-260


# ---- cloud weights ------------------------------------------------------------------------------

@pytest.mark.parametrize("roll,pitch", [(0.0, 0.0), (0.02, -0.03), (-0.3, 0.25)])
def test_cloud_weights_bit_exact(amcl, small, ref_small, roll, pitch):
    g, G = small
    poses = ref_small["particles"][:, :4]
    w_gpu = G.computeCloudWeights(poses, ref_small["scan"], roll, pitch)
    w_orc, cells = O.cloud_weights(g, poses, ref_small["scan"], roll, pitch, yaw_trig=1, cells=True)
    np.testing.assert_array_equal(w_gpu, w_orc)
    if (roll, pitch) != (-0.3, 0.25):
        tag = "rp0" if roll == 0.0 else "rp1"
        w_ref = ref_small["w_" + tag]
        np.testing.assert_allclose(w_gpu, w_ref, rtol=REL_REF, atol=0)


def test_cloud_weight_edge_cases(amcl, small, ref_small):
    g, G = small
    scan = ref_small["scan"]
    pose = ref_small["particles"][0, :4]
    # <= 10 in-grid points gives 0 (Grid3d.cpp:198)
    assert G.computeCloudWeight(scan[:10], *pose[:3], 0, 0, pose[3]) == 0.0
    assert G.computeCloudWeight(scan[:0], *pose[:3], 0, 0, pose[3]) == 0.0
    w11 = G.computeCloudWeight(scan[:40], *pose[:3], 0, 0, pose[3])
    assert w11 == O.cloud_weights(g, [pose], scan[:40], 0, 0, yaw_trig=1)[0]
    # points far outside the grid are skipped, NaN points too
    junk = np.array([[1e3, 0, 0], [0, -1e3, 0], [np.nan, 0, 0], [0, 0, np.inf]], np.float32)
    s2 = np.concatenate([scan[:, :3], junk])
    assert G.computeCloudWeight(s2, *pose[:3], 0, 0, pose[3]) == O.cloud_weights(g, [pose], s2, 0, 0, yaw_trig=1)[0]
    # a pose far outside the map: every point misses
    assert G.computeCloudWeight(scan, 100.0, 100.0, 100.0, 0, 0, 0) == 0.0


def test_cloud_weights_on_lattice_boundaries(amcl, small):
    """Points whose transformed coordinates land exactly on cell boundaries (the
    double add / divide / floor chain of Grid3d.cpp:174-183 decides their cell)."""
    g, G = small
    k = np.arange(1, 90, dtype=np.float64)
    xs = (k * 0.05).astype(np.float32)
    pts = np.zeros((xs.size * 3, 3), np.float32)
    pts[: xs.size, 0] = xs - np.float32(1.0)
    pts[xs.size: 2 * xs.size, 1] = xs - np.float32(1.0)
    pts[2 * xs.size:, 2] = xs - np.float32(1.0)
    poses = np.array([[1.0, 1.0, 1.0, 0.0], [1.05, 0.95, 0.5, 0.0], [2.0, 2.0, 1.0, np.pi / 2],
                      [1.5, 1.5, 1.5, -np.pi]], np.float32)
    w_gpu = G.computeCloudWeights(poses, pts)
    w_orc, cells = O.cloud_weights(g, poses, pts, yaw_trig=1, cells=True)
    np.testing.assert_array_equal(w_gpu, w_orc)


@pytest.mark.parametrize("roll,pitch", [(0.0, 0.0), (0.01, -0.02)])
def test_cloud_weights_one_thread_per_particle(amcl, roll, pitch):
    """Enough particles for the one-thread-per-particle weighting (65,536) on a map whose
    minimum is 0, so every offset is an exact float: the yaw-only path (x and y paired
    in two-wide instructions) and the exact-offset path, against the oracle.  About one
    pair in a million has a transformed coordinate within an ulp of a cell boundary,
    where an extra rounding step (or a missing one) moves the point to the next cell."""
    m = S.make_map(32, size_m=(10.0, 10.0, 4.0), n_boxes=12)
    G = amcl.Grid3d()
    assert G.buildGridMap(m.points, m.min, m.max, m.res, S.SENSOR_DEV)
    pose = S.free_pose(m, 43, height=1.2, clearance=0.4)
    scan = S.ray_cast(m, pose, n_max=1200, max_range=8.0, seed=53)
    poses = np.ascontiguousarray(S.particles_around(pose, 65536, 63)[:, :4])
    w_gpu = G.computeCloudWeights(poses, scan, roll, pitch)
    inf = G.info()
    g = O.GridData(inf["min"], inf["max"], inf["resolution"], inf["size"], G.read_cells()[1])
    np.testing.assert_array_equal(w_gpu, O.cloud_weights(g, poses, scan, roll, pitch, yaw_trig=1))


@pytest.mark.parametrize("nx", [2**21 - 1, 2**21 + 3])
def test_cloud_weights_long_axis(amcl, nx):
    """An x axis of about 2^21 cells (x up to 105 km at 0.05 m): below 2^21 cells the
    two bracket floors settle the cell, from 2^21 on every point goes through the
    threshold table (the upper bracket is +inf).  Particles spread along the whole
    axis, against the oracle on the same cells."""
    size = (nx, 2, 2)
    res = 0.05
    rng = np.random.default_rng(11)
    prob = rng.random(nx * 4, dtype=np.float32)
    dist = np.zeros_like(prob)
    mx = tuple(float(s * res) for s in size)
    G = amcl.Grid3d()
    G.load_cells({"min": (0.0, 0.0, 0.0), "max": mx, "size": size, "resolution": res, "sensor_dev": 0.05}, dist,
                 prob)
    P, N = 4096, 512
    poses = np.zeros((P, 4), np.float32)
    poses[:, 0] = rng.uniform(0.0, mx[0], P).astype(np.float32)
    poses[:, 0][:8] = np.float32(mx[0]) - np.arange(8, dtype=np.float32)  # next to the far end
    scan = np.zeros((N, 3), np.float32)
    scan[:, 0] = rng.uniform(-20.0, 20.0, N).astype(np.float32)
    scan[:, 1] = rng.uniform(0.0, 0.1, N).astype(np.float32)
    scan[:, 2] = rng.uniform(0.0, 0.1, N).astype(np.float32)
    w_gpu = G.computeCloudWeights(poses, scan)
    g = O.GridData((0.0, 0.0, 0.0), mx, res, size, prob)
    w_orc = O.cloud_weights(g, poses, scan, 0.0, 0.0, yaw_trig=1)
    np.testing.assert_array_equal(w_gpu, w_orc)
    assert (w_orc > 0).mean() > 0.9


# ---- update / normalise / mean --------------------------------------------------------------------

def run_update(amcl, G, parts, scan, ranges, alpha=0.5, sigma=0.1, roll=0.0, pitch=0.0, kernel=0, cloud_sum=0):
    pf = amcl.ParticleFilter(seed=1)
    pf.set_option(3, kernel)
    pf.set_option(1, cloud_sum)
    pf.set_particles(parts)
    pf.update(G, scan, ranges, alpha, sigma, roll, pitch)
    return pf


@pytest.mark.parametrize("kernel", [1, 2])
def test_update_bit_exact_vs_exact_oracle(amcl, small, ref_small, kernel):
    g, G = small
    parts = ref_small["particles"].copy()
    parts[:, 5] = np.linspace(0.1, 0.9, parts.shape[0])  # stale wp/wr of out-of-map particles survive
    parts[:, 6] = np.linspace(0.2, 0.3, parts.shape[0])
    pf = run_update(amcl, G, parts, ref_small["scan"], ref_small["ranges"], kernel=kernel)
    got = pf.particles()
    exp, m32, m64, var = O.update_exact(parts, g, ref_small["scan"], ref_small["ranges"], 0.5, 0.1, 0.0, 0.0)
    np.testing.assert_array_equal(got, exp)
    mean = pf.getMean()
    np.testing.assert_array_equal(np.array([mean.x, mean.y, mean.z, mean.a], np.float32), m32)
    mv, vv = pf.mean_var()
    np.testing.assert_array_equal(mv, m64)
    np.testing.assert_allclose(vv, var, rtol=1e-12, atol=1e-18)


def test_update_vs_reference_tolerance(amcl, small, ref_small):
    """Against the reference's own update (float running sums): per-particle raw
    weights within 1e-5 relative (wp, wr before normalisation), normalised
    weights within the float-sum error."""
    g, G = small
    parts = ref_small["particles"]
    pf = run_update(amcl, G, parts, ref_small["scan"], ref_small["ranges"])
    got = pf.particles()
    ref = ref_small["updated"]
    np.testing.assert_array_equal(got[:, :4], ref[:, :4])
    np.testing.assert_allclose(got[:, 4:7], ref[:, 4:7], rtol=1e-5, atol=1e-9)
    m = pf.getMean()
    np.testing.assert_allclose([m.x, m.y, m.z, m.a], ref_small["mean"][:4], rtol=1e-5)


def test_update_all_out_of_map_and_no_ranges(amcl, small, ref_small):
    g, G = small
    parts = ref_small["particles"].copy()
    parts[:, 2] = 50.0  # above the map
    pf = run_update(amcl, G, parts, ref_small["scan"], np.zeros((0, 4), np.float32))
    got = pf.particles()
    assert np.all(got[:, 4] == 0)
    exp, m32, _, _ = O.update_exact(parts, g, ref_small["scan"], np.zeros((0, 4), np.float32), 0.5, 0.1, 0.0, 0.0)
    np.testing.assert_array_equal(got, exp)
    m = pf.getMean()
    assert (m.x, m.y, m.z, m.a) == (0.0, 0.0, 0.0, 0.0)


def test_update_ranges_only(amcl, ref_small):
    pf = amcl.ParticleFilter(seed=2)
    parts = ref_small["particles"]
    pf.set_particles(parts)
    pf.update_ranges(ref_small["ranges"], 0.5, 0.1)
    got = pf.particles()
    wr = np.array([O.range_weight(*parts[i, :3], ref_small["ranges"], 0.1) for i in range(parts.shape[0])],
                  np.float32)
    s = O.fsum32(wr)
    wrn = (wr.astype(np.float64) / s).astype(np.float32)
    np.testing.assert_array_equal(got[:, 6], wrn)
    assert np.all(got[:, 5] == 0)


# ---- resample -------------------------------------------------------------------------------------

@pytest.mark.parametrize("u", [0.0, 0.37, 0.999])
def test_resample_exact_prefix(amcl, small, ref_small, u):
    g, G = small
    pf = run_update(amcl, G, ref_small["particles"], ref_small["scan"], ref_small["ranges"])
    before = pf.particles()
    pf.resample(u)
    idx = pf.resample_index()
    np.testing.assert_array_equal(idx, O.resample_exact(before[:, 4], u))
    after = pf.particles()
    np.testing.assert_array_equal(after[:, :4], before[idx, :4])
    assert np.all(after[:, 4] == np.float32(1) / np.float32(before.shape[0]))


def test_resample_reference_prefix_mode(amcl, small, ref_small):
    g, G = small
    pf = run_update(amcl, G, ref_small["particles"], ref_small["scan"], ref_small["ranges"])
    pf.set_option(2, 1)
    before = pf.particles()
    u = float(ref_small["u"])
    pf.resample(u)
    idx = pf.resample_index()
    ref_idx, over = O.resample_f32(before[:, 4], u)
    assert not over
    np.testing.assert_array_equal(idx, ref_idx)
    np.testing.assert_array_equal(pf.particles()[:, :4], ref_small["resampled"][:, :4])


def test_resample_overrun_clamps(amcl):
    """Float weights summing below the last u: the reference reads past its array;
    here those outputs take the last particle."""
    P = 50
    p = np.zeros((P, 7), np.float32)
    p[:, 0] = np.arange(P)
    p[:, 4] = np.float32(0.9) / P
    pf = amcl.ParticleFilter()
    pf.set_particles(p)
    pf.set_option(2, 1)
    pf.resample(0.5)
    idx = pf.resample_index()
    ref_idx, over = O.resample_f32(p[:, 4], 0.5)
    assert over
    np.testing.assert_array_equal(idx, np.minimum(ref_idx, P - 1))
    pf.set_option(2, 0)
    pf.set_particles(p)
    pf.resample(0.5)
    np.testing.assert_array_equal(pf.resample_index(), O.resample_exact(p[:, 4], 0.5))


def test_resample_all_zero_weights(amcl):
    p = np.zeros((16, 7), np.float32)
    p[:, 0] = np.arange(16)
    pf = amcl.ParticleFilter()
    pf.set_particles(p)
    pf.resample(0.25)
    np.testing.assert_array_equal(pf.resample_index(), O.resample_exact(p[:, 4], 0.25))


# ---- predict / init ---------------------------------------------------------------------------------

def test_predict_bit_exact_given_draws(amcl, ref_small):
    pf = amcl.ParticleFilter(seed=123)
    parts = ref_small["particles"]
    pf.set_particles(parts)
    pf.record_draws(True)
    mods = (0.1, 0.1, 0.01, 0.3)
    deltas = (-0.067421, -0.006161, 0.130909, 0.052421)  # ParticleFilterTest.cpp:50-57
    pf.predict(*mods, *deltas)
    z = pf.draws()
    np.testing.assert_array_equal(pf.particles()[:, :4], O.predict(parts, z, mods, deltas)[:, :4])
    m0 = pf.getMean()
    pf.predict(*mods, *deltas)
    assert pf.getMean() == m0  # predict leaves the stored mean (ParticleFilterTest.cpp:60-71)


def test_init_bit_exact_given_draws(amcl):
    pf = amcl.ParticleFilter(seed=7)
    pf.record_draws(True)
    args = (600, 2.87080164308, 1.63820032984, 0.21460881682, 0.144, 0.05, 0.05, 0.05, 0.1)  # ParticleFilterTest
    pf.init(*args)
    assert pf.isInitialized() and pf.size() == 600
    z = pf.draws()
    p = O.init_pose(600, z, args[1:5], args[5:9])
    wn, m32, m64, var = O.normalize_stats(p[:, 4], p[:, :4])
    got = pf.particles()
    np.testing.assert_array_equal(got[:, :4], p[:, :4])
    np.testing.assert_array_equal(got[:, 4], wn)
    m = pf.getMean()
    np.testing.assert_array_equal(np.array([m.x, m.y, m.z, m.a], np.float32), m32)
    assert abs(m.x - args[1]) < 0.01 and abs(m.a - args[4]) < 0.01  # the commented-out initTest


def test_init_abs_count_and_zero(amcl):
    pf = amcl.ParticleFilter()
    pf.init(-32, 0, 0, 0, 0, 0.1, 0.1, 0.1, 0.1)
    assert pf.size() == 32  # abs(num_particles), ParticleFilter.cpp:51
    with pytest.raises(Exception):
        pf.init(0, 0, 0, 0, 0, 0.1, 0.1, 0.1, 0.1)


def test_normal_draws_statistics(amcl):
    pf = amcl.ParticleFilter(seed=99)
    pf.record_draws(True)
    pf.init(200000, 0, 0, 0, 0, 1, 1, 1, 1)
    z = pf.draws()[1:].ravel().astype(np.float64)
    assert abs(z.mean()) < 0.01 and abs(z.std() - 1.0) < 0.01
    assert abs((np.abs(z) < 1).mean() - 0.6827) < 0.005


def floor_constants_fit(size):
    """Whether the grid gets floor constants (the host's solve, restated): offsets m of
    2^23 with sum_a (0x4B000000 + m[a]) * stride[a] = 0 mod 2^32, each leaving room for
    size[a] + 2 cells below 2^23."""
    sx, sy, sz = size
    two32, b = 1 << 32, 0x4B000000
    r = (two32 - (b * ((1 + sx + sx * sy) % two32)) % two32) % two32
    m2, r2 = divmod(r, sx * sy)
    m1, m0 = divmod(r2, sx)
    return all(m + n + 2 <= (1 << 23) for m, n in zip((m0, m1, m2), size))


@pytest.mark.parametrize("dims,mn,tail,fast,loop", [
    ((10, 11, 10), (0.0, 0.0, 0.0), 0.0, False, 0),
    ((44, 40, 16), (0.0, 0.0, 0.0), 0.0, True, 1),
    ((44, 40, 16), (-17.35, -9.5, -1.4), 0.0, True, 2),
    ((44, 40, 16), (-17.35, -9.5, -1.4), 0.4, True, 0),
    ((44, 40, 16), (-9.5, -4.25, -1.5), 0.0, True, 2),
], ids=["no-floor-constants", "zero-minimum", "real-minimum", "real-minimum-partial-last-cell", "float-minimum"])
def test_cloud_weights_yaw_loops(amcl, dims, mn, tail, fast, loop):
    """The one-thread-per-particle yaw-only weighting (65,536 particles, random cell
    probabilities, scan points inside and outside the grid) against the oracle on each
    loop: a grid too small for floor constants (10 x 11 x 10 cells: the constants'
    offsets would not fit below 2^23); a zero minimum (every offset a float: the cell
    index from the floor bits, a zero pad cell for rejected points); a minimum like a
    real octomap map's (offsets that are not floats: the float estimate with widened
    floors, the reference's double add near cell boundaries and near 0); and the same
    with a partial last cell (the bound then inside a cell: the general path); a float
    minimum (many offsets are then floats, L = 0, and the rest ties often).  A
    thousand particles at yaw 0 and one x see a point placed to land within a few
    ulps of 0 on x, where only the double add decides the side."""
    rng = np.random.default_rng(sum(dims) + int(tail * 10) + int(abs(mn[0]) > 0))
    res = 0.05
    full = tuple(d - (1 if tail else 0) for d in dims)
    mx = tuple(mn[a] + (full[a] + tail) * res for a in range(3))
    size = tuple(int(v) for v in O.grid_sizes(mn, mx, res))
    assert size == dims
    assert floor_constants_fit(size) == fast
    cells = int(np.prod(size))
    prob = rng.uniform(0.0, 8.0, cells).astype(np.float32)
    dist = rng.uniform(0.0, 1.0, cells).astype(np.float32)
    G = amcl.Grid3d()
    G.load_cells({"min": mn, "max": mx, "size": size, "resolution": res, "sensor_dev": 0.05}, dist, prob)
    assert G.weight_loop() == loop
    centre = (np.array(mn) + np.array(mx)) / 2
    ext = np.array(mx) - np.array(mn)
    P = 65536
    poses = np.zeros((P, 4), np.float32)
    poses[:, :3] = centre + rng.uniform(-0.1, 0.1, (P, 3))
    poses[:, 3] = rng.uniform(-3.2, 3.2, P)
    poses[:1000, 3] = 0.0
    poses[:1000, 0] = np.float32(centre[0] + 0.0137)
    scan = np.zeros((700, 4), np.float32)
    scan[:, :3] = rng.uniform(-0.7, 0.7, (700, 3)) * ext / ext.max()
    # the point that lands at ~0 on x for the first thousand particles: x = -fl32(t_x - min_x)
    h = np.float32(float(poses[0, 0]) - mn[0])
    scan[5, 0] = -h
    w_gpu = G.computeCloudWeights(poses, scan)
    g = O.GridData(mn, mx, res, size, prob, dist)
    want = O.cloud_weights(g, poses, scan, 0.0, 0.0, yaw_trig=1)
    assert (want > 0).mean() > 0.5  # most particles keep more than 10 points
    np.testing.assert_array_equal(w_gpu, want)
