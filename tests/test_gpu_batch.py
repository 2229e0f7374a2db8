"""Batched filters (amcl_batch_*): every filter stepped inside a batch computes exactly
what the same filter computes stepped alone (same seed, same inputs), whatever the
other filters in the step and whether the step's weighting runs fused (a thread per
particle) or split over points (slabs summed in cloud order); admission against the
arena budget; the autotuner keeps the filters' state."""

import numpy as np
import pytest

from amcl3d_gb300 import synth as S

pytestmark = pytest.mark.gpu

MODS = S.ODOM_MODS


@pytest.fixture(scope="module")
def world(amcl):
    maps = [S.make_map(31, size_m=(8.0, 6.0, 3.0), n_boxes=8), S.make_map(32, size_m=(10.0, 10.0, 4.0), n_boxes=12)]
    grids = []
    for m in maps:
        G = amcl.Grid3d()
        G.buildGridMap(m.points, m.min, m.max, m.res, S.SENSOR_DEV)
        grids.append(G)
    specs = []  # (map index, P, n points, roll, pitch, seed)
    for k, (mi, P, n, roll, pitch) in enumerate([(0, 300, 400, 0.0, 0.0), (1, 1500, 1000, 0.0, 0.0),
                                                 (0, 6000, 250, 0.03, -0.02), (1, 20000, 1200, 0.0, 0.0),
                                                 (0, 700, 0, 0.0, 0.0)]):
        m = maps[mi]
        pose = S.free_pose(m, 40 + k, height=1.2, clearance=0.4)
        scans = [S.ray_cast(m, pose, n_max=n, max_range=8.0, seed=50 + k + 10 * s) if n else
                 np.zeros((0, 4), np.float32) for s in range(3)]
        parts = S.particles_around(pose, P, 60 + k)
        ranges = S.beacons(m, pose, 3, seed=70 + k)
        specs.append(dict(grid=mi, P=P, scans=scans, parts=parts, ranges=ranges, roll=roll, pitch=pitch,
                          seed=1000 + k))
    return grids, specs


def run_alone(amcl, grids, sp, steps):
    pf = amcl.ParticleFilter(seed=sp["seed"])
    pf.set_particles(sp["parts"])
    out = []
    for s in range(steps):
        pf.predict(*MODS, 0.05, 0.01, 0.0, 0.02)
        pf.update(grids[sp["grid"]], sp["scans"][s], sp["ranges"], 0.5, 0.1, sp["roll"], sp["pitch"])
        m = pf.getMean()
        pf.resample()
        out.append((pf.particles(), np.array([m.x, m.y, m.z, m.a], np.float32)))
    return out


@pytest.mark.parametrize("split", [1, 2], ids=["fused", "split"])
@pytest.mark.parametrize("tuning", [(256, 1024), (128, 256), (512, 2048)])
def test_batch_equals_alone(amcl, world, tuning, split):
    from amcl3d_gb300.batch import FilterBatch

    grids, specs = world
    steps = 3
    alone = [run_alone(amcl, grids, sp, steps) for sp in specs]
    B = FilterBatch(max_filters=8, max_particles=40000, max_points_per_step=8000)
    B.set_tuning(*tuning)
    B.set_split(split)  # fused tiles, or every scan split over the SMs (the 0-point filter stays fused)
    slots = []
    for sp in specs:
        sl = B.add(grids[sp["grid"]], sp["P"], sp["seed"])
        B.set_particles(sl, sp["parts"])
        slots.append(sl)
    odom = (*MODS, 0.05, 0.01, 0.0, 0.02)
    for s in range(steps):
        for sl, sp in zip(slots, specs):
            B.stage(sl, sp["scans"][s], sp["ranges"], odom, 0.5, 0.1, sp["roll"], sp["pitch"], resample=True)
        B.step()
        B.wait()
        for i, (sl, sp) in enumerate(zip(slots, specs)):
            p_alone, m_alone = alone[i][s]
            m, _, _ = B.mean_var(sl)
            np.testing.assert_array_equal(m, m_alone, err_msg=f"filter {i} step {s} mean")
            np.testing.assert_array_equal(B.particles(sl, sp["P"]), p_alone, err_msg=f"filter {i} step {s}")


def test_batch_subset_steps_and_autotune(amcl, world):
    """Only some filters stage a step; the others keep their state.  The autotuner
    restores every filter's state."""
    from amcl3d_gb300.batch import FilterBatch

    grids, specs = world
    B = FilterBatch(max_filters=8, max_particles=40000, max_points_per_step=8000)
    slots = [B.add(grids[sp["grid"]], sp["P"], sp["seed"]) for sp in specs]
    for sl, sp in zip(slots, specs):
        B.set_particles(sl, sp["parts"])
    odom = (*MODS, 0.05, 0.01, 0.0, 0.02)
    B.stage(slots[1], specs[1]["scans"][0], specs[1]["ranges"], odom, 0.5, 0.1)
    B.stage(slots[3], specs[3]["scans"][0], specs[3]["ranges"], odom, 0.5, 0.1)
    B.step()
    B.wait()
    np.testing.assert_array_equal(B.particles(slots[0], specs[0]["P"]), specs[0]["parts"])
    before = [B.particles(sl, sp["P"]) for sl, sp in zip(slots, specs)]
    t, c, ms = B.autotune(reps=2)
    assert t in (128, 256, 512) and c in (256, 512, 1024, 2048) and ms > 0
    assert B.tuning() == (t, c)
    for sl, sp, b in zip(slots, specs, before):
        np.testing.assert_array_equal(B.particles(sl, sp["P"]), b)
    alone = run_alone(amcl, grids, specs[3], 2)
    B.stage(slots[3], specs[3]["scans"][1], specs[3]["ranges"], odom, 0.5, 0.1)
    B.step()
    B.wait()
    np.testing.assert_array_equal(B.particles(slots[3], specs[3]["P"]), alone[1][0])


def test_batch_admission(amcl, world):
    from amcl3d_gb300 import _native as N
    from amcl3d_gb300.batch import FilterBatch

    grids, _ = world
    B = FilterBatch(max_filters=2, max_particles=1000, max_points_per_step=100)
    a = B.add(grids[0], 600, 1)
    assert B.try_add(grids[0], 2000, 2) is None  # beyond the particle arena
    b = B.add(grids[0], 256, 3)
    assert B.try_add(grids[0], 10, 4) is None  # no slot left
    B.remove(a)
    c = B.try_add(grids[0], 500, 5)
    assert c is not None
    free_p, free_s = B.capacity()
    assert free_s == 0
    B.init(b, 200, 1.0, 1.0, 1.0, 0.0, 0.05, 0.05, 0.05, 0.1)
    big = np.zeros((500, 4), np.float32)
    B.stage(b, big, None)
    with pytest.raises(N.AmclError):
        B.step()  # the staged clouds exceed max_points_per_step


def test_stage_many_equals_stage(amcl, world):
    """Staging every filter in one native call gives the same step as staging each."""
    from amcl3d_gb300.batch import FilterBatch

    grids, specs = world
    out = []
    for many in (False, True):
        B = FilterBatch(max_filters=8, max_particles=40000, max_points_per_step=8000)
        slots = [B.add(grids[sp["grid"]], sp["P"], sp["seed"]) for sp in specs]
        for sl, sp in zip(slots, specs):
            B.set_particles(sl, sp["parts"])
        odom = (*MODS, 0.05, 0.01, 0.0, 0.02)
        for s in range(2):
            if many:
                B.stage_many(slots, [sp["scans"][s] for sp in specs], [sp["ranges"] for sp in specs], odom)
            else:
                for sl, sp in zip(slots, specs):
                    B.stage(sl, sp["scans"][s], sp["ranges"], odom)
            B.step()
            B.wait()
        out.append([B.particles(sl, sp["P"]) for sl, sp in zip(slots, specs)])
        B.close()
    for a, b in zip(*out):
        np.testing.assert_array_equal(a, b)


def test_batch_more_grids_than_slots(amcl):
    """Six filters on six maps in one batch: four grids ride in the launch's grid slots,
    two are read from their step descriptors.  Then three filters move to two other maps
    (free slots are reused, the captured graphs rebuilt) and two maps no filter uses are
    destroyed.  Three of the maps sit at a minimum like a real octomap map's (offsets that
    are not floats: the general yaw loop).  Every filter steps exactly as the same filter
    stepped alone over the same maps."""
    import gc

    from amcl3d_gb300.batch import FilterBatch

    maps = [S.make_map(80 + k, size_m=(6.0 + k, 5.0, 3.0), n_boxes=6) for k in range(8)]
    shifts = {2: (-3.35, -1.15, -0.45), 3: (-17.35, -9.5, -1.4), 5: (-0.35, -2.7, -0.15)}  # filters 2, 3, 5 stay

    def moved(k, xyz):  # map-local coordinates into map k's frame
        return (np.asarray(xyz, np.float64) + np.asarray(shifts.get(k, (0.0, 0.0, 0.0)))).astype(np.float32)

    grids = []
    for k, m in enumerate(maps):
        G = amcl.Grid3d()
        assert G.buildGridMap(moved(k, m.points), tuple(np.asarray(m.min) + shifts.get(k, (0.0, 0.0, 0.0))),
                              tuple(np.asarray(m.max) + shifts.get(k, (0.0, 0.0, 0.0))), m.res, S.SENSOR_DEV)
        assert G.weight_loop() == (2 if k in shifts else 1)
        grids.append(G)
    odom = (*MODS, 0.05, 0.01, 0.0, 0.02)
    moves = {0: 6, 1: 7, 4: 6}  # filter -> map from step 2 on
    specs = []
    for k in range(6):
        pose = S.free_pose(maps[k], 90 + k, height=1.2, clearance=0.4)
        seq = [k, k, moves.get(k, k), moves.get(k, k)]  # map of each step
        poses = [pose if g == k else S.free_pose(maps[g], 7 + k, height=1.2, clearance=0.4) for g in seq]
        scans = [S.ray_cast(maps[g], q, n_max=600, max_range=6.0, seed=99 + k + 10 * s)
                 for s, (g, q) in enumerate(zip(seq, poses))]
        parts = S.particles_around(pose, 1000 + 700 * k, 95 + k)
        parts[:, :3] = moved(k, parts[:, :3])
        ranges = S.beacons(maps[k], pose, 3, seed=120 + k)
        ranges[:, 1:4] = moved(k, ranges[:, 1:4])
        specs.append(dict(seq=seq, P=1000 + 700 * k, seed=500 + k, parts=parts, scans=scans, ranges=ranges))
    alone = []
    for sp in specs:
        pf = amcl.ParticleFilter(seed=sp["seed"])
        pf.set_particles(sp["parts"])
        out = []
        for s in range(4):
            pf.predict(*odom)
            pf.update(grids[sp["seq"][s]], sp["scans"][s], sp["ranges"], 0.5, 0.1, 0.0, 0.0)
            pf.getMean()
            pf.resample()
            out.append(pf.particles())
        alone.append(out)
    B = FilterBatch(max_filters=8, max_particles=40000, max_points_per_step=8000)
    slots = []
    for sp in specs:
        sl = B.add(grids[sp["seq"][0]], sp["P"], sp["seed"])
        B.set_particles(sl, sp["parts"])
        slots.append(sl)
    for s in range(4):
        if s == 2:
            for i, g in moves.items():
                B.set_grid(slots[i], grids[g])
            grids[0] = grids[1] = None  # maps no filter uses any more
            gc.collect()
        for sl, sp in zip(slots, specs):
            B.stage(sl, sp["scans"][s], sp["ranges"], odom, 0.5, 0.1)
        B.step()
        B.wait()
        for i, (sl, sp) in enumerate(zip(slots, specs)):
            np.testing.assert_array_equal(B.particles(sl, sp["P"]), alone[i][s], err_msg=f"filter {i} step {s}")
    B.close()


def test_stage_packed_equals_stage_many(amcl, world):
    """Filters staged from one packed cloud (amcl_batch_stage_packed, copied on host
    threads) step exactly as the same filters staged one array each."""
    from amcl3d_gb300.batch import FilterBatch

    grids, specs = world
    sps = [sp for sp in specs if sp["roll"] == 0.0]
    odom = (*MODS, 0.05, 0.01, 0.0, 0.02)
    out = []
    for packed in (False, True):
        B = FilterBatch(max_filters=len(sps), max_particles=sum(sp["P"] + 256 for sp in sps),
                        max_points_per_step=8000)
        slots = [B.add(grids[sp["grid"]], sp["P"], sp["seed"]) for sp in sps]
        for sl, sp in zip(slots, sps):
            B.set_particles(sl, sp["parts"])
        res = []
        for s in range(2):
            clouds = [sp["scans"][s] for sp in sps]
            rgs = [sp["ranges"] for sp in sps]
            if packed:
                B.stage_packed(slots, np.concatenate(clouds), [c.shape[0] for c in clouds], np.concatenate(rgs),
                               [r.shape[0] for r in rgs], odom)
            else:
                B.stage_many(slots, clouds, rgs, odom)
            B.step()
            B.wait()
            res.append([B.particles(sl, sp["P"]) for sl, sp in zip(slots, sps)])
        out.append(res)
        B.close()
    for a, b in zip(out[0], out[1]):
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y)


def test_stage_packed_rejects_a_repeated_slot(amcl, world):
    from amcl3d_gb300 import _native as N
    from amcl3d_gb300.batch import FilterBatch

    grids, specs = world
    sp = specs[1]
    B = FilterBatch(max_filters=2, max_particles=2 * (sp["P"] + 256), max_points_per_step=4000)
    sl = B.add(grids[sp["grid"]], sp["P"], 1)
    B.set_particles(sl, sp["parts"])
    cloud = sp["scans"][0]
    with pytest.raises(N.AmclError):
        B.stage_packed([sl, sl], np.concatenate([cloud, cloud]), [cloud.shape[0]] * 2)
    B.close()


def test_auto_mode_wide_and_long_filters(amcl, world):
    """The automatic weighting choice on a step holding a wide filter with a short scan
    and a narrow one with a long scan, on two maps' worth of launches: both equal the
    same filters stepped alone."""
    from amcl3d_gb300.batch import FilterBatch

    grids, specs = world
    m_wide = S.make_map(31, size_m=(8.0, 6.0, 3.0), n_boxes=8)
    pose = S.free_pose(m_wide, 81, height=1.2, clearance=0.4)
    wide = dict(grid=0, P=100000, scans=[S.ray_cast(m_wide, pose, n_max=150, max_range=8.0, seed=82 + s)
                                          for s in range(2)],
                parts=S.particles_around(pose, 100000, 83), ranges=S.beacons(m_wide, pose, 3, seed=84), roll=0.0,
                pitch=0.0, seed=2001)
    long_scan = dict(specs[3])  # on the other map: two fused launches, run as parallel branches
    long_scan["P"] = 2000
    long_scan["parts"] = specs[3]["parts"][:2000]
    mix = [wide, long_scan]
    steps = 2
    alone = [run_alone(amcl, grids, sp, steps) for sp in mix]
    B = FilterBatch(max_filters=4, max_particles=110000, max_points_per_step=4000)
    B.set_split(0)
    slots = []
    for sp in mix:
        sl = B.add(grids[sp["grid"]], sp["P"], sp["seed"])
        B.set_particles(sl, sp["parts"])
        slots.append(sl)
    odom = (*MODS, 0.05, 0.01, 0.0, 0.02)
    for s in range(steps):
        for sl, sp in zip(slots, mix):
            B.stage(sl, sp["scans"][s], sp["ranges"], odom, 0.5, 0.1)
        B.step()
        B.wait()
        for i, (sl, sp) in enumerate(zip(slots, mix)):
            np.testing.assert_array_equal(B.particles(sl, sp["P"]), alone[i][s][0], err_msg=f"filter {i} step {s}")
