"""The reference arm of bench.py (`--impl reference`): where the grid is too large to
build on the host it computes only the cells its timed particle sample reads.  On a
small map the update over that sparse grid equals, bit for bit, the update over the
full grid, so the arm times exactly the reference's arithmetic.  Host only."""

import numpy as np

import bench
import oracle as O
from amcl3d_gb300 import synth as S


def test_sparse_reference_grid_gives_the_same_update():
    m = S.make_map(17, size_m=(8.0, 6.0, 3.0), n_boxes=8)
    info = dict(min=m.min, max=m.max, res=m.res, dims=m.dims)
    pose = S.free_pose(m, 18, height=1.2, clearance=0.4)
    scan = S.ray_cast(m, pose, n_max=800, max_range=8.0, seed=19)
    ranges = S.beacons(m, pose, 3, seed=20)
    sample = S.particles_around(pose, 300, 21)
    full, how_full = bench.reference_grid(m.points, info, sample, scan, threads=4)
    sparse, how_sparse = bench.reference_grid(m.points, info, sample, scan, threads=4, cell_limit=0)
    assert how_full == "full" and "cells read by the sample" in how_sparse
    a, ma = O.update_f32(sample, full, scan, ranges, 0.5, 0.1, 0.0, 0.0, yaw_trig=0, exp_mode=0)
    b, mb = O.update_f32(sample, sparse, scan, ranges, 0.5, 0.1, 0.0, 0.0, yaw_trig=0, exp_mode=0)
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(ma, mb)
    assert (a[:, 5] > 0).any()  # the sample's weights are not all zero
    touched = np.flatnonzero(sparse.prob)
    assert touched.size < sparse.prob.size
    np.testing.assert_array_equal(sparse.prob[touched], full.prob[touched])


def test_shift_workload_moves_map_particles_and_anchors():
    """`--map-shift` (and the default line's `map_minimum` section) move the map, the
    particles and the beacon anchors; the scans stay in the sensor frame."""
    m = S.make_map(23, size_m=(6.0, 5.0, 3.0), n_boxes=6)
    info = dict(min=m.min, max=m.max, res=m.res, dims=m.dims, n_points=int(m.points.shape[0]))
    pose = S.free_pose(m, 24, height=1.2, clearance=0.4)
    scans = [S.ray_cast(m, pose, n_max=300, max_range=6.0, seed=25)]
    ranges = [S.beacons(m, pose, 3, seed=26)]
    odos = [S.odometry_step(27)]
    parts = S.particles_around(pose, 50, 28)
    sh = (-17.35, -9.5, -1.4)
    occ2, info2, scans2, ranges2, odos2, parts2 = bench.shift_workload(
        (m.points, info, scans, ranges, odos, parts), sh)
    np.testing.assert_allclose(info2["min"], np.asarray(m.min) + sh)
    np.testing.assert_allclose(info2["max"], np.asarray(m.max) + sh)
    assert info2["res"] == info["res"] and info2["dims"] == info["dims"] and info["min"] == m.min
    np.testing.assert_allclose(occ2, m.points.astype(np.float64) + sh, atol=1e-5)
    np.testing.assert_allclose(parts2[:, :3], parts[:, :3].astype(np.float64) + sh, atol=1e-5)
    np.testing.assert_array_equal(parts2[:, 3:], parts[:, 3:])
    np.testing.assert_array_equal(ranges2[0][:, 0], ranges[0][:, 0])
    np.testing.assert_allclose(ranges2[0][:, 1:4], ranges[0][:, 1:4].astype(np.float64) + sh, atol=1e-5)
    assert scans2[0] is scans[0] and odos2[0] is odos[0]
    # every occupied voxel keeps its cell: floor((p - min) / res) is unchanged by the move
    k0 = np.floor((m.points.astype(np.float64) - np.asarray(m.min)) / m.res)
    k1 = np.floor((occ2.astype(np.float64) - np.asarray(info2["min"])) / m.res)
    np.testing.assert_array_equal(k0, k1)
