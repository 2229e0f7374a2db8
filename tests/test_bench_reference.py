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
