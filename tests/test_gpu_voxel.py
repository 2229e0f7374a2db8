"""Scan voxel downsample on the GPU (pcl::VoxelGrid<PointXYZ> as Node.cpp:130-137 runs
it) against the oracle's restatement of PCL's algorithm: the same centroids, bit for
bit, in the same order; edge cases (empty, non-finite points, one leaf, duplicates,
the int32 overflow that returns the input); the device-buffer entry point; and the
fused voxel + update call against the two steps done separately."""

import ctypes as C

import numpy as np
import pytest

import oracle as O
from amcl3d_gb300 import synth as S

pytestmark = pytest.mark.gpu


def _scan(n_elev, n_azim, seed):
    m = S.make_map(seed, size_m=(20.0, 20.0, 5.0), n_boxes=40)
    pose = S.free_pose(m, seed + 1)
    return S.ray_cast(m, pose, n_elev=n_elev, n_azim=n_azim, max_range=15.0, n_max=n_elev * n_azim, seed=seed + 2)


def _cases():
    rng = np.random.default_rng(5)
    out = {}
    out["uniform"] = (rng.uniform(-20, 20, (20000, 4)).astype(np.float32), 0.1)
    out["lidar_64x1024"] = (_scan(64, 1024, 11), 0.1)
    centers = rng.uniform(-5, 5, (500, 3))
    out["clustered"] = ((centers[rng.integers(0, 500, 30000)] + rng.normal(0, 0.02, (30000, 3))).astype(np.float32),
                        0.1)
    nf = rng.uniform(-3, 3, (5000, 4)).astype(np.float32)
    nf[rng.integers(0, 5000, 300), rng.integers(0, 3, 300)] = np.nan
    nf[rng.integers(0, 5000, 50), 0] = np.inf
    nf[rng.integers(0, 5000, 50), 2] = -np.inf
    out["nonfinite"] = (nf, 0.25)
    out["single"] = (np.array([[1.5, -2.25, 0.75, 1.0]], np.float32), 0.1)
    out["one_leaf"] = (rng.uniform(0.01, 0.09, (4000, 4)).astype(np.float32), 0.1)
    dup = np.repeat(rng.uniform(-1, 1, (50, 4)).astype(np.float32), 40, axis=0)
    out["duplicates"] = (dup[rng.permutation(dup.shape[0])], 0.05)
    out["negative_anisotropic"] = (rng.uniform(-40, -0.001, (50000, 4)).astype(np.float32), (0.05, 0.2, 0.5))
    out["large_1M"] = (rng.uniform(-60, 60, (1 << 20, 4)).astype(np.float32) * np.float32([1, 1, 0.1, 1]), 1.0)
    out["overflow"] = (rng.uniform(-100, 100, (3000, 4)).astype(np.float32), 1e-4)
    return out


CASES = _cases()


@pytest.mark.parametrize("name", sorted(CASES))
def test_voxel_bit_exact(amcl, name):
    cloud, leaf = CASES[name]
    exp, ovf = O.voxel_downsample(cloud, leaf)
    assert ovf == (name == "overflow")
    got = amcl.VoxelGrid().downsample(cloud, leaf)
    assert got.shape == exp.shape, (name, got.shape, exp.shape)
    np.testing.assert_array_equal(got, exp)


def test_voxel_xyz_stride3_and_pcl_calls(amcl):
    cloud, leaf = CASES["clustered"]
    v = amcl.VoxelGrid()
    v.setInputCloud(cloud[:, :3])
    v.setLeafSize(leaf, leaf, leaf)
    np.testing.assert_array_equal(v.filter(), O.voxel_downsample(cloud, leaf)[0])


def test_voxel_empty_and_all_nonfinite(amcl):
    v = amcl.VoxelGrid()
    assert v.downsample(np.zeros((0, 4), np.float32), 0.1).shape == (0, 4)
    assert v.downsample(np.full((100, 4), np.nan, np.float32), 0.1).shape == (0, 4)


@pytest.mark.parametrize("leaf", [0.0, -0.1, float("nan"), float("inf"), 1e-45])
def test_voxel_rejects_bad_leaf(amcl, leaf):
    from amcl3d_gb300 import _native as N

    with pytest.raises(N.AmclError) as e:
        amcl.VoxelGrid().downsample(CASES["single"][0], leaf)
    assert e.value.status == 1  # AMCL_EINVAL


def test_voxel_output_too_small(amcl):
    from amcl3d_gb300 import _native as N

    cloud, leaf = CASES["uniform"]
    v = amcl.VoxelGrid()
    out = np.empty((10, 4), np.float32)
    m = C.c_uint64()
    rc = N.lib.amcl_voxel_filter(v.handle, N.fptr(cloud), cloud.shape[0], 4, leaf, leaf, leaf, N.fptr(out), 10,
                                 C.byref(m))
    assert rc == 7 and m.value == O.voxel_downsample(cloud, leaf)[0].shape[0]  # AMCL_ERANGE, size reported


def test_voxel_device_buffers(amcl):
    import torch

    cloud, leaf = CASES["lidar_64x1024"]
    d_in = torch.from_numpy(np.ascontiguousarray(cloud)).cuda()
    d_out = torch.empty_like(d_in)
    v = amcl.VoxelGrid()
    m = v.downsample_dev(d_in.data_ptr(), d_in.shape[0], leaf, d_out.data_ptr())
    np.testing.assert_array_equal(d_out[:m].cpu().numpy(), O.voxel_downsample(cloud, leaf)[0])
    # repeated calls on one handle reuse its scratch and give the same answer
    m2 = v.downsample_dev(d_in.data_ptr(), d_in.shape[0], leaf, d_out.data_ptr())
    assert m2 == m


def test_update_voxel_equals_filter_then_update(amcl):
    m = S.make_map(31, size_m=(20.0, 20.0, 5.0), n_boxes=40)
    G = amcl.Grid3d()
    G.buildGridMap(m.points, m.min, m.max, m.res, S.SENSOR_DEV)
    pose = S.free_pose(m, 32)
    raw = S.ray_cast(m, pose, n_elev=32, n_azim=512, max_range=15.0, n_max=32 * 512, seed=33)
    ranges = S.beacons(m, pose, 3, seed=34)
    parts = S.particles_around(pose, 5000, 35)
    vox = amcl.VoxelGrid()
    a, b = amcl.ParticleFilter(seed=3), amcl.ParticleFilter(seed=3)
    a.set_particles(parts)
    b.set_particles(parts)
    down = a.update_voxel(G, vox, raw, 0.1, ranges, 0.5, 0.1, 0.0, 0.0)
    down_b = vox.downsample(raw, 0.1)
    b.update(G, down_b, ranges, 0.5, 0.1, 0.0, 0.0)
    np.testing.assert_array_equal(down, down_b)
    np.testing.assert_array_equal(down, O.voxel_downsample(raw, 0.1)[0])
    assert down.shape[0] < raw.shape[0]
    np.testing.assert_array_equal(a.particles(), b.particles())
    np.testing.assert_array_equal(a.mean_var()[0], b.mean_var()[0])
    # the size-only form skips the copy back
    assert a.update_voxel(G, vox, raw, 0.1, ranges, 0.5, 0.1, 0.0, 0.0, want_cloud=False) == down.shape[0]
