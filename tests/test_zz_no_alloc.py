"""amcl_grid_cloud_weights_noalloc: the weighting entry point for callers that
cannot allocate device memory (its scratch is a fixed file-scope device array).
Checked through the C ABI against amcl_grid_cloud_weights, which allocates its
own buffers, on two calls in a row: the shared array must not carry anything over
from one call into the next.  Kept in its own file, collected last."""

import ctypes as C

import numpy as np
import pytest

import oracle as O
from conftest import small_grid_data

pytestmark = pytest.mark.gpu


def _noalloc(native, grid, poses_dev, P, cloud_dev, n, out_dev, roll=0.0, pitch=0.0):
    return native.lib.amcl_grid_cloud_weights_noalloc(grid.handle, C.c_void_p(poses_dev), P, C.c_void_p(cloud_dev), n,
                                                      float(roll), float(pitch), C.c_void_p(out_dev), None)


def test_noalloc_matches_allocating_entry_point(amcl, ref_small):
    import torch

    from amcl3d_gb300 import _native as N

    g = small_grid_data(ref_small)
    G = amcl.Grid3d()
    G.load_cells({"min": g.min, "max": g.max, "size": g.size, "resolution": g.res, "sensor_dev": 0.05}, g.dist,
                 g.prob)
    scan = np.ascontiguousarray(ref_small["scan"], np.float32)  # (N, 4)
    rng = np.random.default_rng(3)
    poses_a = np.ascontiguousarray(ref_small["particles"][:, :4])
    poses_b = poses_a.copy()
    poses_b[:, :2] += rng.uniform(-0.3, 0.3, (poses_b.shape[0], 2)).astype(np.float32)
    poses_b[:, 3] += np.float32(0.2)
    dev = torch.device("cuda", 0)
    d_scan = torch.from_numpy(scan).to(dev)
    results = []
    free = []
    for poses, (roll, pitch), cloud in ((poses_a, (0.0, 0.0), scan), (poses_b, (0.02, -0.01), scan[:700])):
        d_poses = torch.from_numpy(poses).to(dev)
        d_out = torch.full((poses.shape[0],), -7.0, dtype=torch.float32, device=dev)
        torch.cuda.synchronize()
        rc = _noalloc(N, G, d_poses.data_ptr(), poses.shape[0], d_scan.data_ptr(), cloud.shape[0], d_out.data_ptr(),
                      roll, pitch)
        assert rc == 0, N.lib.amcl_last_error().decode()
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info(0)[0])
        got = d_out.cpu().numpy()
        want = G.computeCloudWeights(poses, cloud, roll, pitch)
        np.testing.assert_array_equal(got, want)  # same kernels, same bits
        # and the oracle's computeCloudWeight directly (the GPU's sin/cos: yaw_trig=1)
        np.testing.assert_array_equal(got, O.cloud_weights(g, poses, cloud, roll, pitch, yaw_trig=1))
        results.append(got)
    assert not np.array_equal(results[0], results[1])
    assert free[0] == free[1]  # no device memory taken between the calls


def test_noalloc_rejects_sizes_beyond_the_array(amcl, ref_small):
    from amcl3d_gb300 import _native as N

    g = small_grid_data(ref_small)
    G = amcl.Grid3d()
    G.load_cells({"min": g.min, "max": g.max, "size": g.size, "resolution": g.res, "sensor_dev": 0.05}, g.dist,
                 g.prob)
    fake = 1 << 20  # never dereferenced: the size checks come first
    assert _noalloc(N, G, fake, 65537, fake, 10, fake) == 7  # AMCL_ERANGE
    assert b"65536" in N.lib.amcl_last_error()
    assert _noalloc(N, G, fake, 4096, fake, 1025, fake) == 7  # 4096*1025 > 4194304
    assert b"scratch" in N.lib.amcl_last_error()


def test_noalloc_unbuilt_grid_gives_zeros(amcl):
    """computeCloudWeight of a grid that was never opened is 0 (Grid3d.cpp:136-137)."""
    import torch

    from amcl3d_gb300 import _native as N

    G = amcl.Grid3d()
    dev = torch.device("cuda", 0)
    poses = torch.zeros((5, 4), dtype=torch.float32, device=dev)
    cloud = torch.zeros((20, 4), dtype=torch.float32, device=dev)
    out = torch.full((5,), -7.0, dtype=torch.float32, device=dev)
    torch.cuda.synchronize()
    assert _noalloc(N, G, poses.data_ptr(), 5, cloud.data_ptr(), 20, out.data_ptr()) == 0
    assert np.all(out.cpu().numpy() == 0.0)
