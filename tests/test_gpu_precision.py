"""Reduced-precision grids (FP16, uint8 with a per-grid scale) and the compensated
cloud sum, against an FP64 oracle of the per-particle weight: the mean, in double, of
the FP64 probabilities of the cells the reference's arithmetic selects (cells from the
bit-exact restatement, so only the storage and the summation differ)."""

import numpy as np
import pytest

import oracle as O
from amcl3d_gb300 import synth as S

pytestmark = pytest.mark.gpu

TOL = {"f32": 1e-5, "f16": 1e-3}


@pytest.fixture(scope="module")
def case(amcl):
    m = S.make_map(61, size_m=(12.0, 10.0, 3.0), n_boxes=15)
    G = amcl.Grid3d()
    G.buildGridMap(m.points, m.min, m.max, m.res, S.SENSOR_DEV)
    d, p = G.read_cells()
    g = O.GridData(m.min, m.max, m.res, m.dims, p, d)
    pose = S.free_pose(m, 62, height=1.2, clearance=0.4)
    scan = S.ray_cast(m, pose, n_max=4000, max_range=10.0, seed=63)
    poses = S.particles_around(pose, 3000, 64)[:, :4]
    _, cells = O.cloud_weights(g, poses, scan, 0.0, 0.0, yaw_trig=1, cells=True)
    p64 = p.astype(np.float64)
    exact = np.zeros(poses.shape[0])
    for i in range(poses.shape[0]):
        c = cells[i][cells[i] >= 0]
        exact[i] = p64[c].mean() if c.size > 10 else 0.0
    return G, poses, scan, exact


def rel_err(got, exact):
    mask = exact > 0
    return np.abs(got[mask].astype(np.float64) - exact[mask]) / exact[mask]


@pytest.mark.parametrize("storage", ["f32", "f16", "u8"])
@pytest.mark.parametrize("cloud_sum", [0, 1])
def test_weights_vs_fp64(amcl, case, storage, cloud_sum):
    G, poses, scan, exact = case
    G.set_storage(storage)
    try:
        pf = amcl.ParticleFilter(seed=1)
        pf.set_option(1, cloud_sum)
        p7 = np.zeros((poses.shape[0], 7), np.float32)
        p7[:, :4] = poses
        pf.set_particles(p7)
        pf.update(G, scan, np.zeros((0, 4), np.float32), 1.0, 0.1, 0.0, 0.0)
        # the update normalises wp by the exact sum: compare with the normalised FP64 weights
        # (per-particle relative errors e_i give normalised errors within 2 max e_i)
        got = pf.particles()[:, 5].astype(np.float64)
        err = rel_err(got, exact / exact.sum())
        if storage in TOL:
            assert err.max() < 2 * TOL[storage], (storage, cloud_sum, err.max())
        else:
            assert err.max() < 4e-2  # uint8: scale/2 per cell, max prob / 510
        print(f"storage {storage} sum {cloud_sum}: max rel err vs FP64 {err.max():.3e}, mean {err.mean():.3e}")
    finally:
        G.set_storage("f32")


def test_cloud_weights_storage_direct(amcl, case):
    """computeCloudWeight itself per storage (no normalisation in between)."""
    G, poses, scan, exact = case
    res = {}
    for storage in ("f32", "f16", "u8"):
        G.set_storage(storage)
        res[storage] = rel_err(G.computeCloudWeights(poses, scan), exact).max()
    G.set_storage("f32")
    assert res["f32"] < 1e-5 and res["f16"] < 1e-3 and res["u8"] < 2e-2, res
