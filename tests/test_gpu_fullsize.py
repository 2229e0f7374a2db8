"""Parity at the large single-filter size (2000x2000x400-cell warehouse, 200,000
particles, ~19,400-point scan), where the oracle cannot run everything: the GPU
distance field equals the oracle's computeGrid on a 4x4x2 m sub-block around the
robot (the comparison the large configuration names), 64 sampled particles' cloud
weights equal the oracle's on the GPU-built cells, and size-independent properties
of the full update and resample hold (normalised weights summing to one, resample
indices sorted and in range, mean inside the particle cloud, variances >= 0)."""

import numpy as np
import pytest

import bench
import oracle as O
from amcl3d_gb300 import synth as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def warehouse(amcl):
    cfg = bench.CONFIGS["warehouse"]
    occ, info, scans, ranges, odos, parts = bench.make_workload(cfg, 1000)
    G = amcl.Grid3d()
    G.buildGridMap(occ, info["min"], info["max"], info["res"], S.SENSOR_DEV)
    return G, occ, info, scans, ranges, parts


def test_distance_field_subblock(warehouse):
    G, occ, info, scans, ranges, parts = warehouse
    sx, sy, sz = info["dims"]
    # 80 x 80 x 40 cells (4 x 4 x 2 m) around the particle cloud's centre
    c = [int((float(np.mean(parts[:, a])) - info["min"][a]) / info["res"]) for a in range(3)]
    lo = (max(0, c[0] - 40), max(0, c[1] - 40), max(0, c[2] - 20))
    hi = (min(sx, lo[0] + 80), min(sy, lo[1] + 80), min(sz, lo[2] + 40))
    d_ref, p_ref = O.compute_grid(occ, info["min"], info["max"], info["res"], S.SENSOR_DEV, lo=lo, hi=hi,
                                  exp_mode=1)
    d_gpu = np.empty_like(d_ref)
    p_gpu = np.empty_like(p_ref)
    for z in range(lo[2], hi[2]):
        for y in range(lo[1], hi[1]):
            first = (z * sy + y) * sx + lo[0]
            d, p = G.read_cells(first, hi[0] - lo[0])
            d_gpu[z - lo[2], y - lo[1]] = d
            p_gpu[z - lo[2], y - lo[1]] = p
    np.testing.assert_array_equal(d_gpu, d_ref)
    np.testing.assert_array_equal(p_gpu, p_ref)


@pytest.fixture(scope="module")
def warehouse_cells(warehouse):
    """The warehouse's probabilities read back: the oracle's grid."""
    G, occ, info, scans, ranges, parts = warehouse
    cells = int(np.prod(info["dims"]))
    prob = np.empty(cells, np.float32)
    step = 1 << 28
    for first in range(0, cells, step):
        prob[first:first + min(step, cells - first)] = G.read_cells(first, min(step, cells - first))[1]
    return O.GridData(info["min"], info["max"], info["res"], info["dims"], prob)


def test_full_update_sample_and_properties(amcl, warehouse, warehouse_cells):
    G, occ, info, scans, ranges, parts = warehouse
    pf = amcl.ParticleFilter(seed=77)
    pf.set_particles(parts)
    pf.update(G, scans[0], ranges[0], 0.5, 0.1, 0.0, 0.0)
    after = pf.particles()
    # a sample of particles' cloud weights against the oracle on the GPU-built cells
    g = warehouse_cells
    idx = np.random.default_rng(5).choice(parts.shape[0], 64, replace=False)
    want = O.cloud_weights(g, parts[idx, :4], scans[0], 0.0, 0.0, yaw_trig=1)
    got = G.computeCloudWeights(parts[idx, :4], scans[0])
    np.testing.assert_array_equal(got, want)
    # size-independent properties of the full update
    w = after[:, 4].astype(np.float64)
    assert abs(w.sum() - 1.0) < parts.shape[0] * 2.0**-24
    mean, var = pf.mean_var()
    for a in range(3):
        assert after[:, a].min() <= mean[a] <= after[:, a].max()
    assert (np.asarray(var) >= 0).all()
    pf.resample(0.37)
    ri = pf.resample_index()
    assert ri.shape[0] == parts.shape[0] and (np.diff(ri) >= 0).all()
    assert ri.min() >= 0 and ri.max() < parts.shape[0]
    np.testing.assert_array_equal(ri, O.resample_exact(after[:, 4], 0.37))


@pytest.mark.parametrize("storage,tol", [("f32", 1e-5), ("f16", 1e-3), ("u8", 4e-2)])
def test_storage_weights_vs_fp64_at_full_size(amcl, warehouse, warehouse_cells, storage, tol):
    """The reduced-precision grids at the large configuration's size: 64 sampled
    particles on the 1.6 G-cell warehouse with the ~19.4k-point scan, per cell storage,
    against the FP64 oracle (the mean in double of the FP64 probabilities of the cells
    the reference's arithmetic selects).  With the compensated cloud sum
    (AMCL_OPT_CLOUD_SUM=1): FP32 within 1e-5 and FP16 within 1e-3 relative (the stated
    tolerances), uint8 within its quantisation (max prob / 510 per cell).  The
    reference's own float running sum over this many points is itself further from
    FP64 (printed, and bounded by 1e-3), which is why the compensated sum exists."""
    G, occ, info, scans, ranges, parts = warehouse
    g = warehouse_cells
    idx = np.random.default_rng(11).choice(parts.shape[0], 64, replace=False)
    sample = parts[idx].copy()
    _, cells = O.cloud_weights(g, sample[:, :4], scans[1], 0.0, 0.0, yaw_trig=1, cells=True)
    p64 = g.prob.astype(np.float64)
    exact = np.array([p64[c[c >= 0]].mean() if (c >= 0).sum() > 10 else 0.0 for c in cells])
    mask = exact > 0
    assert mask.sum() >= 32
    G.set_storage(storage)
    try:
        errs = {}
        for cloud_sum in (0, 1):
            pf = amcl.ParticleFilter(seed=1)
            pf.set_option(1, cloud_sum)
            pf.set_particles(sample)
            pf.update(G, scans[1], np.zeros((0, 4), np.float32), 1.0, 0.1, 0.0, 0.0)
            # wp is normalised by the exact sum of the sample's weights: compare with the
            # normalised FP64 weights (per-particle errors e_i give normalised errors
            # within 2 max e_i)
            got = pf.particles()[:, 5].astype(np.float64)
            want = exact / exact.sum()
            errs[cloud_sum] = np.abs(got[mask] - want[mask]) / want[mask]
    finally:
        G.set_storage("f32")
    print(f"{storage}: max rel err vs FP64, running sum {errs[0].max():.3e}, compensated {errs[1].max():.3e}")
    assert errs[1].max() < 2 * tol, (storage, errs[1].max())
    assert errs[0].max() < max(2 * tol, 2e-3), (storage, errs[0].max())
