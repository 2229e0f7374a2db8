"""The library's octomap reader (amcl_octomap_read: openOcTree + computePointCloud,
PointCloudTools.cpp:26-82, from octomap's published file formats) against the
oracle's Python restatement, on .bt and .ot maps written from spec: occupied leaf
centres in leaf-iterator order, metric bounds over all leaves, node counts, pruned
(coarser) leaves, free leaves; the error cases of PointCloudToolsTest.cpp:64-101
(missing file, wrong .bt/.ot, unknown extension) and the empty tree; and the
bounds PointCloudToolsTest.cpp:40-53 expects of the reference's test map, rebuilt
from that map's published point cloud (mappointcloud_msg.bin).  Host code only: no GPU."""

import numpy as np
import pytest

from oracle import octomap as OM


@pytest.fixture(scope="module")
def lib(native_lib):
    from amcl3d_gb300 import _native as N
    from amcl3d_gb300 import filter as F

    return N, F


def _random_leaves(seed, n_occ=3000, n_free=2000, n_coarse=40, res=0.1):
    rng = np.random.default_rng(seed)
    leaves = {}
    pts = rng.uniform(-30, 30, (n_occ, 3))
    leaves.update(OM.leaves_from_points(pts, res, True))
    leaves.update({k: v for k, v in OM.leaves_from_points(rng.uniform(-30, 30, (n_free, 3)), res, False).items()
                   if k not in leaves})
    # coarse (pruned) leaves at depths 12-15 in a far corner, both states
    for j in range(n_coarse):
        d = int(rng.integers(12, 16))
        c = rng.uniform(40, 60, 3)
        key = tuple(OM.coord_to_key(float(v), res) for v in c)
        leaves[(key, d)] = bool(j % 2)
    # drop full-depth leaves that fall inside a coarse one (a leaf cannot hold leaves)
    coarse = [(k, d) for (k, d) in leaves if d < OM.DEPTH]
    for (k, d) in list(leaves):
        if d == OM.DEPTH:
            for (ck, cd) in coarse:
                if all((k[a] >> (OM.DEPTH - cd)) == (ck[a] >> (OM.DEPTH - cd)) for a in range(3)):
                    leaves.pop((k, d), None)
                    break
    # coarse leaves inside other coarse leaves
    for (k, d) in sorted(coarse, key=lambda x: x[1]):
        for (k2, d2) in coarse:
            if (k2, d2) != (k, d) and d2 < d and (k, d) in leaves and \
                    all((k[a] >> (OM.DEPTH - d2)) == (k2[a] >> (OM.DEPTH - d2)) for a in range(3)):
                leaves.pop((k, d), None)
    return leaves


@pytest.mark.parametrize("seed", [1, 2])
@pytest.mark.parametrize("fmt", ["bt", "ot"])
def test_reader_matches_oracle(lib, tmp_path, seed, fmt):
    N, F = lib
    res = 0.1 if seed == 1 else 0.05
    leaves = _random_leaves(seed, res=res)
    path = tmp_path / f"map.{fmt}"
    n_nodes = (OM.write_bt if fmt == "bt" else OM.write_ot)(path, leaves, res)
    exp = OM.read(path)
    got = F.read_octomap(path)
    assert got["nodes"] == exp["nodes"] == n_nodes
    assert got["res"] == exp["res"] == res
    assert got["min"] == exp["min"] and got["max"] == exp["max"]
    np.testing.assert_array_equal(got["points"][:, :3], exp["points"])
    assert (got["points"][:, 3] == 1.0).all()
    assert got["points"].shape[0] == sum(1 for v in leaves.values() if v)


def test_bt_and_ot_agree(lib, tmp_path):
    N, F = lib
    leaves = _random_leaves(3)
    OM.write_bt(tmp_path / "m.bt", leaves, 0.1)
    OM.write_ot(tmp_path / "m.ot", leaves, 0.1)
    a, b = F.read_octomap(tmp_path / "m.bt"), F.read_octomap(tmp_path / "m.ot")
    np.testing.assert_array_equal(a["points"], b["points"])
    assert a["min"] == b["min"] and a["max"] == b["max"] and a["nodes"] == b["nodes"]


def _expect_error(F, N, path, status):
    with pytest.raises(N.AmclError) as e:
        F.read_octomap(path)
    assert e.value.status == status, str(e.value)
    with pytest.raises(OM.OctomapError):
        OM.read(path)


def test_error_cases(lib, tmp_path):
    N, F = lib
    EIO, EINVAL = 6, 1
    _expect_error(F, N, tmp_path / "unknown_file.bt", EIO)  # PointCloudToolsTest.cpp:64-75
    _expect_error(F, N, tmp_path / "unknown_file.ot", EIO)
    for name in ("mapfile_wrong.bt", "mapfile_wrong.ot", "mapfile_unknown_extension.unk"):  # :77-101 (empty files)
        (tmp_path / name).write_bytes(b"")
        _expect_error(F, N, tmp_path / name, EINVAL)
    leaves = _random_leaves(4, n_occ=50, n_free=0, n_coarse=0)
    good = tmp_path / "good.bt"
    OM.write_bt(good, leaves, 0.1)
    body = good.read_bytes()
    (tmp_path / "trunc.bt").write_bytes(body[:-3])
    _expect_error(F, N, tmp_path / "trunc.bt", EINVAL)
    (tmp_path / "color.bt").write_bytes(body.replace(b"id OcTree", b"id ColorOcTree"))
    _expect_error(F, N, tmp_path / "color.bt", EINVAL)
    (tmp_path / "size.bt").write_bytes(body.replace(b"size ", b"size 1"))
    _expect_error(F, N, tmp_path / "size.bt", EINVAL)
    (tmp_path / "nores.bt").write_bytes(body.replace(b"res 0.1", b"res 0"))
    _expect_error(F, N, tmp_path / "nores.bt", EINVAL)
    (tmp_path / "empty.bt").write_bytes(f"{OM.BT_HEADER}\nid OcTree\nsize 1\nres 0.1\ndata\n".encode() + b"\0\0")
    _expect_error(F, N, tmp_path / "empty.bt", EINVAL)  # computePointCloud: size <= 1 is empty
    # the deprecated id "1", comments and unknown keywords in the header are accepted
    (tmp_path / "old.bt").write_bytes(body.replace(b"id OcTree", b"id 1\nfoo bar baz\n# note"))
    assert F.read_octomap(tmp_path / "old.bt")["points"].shape[0] == 50


def test_fixture_map_bounds(lib, refdata, tmp_path):
    """The reference's test map as a .bt built from its published occupied-point cloud:
    179,551 occupied leaves and the metric bounds PointCloudToolsTest.cpp:40-53 asserts
    (ASSERT_DOUBLE_EQ: within 4 ulps)."""
    N, F = lib
    lo = np.array([-17.35, -9.5, -1.4])
    hi = np.array([8.75, 9.7, 6.25])
    # the fixture cloud is in the map frame shifted by the metric minimum
    centres = refdata["map_points"].astype(np.float64) + lo
    # a leaf at depth d has its centre at an odd multiple of res * 2^(16-d) / 2 on every
    # axis: the fixture holds 136 pruned depth-15 leaves beside the full-depth ones
    t = np.round(2 * centres / 0.05).astype(np.int64)
    assert np.abs(2 * centres / 0.05 - t).max() < 1e-3
    v2 = np.zeros_like(t)
    odd = t.copy()
    while ((odd % 2 == 0) & (odd != 0)).any():
        m = (odd % 2 == 0) & (odd != 0)
        v2[m] += 1
        odd[m] //= 2
    assert (v2 == v2[:, :1]).all()
    depth = OM.DEPTH - v2[:, 0]
    assert sorted(np.unique(depth)) == [15, 16] and (depth == 15).sum() == 136
    leaves = {(tuple(OM.coord_to_key(float(c), 0.05) for c in centres[i]), int(depth[i])): True
              for i in range(centres.shape[0])}
    path = tmp_path / "mapfile_complete.bt"
    OM.write_bt(path, leaves, 0.05)
    got = F.read_octomap(path)
    assert got["points"].shape[0] == 179551
    assert got["res"] == 0.05
    for a in range(3):
        assert abs(got["min"][a] - lo[a]) <= 4 * np.spacing(abs(lo[a]))
        assert abs(got["max"][a] - hi[a]) <= 4 * np.spacing(abs(hi[a]))
    # the leaf centres are the fixture points, shifted back, to float precision
    mine = np.sort(got["points"][:, :3].astype(np.float64) - lo, axis=0)
    np.testing.assert_allclose(mine, np.sort(refdata["map_points"].astype(np.float64), axis=0), atol=2e-6)
