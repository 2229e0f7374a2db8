"""Grid3d::open on the GPU library (amcl_grid_open, Grid3d.cpp:25-78): an octomap .bt
or .ot map read by the library, its distance field built on the device and written
to the .grid file beside the map, which the next open loads instead; the cells equal
those of a grid built from the oracle's reading of the same file."""

import numpy as np
import pytest

from amcl3d_gb300 import synth as S
from oracle import octomap as OM

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fmt", ["bt", "ot"])
def test_grid_open_build_cache_and_mismatch(amcl, tmp_path, fmt):
    m = S.make_map(77, size_m=(6.0, 5.0, 3.0), n_boxes=6)
    rng = np.random.default_rng(78)
    leaves = OM.leaves_from_points(rng.uniform(-0.5, 6.5, (300, 3)), m.res, False)
    leaves.update(OM.leaves_from_points(m.points, m.res, True))
    path = tmp_path / f"map.{fmt}"
    (OM.write_bt if fmt == "bt" else OM.write_ot)(path, leaves, m.res)
    info = OM.read(path)

    G = amcl.Grid3d()
    assert G.open(path, 0.05), G.last_error
    assert (tmp_path / "map.grid").exists()
    ref = amcl.Grid3d()
    ref.buildGridMap(info["points"], info["min"], info["max"], info["res"], 0.05)
    d0, p0 = ref.read_cells()
    d1, p1 = G.read_cells()
    np.testing.assert_array_equal(d1, d0)
    np.testing.assert_array_equal(p1, p0)
    gi = G.info()
    assert tuple(gi["min"]) == info["min"] and tuple(gi["max"]) == info["max"]

    mtime = (tmp_path / "map.grid").stat().st_mtime_ns
    C = amcl.Grid3d()
    assert C.open(path, 0.05)  # from the cache
    assert (tmp_path / "map.grid").stat().st_mtime_ns == mtime
    np.testing.assert_array_equal(C.read_cells()[1], p0)

    D = amcl.Grid3d()
    assert D.open(path, 0.1)  # sensor_dev differs from the cache: rebuilt and rewritten
    ref.buildGridMap(info["points"], info["min"], info["max"], info["res"], 0.1)
    np.testing.assert_array_equal(D.read_cells()[1], ref.read_cells()[1])


def test_grid_open_errors(amcl, tmp_path):
    G = amcl.Grid3d()
    assert not G.open(tmp_path / "missing.bt", 0.05)
    (tmp_path / "wrong.bt").write_bytes(b"")
    assert not G.open(tmp_path / "wrong.bt", 0.05)
    assert "header" in G.last_error or "first line" in G.last_error
    assert G.computeCloudWeight(np.zeros((5, 4), np.float32), 0, 0, 0, 0, 0, 0) == 0.0
