"""The C++ drop-in classes (amcl3d_gb300/cpp: amcl3d::Grid3d, amcl3d::ParticleFilter
with the reference's signatures) driven the way amcl3d::Node drives them, checked
against the oracle.  Compiles tests/native/dropin_check.cpp against the stand-in
ROS/PCL/octomap headers and links the drop-in and the CUDA library."""

import subprocess

import numpy as np
import pytest

import oracle as O
from conftest import ROOT

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dropin_bin(native_lib, tmp_path_factory):
    from amcl3d_gb300 import build

    so = build.build_dropin()
    exe = tmp_path_factory.mktemp("dropin") / "dropin_check"
    subprocess.run(["g++", "-std=c++14", "-O2", "-ffp-contract=off", f"-I{build.CPP}", f"-I{build.INCLUDE}",
                    f"-I{build.SHIM}", "-o", str(exe), str(ROOT / "tests" / "native" / "dropin_check.cpp"),
                    f"-L{build.LIB}", "-lamcl3d_dropin", "-lamcl3d_gpu", f"-Wl,-rpath,{build.LIB}"],
                   check=True, capture_output=True)
    assert so.exists()
    return exe


def test_dropin_like_the_node(dropin_bin, ref_small, tmp_path):
    b = ref_small["bounds"]
    mn, mx, res = tuple(b[:3]), tuple(b[3:6]), float(b[6])
    map_path = tmp_path / "map.bt"
    O.write_points_map(map_path, ref_small["points"], mn, mx, res)
    scan = np.ascontiguousarray(ref_small["scan"], np.float32)
    scan.tofile(tmp_path / "scan.f32")
    ranges = np.ascontiguousarray(ref_small["ranges"], np.float32)
    ranges.tofile(tmp_path / "ranges.f32")
    r = subprocess.run([str(dropin_bin), str(map_path), str(tmp_path / "scan.f32"), str(tmp_path / "ranges.f32"),
                        str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out = {ln.split()[0]: ln.split()[1:] for ln in r.stdout.splitlines() if ln.strip()}
    assert out["open_short"] == ["0"] and out["open_missing"] == ["0"]  # Grid3dTest.cpp:29-42
    assert float(out["weight_unopened"][0]) == 0.0
    assert out["open"] == ["1"] and out["open_cached"] == ["1"]
    assert (tmp_path / "map.grid").exists()  # the .grid cache next to the map
    dims = tuple(int(v) for v in ref_small["dims"])
    assert out["slice"] == ["1", str(dims[0]), str(dims[1]), str(dims[0] + dims[1] * dims[0])]
    assert out["mapcloud"] == ["1", str(ref_small["points"].shape[0])]
    assert out["into"] == ["1", "0"]
    assert out["initialized_before"] == ["0"]
    im = [float(v) for v in out["init_mean"][:4]]
    assert abs(im[0] - 2.5) < 0.01 and abs(im[3] - 0.3) < 0.02 and out["init_mean"][4] == "1"

    before = np.fromfile(tmp_path / "before_update.bin", np.float32).reshape(-1, 7)
    after = np.fromfile(tmp_path / "after_update.bin", np.float32).reshape(-1, 7)
    d, p = O.compute_grid(ref_small["points"], mn, mx, res, 0.05, exp_mode=1)
    g = O.GridData(mn, mx, res, dims, p.ravel(), d.ravel())
    exp, m32, _, _ = O.update_exact(before, g, scan, ranges, 0.5, 0.1, 0.0, 0.0)
    np.testing.assert_array_equal(after, exp)
    np.testing.assert_array_equal(np.array([float(v) for v in out["mean"]], np.float32), m32)
    assert out["poses"][0] == "600"
    w = O.cloud_weights(g, [[2.5, 2.0, 1.2, 0.3]], scan, 0.0, 0.0, yaw_trig=1)[0]
    assert np.float32(float(out["weight"][0])) == w
    assert float(out["ranges_only_mean"][0]) == 0.0
    # the scan filter the node runs first (Node.cpp:130-137), against the oracle's VoxelGrid
    down, ovf = O.voxel_downsample(scan, 0.1)
    assert not ovf and out["voxel"] == [str(down.shape[0])] * 2
    got = np.fromfile(tmp_path / "voxel.bin", np.float32).reshape(-1, 3)
    np.testing.assert_array_equal(got, down[:, :3])
