"""Generates the committed golden fixtures under tests/golden/.

Run where the reference tree is readable (a `reference` checkout beside this
repository by default, override with AMCL3D_REF_ROOT) after `make -C oracle all ref`:

    python tests/golden/make_golden.py

Outputs:
* refdata.npz   - the reference's own test fixtures decoded from their ROS
                  serialisation (amcl3d/tests/data): the 25,809-point scan of
                  grid_info.bin (computeCloudWeightTest, Grid3dTest.cpp:120-169),
                  the 179,551 map points of mappointcloud_msg.bin and the
                  522x384 z=1.0 occupancy slice of nav_msg.bin.
* ref_small.npz - outputs of the reference filter core compiled verbatim
                  (oracle/_ref) on a seeded synthetic case: grid cells, cloud
                  weights, one update, one resample.
* ref_kat.json  - the computeCloudWeightTest known answer recomputed on the grid
                  rebuilt from mappointcloud_msg.bin, plus the slice agreement.
"""

from __future__ import annotations

import hashlib
import json
import os
import struct
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import oracle as O  # noqa: E402
from amcl3d_gb300 import synth as S  # noqa: E402

# the reference checkout: AMCL3D_REF_ROOT, else a `reference` directory beside this repository
REF_ROOT = Path(os.environ.get("AMCL3D_REF_ROOT", str(ROOT.parent / "reference")))
DATA = REF_ROOT / "amcl3d" / "tests" / "data"


def _skip_header(b: bytes, o: int) -> int:
    _seq, _s, _ns, ln = struct.unpack_from("<IIII", b, o)
    return o + 16 + ln


def decode_pose_array(path: Path) -> np.ndarray:
    b = path.read_bytes()
    o = _skip_header(b, 0)
    (n,) = struct.unpack_from("<I", b, o)
    o += 4
    return np.frombuffer(b, dtype="<f8", count=n * 7, offset=o).reshape(n, 7).copy()


def decode_pointcloud2(path: Path) -> np.ndarray:
    b = path.read_bytes()
    o = _skip_header(b, 0)
    _h, _w, nf = struct.unpack_from("<III", b, o)
    o += 12
    for _ in range(nf):
        (ln,) = struct.unpack_from("<I", b, o)
        o += 4 + ln + 9
    _be, ps, _rs, dl = struct.unpack_from("<BIII", b, o)
    o += 13
    return np.frombuffer(b, dtype=np.uint8, count=dl, offset=o).view("<f4").reshape(-1, ps // 4)[:, :3].copy()


def decode_occupancy_grid(path: Path):
    b = path.read_bytes()
    o = _skip_header(b, 0)
    _ms, _mns, res, w, h = struct.unpack_from("<IIfII", b, o)
    o += 20
    origin = struct.unpack_from("<7d", b, o)
    o += 56
    (n,) = struct.unpack_from("<I", b, o)
    o += 4
    return np.frombuffer(b, dtype=np.int8, count=n, offset=o).copy(), res, w, h, origin


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main() -> None:
    scan = decode_pose_array(DATA / "grid_info.bin")[:, :3].astype(np.float32)
    cloud = decode_pointcloud2(DATA / "mappointcloud_msg.bin").astype(np.float32)
    nav, res, w, h, origin = decode_occupancy_grid(DATA / "nav_msg.bin")
    np.savez_compressed(HERE / "refdata.npz", scan=scan, map_points=cloud, nav_slice=nav,
                        nav_meta=np.array([res, w, h, origin[2]], np.float64))

    # Seeded synthetic case through the verbatim reference.
    m = S.make_map(1, size_m=(6.0, 5.0, 3.0), res=0.05, n_boxes=6)
    rg = O.RefGrid(m.points, m.min, m.max, m.res, S.SENSOR_DEV)
    assert rg.ok
    d_ref, p_ref = rg.cells()
    pose = S.free_pose(m, 3)
    pscan = S.ray_cast(m, pose, n_max=1000, max_range=8.0, seed=2)
    parts = S.particles_around(pose, 64, 5)
    parts[60, :3] = (-1.0, 1.0, 1.0)  # out of the map
    parts[61, :3] = (1.0, 1.0, 5.0)  # out of the map (z)
    ranges = S.beacons(m, pose, 3, seed=4)
    wts = {}
    for tag, (roll, pitch) in {"rp0": (0.0, 0.0), "rp1": (0.02, -0.03)}.items():
        wts[tag] = np.array([rg.cloud_weight(pscan, *parts[i, :3], roll, pitch, parts[i, 3]) for i in range(64)],
                            np.float32)
    rf = O.RefFilter(7)
    rf.set_particles(parts)
    rf.update(rg, pscan, ranges, 0.5, 0.1, 0.0, 0.0)
    upd = rf.particles()
    mean = rf.mean()
    u = rf.peek_uniform()
    rf.resample()
    res_p = rf.particles()
    sub = (slice(10, 30), slice(20, 60), slice(30, 80))  # z, y, x
    np.savez_compressed(
        HERE / "ref_small.npz", points=m.points, bounds=np.array([*m.min, *m.max, m.res], np.float64),
        dims=np.array(m.dims, np.int64), dist_sub=d_ref.reshape(m.dims[::-1])[sub],
        prob_sub=p_ref.reshape(m.dims[::-1])[sub], sub=np.array([10, 30, 20, 60, 30, 80], np.int64),
        scan=pscan, particles=parts, ranges=ranges, w_rp0=wts["rp0"], w_rp1=wts["rp1"], updated=upd, mean=mean,
        u=np.float32(u), resampled=res_p)
    meta = {"dist_sha256": sha(d_ref), "prob_sha256": sha(p_ref)}
    rg.close()
    rf.close()

    # KAT of Grid3dTest.cpp:128-168 on the grid rebuilt from the map-cloud fixture
    # (the shipped map file is not in the reference tree).
    mn, mx, r = (0.0, 0.0, 0.0), (26.1, 19.2, 7.65), 0.05
    size = O.grid_sizes(mn, mx, r)
    dist, prob = O.compute_grid(cloud, mn, mx, r, S.SENSOR_DEV, exp_mode=0)
    g = O.GridData(mn, mx, r, size, prob.ravel(), dist.ravel())
    kat = float(O.cloud_weights(g, [[20.017967, 10.140815, 3.372801, 0.166781]], scan, 0.0, 0.0, yaw_trig=0)[0])
    layer = prob.reshape(size[2], size[1], size[0])[20].ravel()
    mxp = max(np.float32(layer.max()), np.float32(1e-6))
    sl = (layer * (np.float32(100.0) / mxp)).astype(np.float32).astype(np.int8)
    meta.update({
        "kat_expected": 3.8109049797058105,
        "kat_on_rebuilt_grid": kat,
        "fixture_grid_size": list(size),
        "fixture_dist_sha256": sha(dist.ravel()),
        "fixture_prob_sha256": sha(prob.ravel()),
        "slice_match_fraction": float((sl == nav).mean()),
        "slice_mismatch": int((sl != nav).sum()),
    })
    (HERE / "ref_kat.json").write_text(json.dumps(meta, indent=1) + "\n")
    print(json.dumps(meta, indent=1))


if __name__ == "__main__":
    main()
