"""Seeded synthetic workloads of the benchmark configurations.

The reference publishes no dataset for its benchmarks, so maps, scans, particle
sets, beacons and odometry are generated here from a seed with the shapes the
configurations name:

* map: an axis-aligned room (floor, ceiling and four walls one voxel thick) with
  axis-aligned cuboid obstacles standing on the floor; the occupied voxels are
  the room shell and every cuboid's surface voxels, served as voxel centres
  ``min + (i + 0.5) * res`` (what an octomap's finest leaves give);
* scan: ray-cast ``elevations x azimuths`` beams from the true pose through the
  voxel occupancy, Gaussian range noise, first N hits kept, expressed in the
  sensor frame (yaw-only pose, as the node applies roll/pitch separately);
* particles: uniform around the true pose; beacons: fixed ceiling corners with
  noisy ranges; odometry: a forward step with Gaussian noise.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class MapSpec:
    size_m: tuple
    res: float
    occ: np.ndarray  # bool, shape (sz, sy, sx)
    points: np.ndarray  # (M, 3) float32 voxel centres
    min: tuple = (0.0, 0.0, 0.0)
    max: tuple = field(default=None)

    @property
    def dims(self):
        return tuple(int(v) for v in self.occ.shape[::-1])


def make_map(seed: int, size_m=(20.0, 20.0, 5.0), res=0.05, n_boxes=40, box_range=(0.3, 3.0),
             max_box_height=None) -> MapSpec:
    rng = np.random.default_rng(seed)
    sx, sy, sz = (int(round(s / res)) for s in size_m)
    occ = np.zeros((sz, sy, sx), dtype=bool)
    # room shell
    occ[0, :, :] = True
    occ[-1, :, :] = True
    occ[:, 0, :] = True
    occ[:, -1, :] = True
    occ[:, :, 0] = True
    occ[:, :, -1] = True
    hmax = size_m[2] if max_box_height is None else max_box_height
    for _ in range(n_boxes):
        ext = rng.uniform(box_range[0], box_range[1], size=3)
        ext[2] = min(ext[2], hmax)
        nx, ny, nz = (max(1, int(round(e / res))) for e in ext)
        nx, ny, nz = min(nx, sx - 2), min(ny, sy - 2), min(nz, sz - 2)
        x0 = int(rng.integers(1, sx - nx))
        y0 = int(rng.integers(1, sy - ny))
        z0 = 1
        x1, y1, z1 = x0 + nx, y0 + ny, z0 + nz
        occ[z0:z1, y0:y1, x0] = True
        occ[z0:z1, y0:y1, x1 - 1] = True
        occ[z0:z1, y0, x0:x1] = True
        occ[z0:z1, y1 - 1, x0:x1] = True
        occ[z0, y0:y1, x0:x1] = True
        occ[z1 - 1, y0:y1, x0:x1] = True
    iz, iy, ix = np.nonzero(occ)
    pts = np.empty((ix.shape[0], 3), np.float32)
    pts[:, 0] = (0.0 + (ix.astype(np.float64) + 0.5) * res).astype(np.float32)
    pts[:, 1] = (0.0 + (iy.astype(np.float64) + 0.5) * res).astype(np.float32)
    pts[:, 2] = (0.0 + (iz.astype(np.float64) + 0.5) * res).astype(np.float32)
    return MapSpec(size_m=tuple(size_m), res=res, occ=occ, points=pts, min=(0.0, 0.0, 0.0),
                   max=tuple(float(v) for v in size_m))


def free_pose(m: MapSpec, seed: int, height=1.5, clearance=0.6):
    """A pose at `height` whose surrounding (2*clearance)^3 cube is free."""
    rng = np.random.default_rng(seed)
    c = max(1, int(round(clearance / m.res)))
    mx = min(2.0, m.size_m[0] / 4)
    my = min(2.0, m.size_m[1] / 4)
    for _ in range(10000):
        x = rng.uniform(mx, m.size_m[0] - mx)
        y = rng.uniform(my, m.size_m[1] - my)
        z = min(height, m.size_m[2] - 1.0)
        ix, iy, iz = int(x / m.res), int(y / m.res), int(z / m.res)
        blk = m.occ[max(iz - c, 0):iz + c, max(iy - c, 0):iy + c, max(ix - c, 0):ix + c]
        if not blk.any():
            return np.array([x, y, z, rng.uniform(-math.pi, math.pi)], np.float64)
    raise RuntimeError("no free pose found")


def ray_cast(m: MapSpec, pose, n_elev=32, n_azim=32, elev_deg=(-25.0, 25.0), max_range=15.0, noise=0.02,
             n_max=1000, seed=0) -> np.ndarray:
    """Scan points (N, 4) float32 (x, y, z, 0) in the sensor frame."""
    rng = np.random.default_rng(seed)
    el = np.deg2rad(np.linspace(elev_deg[0], elev_deg[1], n_elev))
    az = np.linspace(-math.pi, math.pi, n_azim, endpoint=False)
    E, A = np.meshgrid(el, az, indexing="ij")
    d_s = np.stack([np.cos(E) * np.cos(A), np.cos(E) * np.sin(A), np.sin(E)], -1).reshape(-1, 3)
    cy, sy = math.cos(pose[3]), math.sin(pose[3])
    d_w = np.stack([cy * d_s[:, 0] - sy * d_s[:, 1], sy * d_s[:, 0] + cy * d_s[:, 1], d_s[:, 2]], -1)
    o = np.asarray(pose[:3], np.float64)
    step = m.res * 0.5
    nsteps = int(max_range / step)
    hit_t = np.full(d_w.shape[0], np.inf)
    alive = np.ones(d_w.shape[0], bool)
    sz, sy_, sx = m.occ.shape
    t = step
    for _ in range(nsteps):
        idx = np.nonzero(alive)[0]
        if idx.size == 0:
            break
        p = o + t * d_w[idx]
        ix = np.floor(p[:, 0] / m.res).astype(np.int64)
        iy = np.floor(p[:, 1] / m.res).astype(np.int64)
        iz = np.floor(p[:, 2] / m.res).astype(np.int64)
        inside = (ix >= 0) & (iy >= 0) & (iz >= 0) & (ix < sx) & (iy < sy_) & (iz < sz)
        hit = np.zeros(idx.size, bool)
        hit[inside] = m.occ[iz[inside], iy[inside], ix[inside]]
        hit_t[idx[hit]] = t
        alive[idx[hit | ~inside]] = False
        t += step
    ok = np.isfinite(hit_t)
    r = hit_t[ok] + rng.normal(0.0, noise, ok.sum())
    pts = d_s[ok] * r[:, None]
    pts = pts[:n_max]
    out = np.zeros((pts.shape[0], 4), np.float32)
    out[:, :3] = pts.astype(np.float32)
    return out


def particles_around(pose, n, seed, dxy=0.5, dz=0.1, da=0.1) -> np.ndarray:
    rng = np.random.default_rng(seed)
    p = np.zeros((n, 7), np.float32)
    p[:, 0] = pose[0] + rng.uniform(-dxy, dxy, n)
    p[:, 1] = pose[1] + rng.uniform(-dxy, dxy, n)
    p[:, 2] = pose[2] + rng.uniform(-dz, dz, n)
    p[:, 3] = pose[3] + rng.uniform(-da, da, n)
    p[:, 4] = 1.0 / n
    return p


def beacons(m: MapSpec, pose, n=3, sigma=0.1, seed=0) -> np.ndarray:
    """(n, 4) float32 ranges (r, ax, ay, az) from fixed anchors near the ceiling."""
    rng = np.random.default_rng(seed)
    X, Y, Z = m.size_m
    anchors = [(0.5, 0.5, Z - 0.5), (X - 0.5, 0.5, Z - 0.5), (0.5, Y - 0.5, Z - 0.5), (X - 0.5, Y - 0.5, Z - 0.5),
               (X / 2, 0.5, Z - 0.5), (X / 2, Y - 0.5, Z - 0.5)]
    out = np.zeros((n, 4), np.float32)
    for i in range(n):
        a = np.array(anchors[i % len(anchors)])
        out[i, 1:] = a
        out[i, 0] = np.linalg.norm(np.asarray(pose[:3]) - a) + rng.normal(0.0, sigma)
    return out


def odometry_step(seed, step=0.1, noise=0.05):
    """(delta_x, delta_y, delta_z, delta_a) of one update."""
    rng = np.random.default_rng(seed)
    return (step + rng.normal(0.0, noise), rng.normal(0.0, noise), rng.normal(0.0, noise * 0.1),
            rng.normal(0.0, noise * 0.2))


# Launch-file filter parameters (amcl3d/launch/amcl3d.launch:79-105).
SENSOR_DEV = 0.05
ODOM_MODS = (0.1, 0.1, 0.01, 0.3)
