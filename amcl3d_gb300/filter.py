"""Python mirror of amcl3d's ``Grid3d`` and ``ParticleFilter`` over the C ABI.

Same class and method names, argument meaning and error behaviour as the
reference (amcl3d/src/Grid3d.h:34-159, ParticleFilter.h:67-213): methods that
return ``bool`` there return ``bool`` here, ``computeCloudWeight`` returns 0 when
no grid is loaded, ``isIntoMap`` returns False.  Everything runs in
``libamcl3d_gpu.so``; this module only converts arguments.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as N


@dataclass
class Particle:
    """amcl3d::Particle (ParticleFilter.h:35-49)."""

    x: float = 0.0
    y: float = 0.0
    z: float = 0.0
    a: float = 0.0
    w: float = 0.0
    wp: float = 0.0
    wr: float = 0.0


def _cloud_array(cloud) -> tuple[np.ndarray, int]:
    a = np.ascontiguousarray(np.asarray(cloud, dtype=np.float32))
    if a.ndim != 2 or a.shape[1] < 3:
        raise ValueError("cloud must be an (N, 3) or (N, 4) float array")
    return a, a.shape[1]


def _ranges_array(range_data) -> np.ndarray:
    if range_data is None:
        return np.zeros((0, 4), np.float32)
    r = np.ascontiguousarray(np.asarray(range_data, dtype=np.float32).reshape(-1, 4))
    return r


def read_octomap(path) -> dict:
    """openOcTree + computePointCloud (PointCloudTools.cpp:26-82) by the library's
    octomap reader: {points (n, 4) float32, min, max, res, nodes}; raises AmclError
    where the reference throws."""
    n, nodes, res = C.c_uint64(), C.c_uint64(), C.c_double()
    mn, mx = np.zeros(3), np.zeros(3)
    N.call("amcl_octomap_read", str(path).encode(), None, 0, C.byref(n), N.dptr(mn), N.dptr(mx), C.byref(res),
           C.byref(nodes))
    pts = np.empty((max(n.value, 1), 4), np.float32)
    N.call("amcl_octomap_read", str(path).encode(), N.fptr(pts), pts.shape[0], C.byref(n), N.dptr(mn), N.dptr(mx),
           C.byref(res), C.byref(nodes))
    return {"points": pts[: n.value], "min": tuple(mn), "max": tuple(mx), "res": res.value, "nodes": nodes.value}


class Grid3d:
    """amcl3d::Grid3d on the GPU."""

    def __init__(self, stream: int | None = None):
        self._h = C.c_void_p()
        N.call("amcl_grid_create", C.byref(self._h), C.c_void_p(stream) if stream else None)

    def close(self) -> None:
        if self._h:
            N.lib.amcl_grid_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    # -- map building ------------------------------------------------------------------
    def open(self, map_path: str, sensor_dev: float) -> bool:
        """Grid3d::open (Grid3d.cpp:25-78): octomap .bt/.ot -> occupied leaf centres ->
        the .grid file beside the map, or the GPU distance field (then saved there).
        False (with the reason in ``last_error``) where the reference logs and returns false."""
        n = C.c_uint64()
        rc = N.lib.amcl_grid_open(self._h, str(map_path).encode(), float(sensor_dev), C.byref(n))
        self.last_error = None if rc == N.AMCL_OK else N.lib.amcl_last_error().decode(errors="replace")
        return rc == N.AMCL_OK

    def buildGridMap(self, points, bounds_min, bounds_max, resolution: float, sensor_dev: float) -> bool:
        """computeGrid (PointCloudTools.cpp:84-149) on the occupied-leaf centres."""
        pts, stride = _cloud_array(points)
        mn = np.ascontiguousarray(bounds_min, dtype=np.float64)
        mx = np.ascontiguousarray(bounds_max, dtype=np.float64)
        N.call("amcl_grid_build", self._h, N.fptr(pts), pts.shape[0], stride, N.dptr(mn), N.dptr(mx),
               float(resolution), float(sensor_dev))
        return True

    def loadGrid(self, path: str, bounds_min, bounds_max, resolution: float, sensor_dev: float) -> bool:
        """Grid3d::loadGrid (Grid3d.cpp:239-275); False on error or sensor_dev mismatch."""
        mn = np.ascontiguousarray(bounds_min, dtype=np.float64)
        mx = np.ascontiguousarray(bounds_max, dtype=np.float64)
        rc = N.lib.amcl_grid_load(self._h, str(path).encode(), N.dptr(mn), N.dptr(mx), float(resolution),
                                  float(sensor_dev))
        return rc == N.AMCL_OK

    def saveGrid(self, path: str) -> bool:
        """Grid3d::saveGrid (Grid3d.cpp:210-237)."""
        return N.lib.amcl_grid_save(self._h, str(path).encode()) == N.AMCL_OK

    def load_cells(self, info: dict, dist, prob) -> None:
        gi = N.GridInfo()
        for a in range(3):
            gi.min[a] = info["min"][a]
            gi.max[a] = info["max"][a]
            gi.size[a] = info["size"][a]
        gi.resolution = info["resolution"]
        gi.sensor_dev = info["sensor_dev"]
        p = np.ascontiguousarray(prob, dtype=np.float32).ravel()
        d = None if dist is None else np.ascontiguousarray(dist, dtype=np.float32).ravel()
        N.call("amcl_grid_load_cells", self._h, C.byref(gi), N.fptr(d) if d is not None else None, N.fptr(p))

    def info(self) -> dict:
        gi = N.GridInfo()
        N.call("amcl_grid_info_get", self._h, C.byref(gi))
        return {
            "min": tuple(gi.min), "max": tuple(gi.max), "resolution": gi.resolution,
            "sensor_dev": gi.sensor_dev, "size": tuple(int(s) for s in gi.size),
            "storage": int(gi.storage), "u8_scale": gi.u8_scale,
        }

    def read_cells(self, first: int = 0, count: int | None = None) -> tuple[np.ndarray, np.ndarray]:
        inf = self.info()
        total = inf["size"][0] * inf["size"][1] * inf["size"][2]
        if count is None:
            count = total - first
        d = np.empty(count, np.float32)
        p = np.empty(count, np.float32)
        N.call("amcl_grid_read_cells", self._h, first, count, N.fptr(d), N.fptr(p))
        return d, p

    def weight_loop(self) -> int:
        """The yaw-only weighting loop the grid selects: 0 general, 1 zero minimum (offsets
        are floats), 2 general yaw loop (a real map's minimum)."""
        v = C.c_int()
        N.call("amcl_grid_weight_loop", self._h, C.byref(v))
        return int(v.value)

    def set_storage(self, storage: str | int) -> None:
        code = {"f32": N.GRID_F32, "f16": N.GRID_F16, "u8": N.GRID_U8}.get(storage, storage)
        N.call("amcl_grid_set_storage", self._h, int(code))

    def set_l2_window(self, enable: bool) -> None:
        N.call("amcl_grid_set_l2_window", self._h, 1 if enable else 0)

    # -- queries -----------------------------------------------------------------------
    def isIntoMap(self, x: float, y: float, z: float) -> bool:
        out = C.c_int()
        N.call("amcl_grid_is_into_map", self._h, float(x), float(y), float(z), C.byref(out))
        return bool(out.value)

    def computeCloudWeights(self, poses, cloud, roll: float = 0.0, pitch: float = 0.0) -> np.ndarray:
        """Grid3d::computeCloudWeight for each (x, y, z, yaw) pose."""
        ps = np.ascontiguousarray(np.asarray(poses, dtype=np.float32).reshape(-1, 4))
        pts, stride = _cloud_array(cloud)
        out = np.empty(ps.shape[0], np.float32)
        N.call("amcl_grid_cloud_weights", self._h, N.fptr(ps), ps.shape[0], N.fptr(pts), pts.shape[0], stride,
               float(roll), float(pitch), N.fptr(out))
        return out

    def computeCloudWeight(self, cloud, tx, ty, tz, roll, pitch, yaw) -> float:
        """Grid3d::computeCloudWeight (Grid3d.cpp:133-199)."""
        return float(self.computeCloudWeights([[tx, ty, tz, yaw]], cloud, roll, pitch)[0])

    def buildGridSliceMsg(self, z: float):
        """Grid3d::buildGridSliceMsg: (data int8, width, height), or None where the reference returns false."""
        ln, w, h = C.c_uint64(), C.c_uint32(), C.c_uint32()
        rc = N.lib.amcl_grid_slice(self._h, float(z), None, 0, C.byref(ln), C.byref(w), C.byref(h))
        if rc != N.AMCL_OK:
            return None
        out = np.empty(ln.value, np.int8)
        N.call("amcl_grid_slice", self._h, float(z), out.ctypes.data_as(C.POINTER(C.c_int8)), out.size,
               C.byref(ln), C.byref(w), C.byref(h))
        return out, int(w.value), int(h.value)


class ParticleFilter:
    """amcl3d::ParticleFilter on the GPU (device-resident particles)."""

    def __init__(self, seed: int = 0, stream: int | None = None):
        self._h = C.c_void_p()
        N.call("amcl_pf_create", C.byref(self._h), int(seed) & (2**64 - 1), C.c_void_p(stream) if stream else None)

    def close(self) -> None:
        if self._h:
            N.lib.amcl_pf_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def stream(self) -> int:
        s = C.c_void_p()
        N.call("amcl_pf_stream", self._h, C.byref(s))
        return int(s.value or 0)

    def isInitialized(self) -> bool:
        v = C.c_int()
        N.call("amcl_pf_is_initialized", self._h, C.byref(v))
        return bool(v.value)

    def size(self) -> int:
        v = C.c_uint32()
        N.call("amcl_pf_size", self._h, C.byref(v))
        return int(v.value)

    def init(self, num_particles, x_init, y_init, z_init, a_init, x_dev, y_dev, z_dev, a_dev) -> None:
        """ParticleFilter::init (ParticleFilter.cpp:46-95)."""
        N.call("amcl_pf_init", self._h, int(num_particles), float(x_init), float(y_init), float(z_init),
               float(a_init), float(x_dev), float(y_dev), float(z_dev), float(a_dev))

    buildParticlesPool = init

    def predict(self, odom_x_mod, odom_y_mod, odom_z_mod, odom_a_mod, delta_x, delta_y, delta_z, delta_a) -> None:
        """ParticleFilter::predict (ParticleFilter.cpp:97-119)."""
        N.call("amcl_pf_predict", self._h, float(odom_x_mod), float(odom_y_mod), float(odom_z_mod),
               float(odom_a_mod), float(delta_x), float(delta_y), float(delta_z), float(delta_a))

    def update(self, grid3d: Grid3d, cloud, range_data, alpha, sigma, roll, pitch) -> None:
        """ParticleFilter::update (ParticleFilter.cpp:121-196)."""
        pts, stride = _cloud_array(cloud)
        rg = _ranges_array(range_data)
        N.call("amcl_pf_update", self._h, grid3d.handle, N.fptr(pts), pts.shape[0], stride,
               N.fptr(rg) if rg.size else None, rg.shape[0], float(alpha), float(sigma), float(roll), float(pitch))

    def update_voxel(self, grid3d: Grid3d, voxel: "VoxelGrid", cloud, leaf, range_data, alpha, sigma, roll,
                     pitch, want_cloud: bool = True):
        """Node.cpp:130-162 on the device: voxel-downsample the raw scan (pcl::VoxelGrid,
        leaf = voxel_size) and update with the result without a host round trip.
        Returns the downsampled cloud ((m, 4) float32; the node publishes it) or its size."""
        pts, stride = _cloud_array(cloud)
        rg = _ranges_array(range_data)
        lf = np.broadcast_to(np.asarray(leaf, dtype=np.float32), (3,))
        out = np.empty((max(pts.shape[0], 1), 4), np.float32) if want_cloud else None
        m = C.c_uint64()
        N.call("amcl_pf_update_voxel", self._h, grid3d.handle, voxel.handle, N.fptr(pts), pts.shape[0], stride,
               float(lf[0]), float(lf[1]), float(lf[2]), N.fptr(rg) if rg.size else None, rg.shape[0], float(alpha),
               float(sigma), float(roll), float(pitch), N.fptr(out) if want_cloud else None,
               out.shape[0] if want_cloud else 0, C.byref(m))
        return out[: m.value].copy() if want_cloud else int(m.value)

    def update_ranges(self, range_data, alpha, sigma) -> None:
        """Range-only update (declared at ParticleFilter.h:157, not defined by the reference)."""
        rg = _ranges_array(range_data)
        N.call("amcl_pf_update_ranges", self._h, N.fptr(rg) if rg.size else None, rg.shape[0], float(alpha),
               float(sigma))

    def resample(self, u01: float | None = None) -> None:
        """ParticleFilter::resample (ParticleFilter.cpp:198-222); u01 injects the uniform draw."""
        if u01 is None:
            N.call("amcl_pf_resample", self._h)
        else:
            N.call("amcl_pf_resample_with", self._h, float(u01))

    def getMean(self) -> Particle:
        m = np.zeros(7, np.float32)
        N.call("amcl_pf_get_mean", self._h, N.fptr(m), None)
        return Particle(*[float(v) for v in m])

    def mean_var(self) -> tuple[np.ndarray, np.ndarray]:
        m = np.zeros(7, np.float32)
        mv = np.zeros(8, np.float64)
        N.call("amcl_pf_get_mean", self._h, N.fptr(m), N.dptr(mv))
        return mv[:4].copy(), mv[4:].copy()

    def particles(self) -> np.ndarray:
        n = self.size()
        out = np.empty((n, 7), np.float32)
        N.call("amcl_pf_get_particles", self._h, N.fptr(out), n)
        return out

    def set_particles(self, p7) -> None:
        a = np.ascontiguousarray(np.asarray(p7, dtype=np.float32).reshape(-1, 7))
        N.call("amcl_pf_set_particles", self._h, N.fptr(a), a.shape[0])

    def buildParticlesPoseMsg(self) -> np.ndarray:
        """ParticleFilter::buildParticlesPoseMsg (ParticleFilter.cpp:30-44): poses as
        (x, y, z, qx, qy, qz, qw) doubles, yaw-only quaternion."""
        p = self.particles()
        half = (p[:, 3] * np.float32(0.5)).astype(np.float64)
        out = np.zeros((p.shape[0], 7), np.float64)
        out[:, 0:3] = p[:, 0:3]
        out[:, 5] = np.sin(half)
        out[:, 6] = np.cos(half)
        return out

    def set_option(self, option: int, value: int) -> None:
        N.call("amcl_pf_set_option", self._h, int(option), int(value))

    def record_draws(self, enable: bool = True) -> None:
        N.call("amcl_pf_record_draws", self._h, 1 if enable else 0)

    def draws(self) -> np.ndarray:
        n = self.size()
        out = np.empty((n, 4), np.float32)
        N.call("amcl_pf_get_draws", self._h, N.fptr(out), out.size)
        return out

    def resample_index(self) -> np.ndarray:
        n = self.size()
        out = np.empty(n, np.int32)
        N.call("amcl_pf_get_resample_index", self._h, out.ctypes.data_as(C.POINTER(C.c_int32)), n)
        return out

    def profile(self, enable: bool = True) -> None:
        N.call("amcl_pf_profile", self._h, 1 if enable else 0)

    def profile_read(self, reset: bool = False) -> dict:
        ms = (C.c_double * 5)()
        cnt = (C.c_uint64 * 5)()
        N.call("amcl_pf_profile_read", self._h, ms, cnt, 1 if reset else 0)
        return {name: (ms[i], int(cnt[i])) for i, name in enumerate(N.PROF_NAMES)}


class VoxelGrid:
    """pcl::VoxelGrid<pcl::PointXYZ> as the node uses it (Node.cpp:130-137) on the GPU:
    ``setInputCloud``, ``setLeafSize``, ``filter``."""

    def __init__(self, stream: int | None = None):
        self._h = C.c_void_p()
        N.call("amcl_voxel_create", C.byref(self._h), C.c_void_p(stream) if stream else None)
        self._cloud = np.zeros((0, 4), np.float32)
        self._leaf = (1.0, 1.0, 1.0)

    def close(self) -> None:
        if self._h:
            N.lib.amcl_voxel_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def setInputCloud(self, cloud) -> None:
        self._cloud = _cloud_array(cloud)[0]

    def setLeafSize(self, lx: float, ly: float, lz: float) -> None:
        self._leaf = (float(lx), float(ly), float(lz))

    def filter(self) -> np.ndarray:
        return self.downsample(self._cloud, self._leaf)

    def downsample(self, cloud, leaf) -> np.ndarray:
        """Centroids ((m, 4) float32, w = 1) of the occupied leaves, in voxel-key order."""
        pts, stride = _cloud_array(cloud)
        lf = np.broadcast_to(np.asarray(leaf, dtype=np.float32), (3,))
        out = np.empty((max(pts.shape[0], 1), 4), np.float32)
        m = C.c_uint64()
        N.call("amcl_voxel_filter", self._h, N.fptr(pts), pts.shape[0], stride, float(lf[0]), float(lf[1]),
               float(lf[2]), N.fptr(out), out.shape[0], C.byref(m))
        return out[: m.value].copy()

    def downsample_dev(self, in_ptr: int, n: int, leaf, out_ptr: int) -> int:
        """Device float4 buffers (16-byte aligned; out has room for n points); returns the count."""
        lf = np.broadcast_to(np.asarray(leaf, dtype=np.float32), (3,))
        m = C.c_uint64()
        N.call("amcl_voxel_filter_dev", self._h, C.c_void_p(in_ptr), int(n), float(lf[0]), float(lf[1]),
               float(lf[2]), C.c_void_p(out_ptr), C.byref(m))
        return int(m.value)
