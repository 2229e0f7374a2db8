"""CPU oracles for amcl3d's particle-filter hot path.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may use this package, and only as the checker:
the GPU library never calls into it.

Two oracles:

* ``liboracle.so`` (``amcl3d_oracle.c``): a C restatement of the reference's
  arithmetic (each function cites amcl3d/src file:line), plus the exact-sum
  semantics of the GPU build restated here with ``math.fsum`` / Python integers;
* ``_ref/libamcl3d_ref.so`` (``ref_harness.cpp``): the reference's own
  ParticleFilter.cpp / Grid3d.cpp / PointCloudTools.cpp compiled verbatim against
  the stand-in headers in ``tests/stand_in/``.  It exists only where the reference tree is
  available at build time; the committed golden fixtures under ``tests/golden``
  carry its outputs elsewhere.
"""

from __future__ import annotations

import ctypes as C
import math
import os
import struct
import subprocess
import tempfile
from fractions import Fraction
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_ORC_PATH = HERE / "_build" / "liboracle.so"
_REF_PATH = HERE / "_ref" / "libamcl3d_ref.so"

_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)
_i64p = C.POINTER(C.c_int64)
_i32p = C.POINTER(C.c_int32)
_u32p = C.POINTER(C.c_uint32)


def _f(a):
    return a.ctypes.data_as(_fp)


def _d(a):
    return a.ctypes.data_as(_dp)


class OrcGrid(C.Structure):
    _fields_ = [
        ("min", C.c_double * 3),
        ("max", C.c_double * 3),
        ("res", C.c_double),
        ("size", C.c_uint32 * 3),
        ("prob", _fp),
    ]


def _load_oracle():
    subprocess.run(["make", "-s", "-C", str(HERE), "all"], check=True)
    lib = C.CDLL(str(_ORC_PATH))
    lib.orc_cloud_weights.argtypes = [C.POINTER(OrcGrid), _fp, C.c_uint64, _fp, C.c_uint64, C.c_uint32, C.c_float,
                                      C.c_float, C.c_int, _fp, _i64p]
    lib.orc_cloud_weights.restype = None
    lib.orc_is_into_map.argtypes = [C.POINTER(OrcGrid), C.c_float, C.c_float, C.c_float]
    lib.orc_is_into_map.restype = C.c_int
    lib.orc_range_weight.argtypes = [C.c_float, C.c_float, C.c_float, _fp, C.c_uint32, C.c_double, C.c_int]
    lib.orc_range_weight.restype = C.c_float
    lib.orc_update_f32.argtypes = [_fp, C.c_uint64, C.POINTER(OrcGrid), _fp, C.c_uint64, C.c_uint32, _fp, C.c_uint32,
                                   C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, _fp]
    lib.orc_update_f32.restype = None
    lib.orc_resample_f32.argtypes = [_fp, C.c_uint64, C.c_float, _i32p]
    lib.orc_resample_f32.restype = C.c_int
    lib.orc_predict.argtypes = [_fp, C.c_uint64, _fp] + [C.c_double] * 8 + [C.c_int]
    lib.orc_predict.restype = None
    lib.orc_init_pose.argtypes = [_fp, C.c_uint64, _fp] + [C.c_float] * 8 + [C.c_int]
    lib.orc_init_pose.restype = None
    lib.orc_compute_grid.argtypes = [_fp, C.c_uint64, C.c_uint32, _dp, _dp, C.c_double, C.c_double, _u32p, _u32p,
                                     C.c_int, C.c_int, _fp, _fp]
    lib.orc_compute_grid.restype = C.c_int
    lib.orc_philox4x32_10.argtypes = [_u32p, _u32p, _u32p]
    lib.orc_philox4x32_10.restype = None
    lib.orc_grid_cell_probs.argtypes = [_fp, C.c_uint64, C.c_uint32, _dp, C.c_double, C.c_double, _u32p,
                                        C.POINTER(C.c_uint64), C.c_uint64, C.c_int, C.c_int, _fp]
    lib.orc_grid_cell_probs.restype = C.c_int
    lib.orc_voxel_downsample.argtypes = [_fp, C.c_uint64, C.c_uint32, _fp, _fp, C.POINTER(C.c_uint64)]
    lib.orc_voxel_downsample.restype = C.c_int
    return lib


orc = _load_oracle()


# ---- grid descriptor ------------------------------------------------------------------------

class GridData:
    """Bounds, resolution and the per-cell probabilities of one grid (host copy)."""

    def __init__(self, mn, mx, res, size, prob, dist=None, sensor_dev=0.05):
        self.min = tuple(float(v) for v in mn)
        self.max = tuple(float(v) for v in mx)
        self.res = float(res)
        self.size = tuple(int(s) for s in size)
        self.prob = np.ascontiguousarray(prob, dtype=np.float32).ravel()
        self.dist = None if dist is None else np.ascontiguousarray(dist, dtype=np.float32).ravel()
        self.sensor_dev = sensor_dev
        self._s = OrcGrid()
        for a in range(3):
            self._s.min[a] = self.min[a]
            self._s.max[a] = self.max[a]
            self._s.size[a] = self.size[a]
        self._s.res = self.res
        self._s.prob = _f(self.prob)

    @property
    def c(self):
        return C.byref(self._s)


def grid_sizes(mn, mx, res):
    """PointCloudTools.cpp:96-101: ceil((max - min) / res) per axis."""
    return tuple(int(math.ceil((mx[a] - mn[a]) / res)) for a in range(3))


# ---- per-particle functions -----------------------------------------------------------------

def cloud_weights(g: GridData, poses, cloud, roll=0.0, pitch=0.0, yaw_trig=1, cells=False):
    ps = np.ascontiguousarray(np.asarray(poses, np.float32).reshape(-1, 4))
    pts = np.ascontiguousarray(np.asarray(cloud, np.float32))
    out = np.empty(ps.shape[0], np.float32)
    cl = np.empty((ps.shape[0], pts.shape[0]), np.int64) if cells else None
    orc.orc_cloud_weights(g.c, _f(ps), ps.shape[0], _f(pts), pts.shape[0], pts.shape[1], float(roll), float(pitch),
                          int(yaw_trig), _f(out), cl.ctypes.data_as(_i64p) if cells else None)
    return (out, cl) if cells else out


def is_into_map(g: GridData, x, y, z) -> bool:
    return bool(orc.orc_is_into_map(g.c, float(x), float(y), float(z)))


def range_weight(x, y, z, ranges, sigma, exp_mode=1):
    rg = np.ascontiguousarray(np.asarray(ranges, np.float32).reshape(-1, 4))
    return float(orc.orc_range_weight(float(x), float(y), float(z), _f(rg) if rg.size else None, rg.shape[0],
                                      float(sigma), int(exp_mode)))


def update_f32(p7, g: GridData, cloud, ranges, alpha, sigma, roll, pitch, yaw_trig=0, exp_mode=0):
    """The reference's update arithmetic (float running sums); returns (particles, mean4)."""
    p = np.ascontiguousarray(np.array(p7, np.float32).reshape(-1, 7))
    pts = np.ascontiguousarray(np.asarray(cloud, np.float32))
    rg = np.ascontiguousarray(np.asarray(ranges, np.float32).reshape(-1, 4))
    mean = np.zeros(4, np.float32)
    orc.orc_update_f32(_f(p), p.shape[0], g.c, _f(pts), pts.shape[0], pts.shape[1], _f(rg) if rg.size else None,
                       rg.shape[0], float(alpha), float(sigma), float(roll), float(pitch), int(yaw_trig),
                       int(exp_mode), _f(mean))
    return p, mean


# ---- the GPU build's exact sums, restated -------------------------------------------------------

def fsum32(values) -> float:
    """Exact sum of float32 values, correctly rounded to double (what X320 gives)."""
    return math.fsum(np.asarray(values, np.float32).astype(np.float64).tolist())


def two_prod32(a, b):
    """(p, e) float32 with a*b = p + e, e the residual rounded once (FMA semantics)."""
    a64 = np.asarray(a, np.float32).astype(np.float64)
    b64 = np.asarray(b, np.float32).astype(np.float64)
    prod = a64 * b64  # exact: 24 x 24 bits
    p = prod.astype(np.float32)
    e = (prod - p.astype(np.float64)).astype(np.float32)
    return p, e


def normalize_stats(w, pose4):
    """Exact-sum normalisation of w and the mean / variance terms (filter.cu k_normalize
    + k_finalize_stats), restated.  Returns (w_normalised, mean4 float32, mean4 f64, var4)."""
    w = np.asarray(w, np.float32)
    tot = fsum32(w)
    if tot > 0:
        wn = (w.astype(np.float64) / tot).astype(np.float32)
    else:
        wn = np.zeros_like(w)
    s2 = fsum32(wn)
    m1 = np.zeros(4)
    var = np.zeros(4)
    for k in range(4):
        c = np.asarray(pose4[:, k], np.float32)
        h, l = two_prod32(wn, c)
        m1[k] = math.fsum(np.concatenate([h, l]).astype(np.float64).tolist())
        s, t = two_prod32(c, c)
        h1, l1 = two_prod32(wn, s)
        h2, l2 = two_prod32(wn, t)
        m2 = math.fsum(np.concatenate([h1, l1, h2, l2]).astype(np.float64).tolist())
        if s2 > 0:
            mu = m1[k] / s2
            var[k] = m2 / s2 - mu * mu
    return wn, m1.astype(np.float32), m1, var


def update_exact(p7, g: GridData, cloud, ranges, alpha, sigma, roll, pitch, yaw_trig=1, exp_mode=1, cloud_w=None):
    """ParticleFilter::update with the GPU build's exact sums (ParticleFilter.cpp:121-196).

    Per-particle weights come from the C restatement (or ``cloud_w`` if given);
    returns (particles, mean4 float32, mean4 f64, var4)."""
    p = np.array(p7, np.float32).reshape(-1, 7).copy()
    P = p.shape[0]
    inm = np.array([is_into_map(g, *p[i, :3]) for i in range(P)], bool)
    if cloud_w is None:
        cw = cloud_weights(g, p[:, :4], cloud, roll=np.float32(roll), pitch=np.float32(pitch), yaw_trig=yaw_trig)
    else:
        cw = np.asarray(cloud_w, np.float32)
    rg = np.asarray(ranges, np.float32).reshape(-1, 4)
    for i in np.nonzero(inm)[0]:
        p[i, 5] = cw[i]
        p[i, 6] = range_weight(p[i, 0], p[i, 1], p[i, 2], rg, sigma, exp_mode)
    sp = fsum32(p[inm, 5])
    sr = fsum32(p[inm, 6])
    p[:, 5] = (p[:, 5].astype(np.float64) / sp).astype(np.float32) if sp > 0 else 0
    p[:, 6] = (p[:, 6].astype(np.float64) / sr).astype(np.float32) if sr > 0 else 0
    blend = (p[:, 5].astype(np.float64) * alpha + p[:, 6].astype(np.float64) * (1 - alpha)).astype(np.float32)
    p[:, 4] = np.where(inm, blend, np.float32(0))
    wn, m32, m64, var = normalize_stats(p[:, 4], p[:, :4])
    p[:, 4] = wn
    return p, m32, m64, var


def float_to_fraction(v) -> Fraction:
    return Fraction(float(v))


def resample_exact(w, u01):
    """Systematic resampling with the exact prefix (ParticleFilter.cpp:198-222 with
    real-number cumulative weights): idx[m] = first i with C_i >= u_m, clamped to P-1."""
    w = np.asarray(w, np.float32)
    P = w.shape[0]
    factor = np.float32(1.0) / np.float32(P)
    r = np.float32(factor * np.float32(u01))
    # exact prefix as integers in units of 2^-149
    scale = 1 << 149
    ints = [int(Fraction(float(x)) * scale) for x in w]
    pref = []
    acc = 0
    for v in ints:
        acc += v
        pref.append(acc)
    m_idx = np.arange(P, dtype=np.float32)
    u = (r + factor * m_idx).astype(np.float32)  # float ops, as the reference
    out = np.empty(P, np.int32)
    i = 0
    for m in range(P):
        um = int(Fraction(float(u[m])) * scale)
        while i < P and pref[i] < um:
            i += 1
        out[m] = min(i, P - 1)
    return out


def resample_f32(w, u01):
    """The reference's float running-sum resampling; indices == P mark its overrun."""
    w = np.ascontiguousarray(np.asarray(w, np.float32))
    idx = np.empty(w.shape[0], np.int32)
    over = orc.orc_resample_f32(_f(w), w.shape[0], float(u01), idx.ctypes.data_as(_i32p))
    return idx, bool(over)


def predict(p7, draws, odom_mods, deltas, yaw_trig=1):
    p = np.ascontiguousarray(np.array(p7, np.float32).reshape(-1, 7))
    z = np.ascontiguousarray(np.asarray(draws, np.float32).reshape(-1, 4))
    orc.orc_predict(_f(p), p.shape[0], _f(z), *[float(v) for v in odom_mods], *[float(v) for v in deltas],
                    int(yaw_trig))
    return p


def init_pose(n, draws, pose4, devs4, exp_mode=1):
    p = np.zeros((n, 7), np.float32)
    z = np.ascontiguousarray(np.asarray(draws, np.float32).reshape(-1, 4))
    orc.orc_init_pose(_f(p), n, _f(z), *[float(v) for v in pose4], *[float(v) for v in devs4], int(exp_mode))
    return p


def compute_grid(points, mn, mx, res, sensor_dev, lo=None, hi=None, exp_mode=1, threads=None):
    """computeGrid on the cell sub-block [lo, hi) (x-fastest arrays)."""
    pts = np.ascontiguousarray(np.asarray(points, np.float32))
    size = grid_sizes(mn, mx, res)
    lo = np.array(lo if lo is not None else (0, 0, 0), np.uint32)
    hi = np.array(hi if hi is not None else size, np.uint32)
    shape = tuple(int(hi[a] - lo[a]) for a in (2, 1, 0))
    dist = np.empty(shape, np.float32)
    prob = np.empty(shape, np.float32)
    mn64 = np.ascontiguousarray(mn, np.float64)
    mx64 = np.ascontiguousarray(mx, np.float64)
    rc = orc.orc_compute_grid(_f(pts), pts.shape[0], pts.shape[1], _d(mn64), _d(mx64), float(res), float(sensor_dev),
                              lo.ctypes.data_as(_u32p), hi.ctypes.data_as(_u32p), int(exp_mode),
                              int(threads or os.cpu_count() or 1), _f(dist), _f(prob))
    if rc:
        raise RuntimeError(f"orc_compute_grid failed ({rc})")
    return dist, prob


def grid_cell_probs(points, mn, res, sensor_dev, size, cells, exp_mode=0, threads=None) -> np.ndarray:
    """computeGrid's prob for the given linear cell indices only (see orc_grid_cell_probs)."""
    pts = np.ascontiguousarray(np.asarray(points, np.float32)[:, :3])
    c = np.ascontiguousarray(cells, dtype=np.uint64)
    out = np.empty(c.size, np.float32)
    sz = np.ascontiguousarray(size, dtype=np.uint32)
    mn64 = np.ascontiguousarray(mn, dtype=np.float64)
    rc = orc.orc_grid_cell_probs(_f(pts), pts.shape[0], 3, _d(mn64), float(res),
                                 float(sensor_dev), sz.ctypes.data_as(_u32p), c.ctypes.data_as(C.POINTER(C.c_uint64)),
                                 c.size, int(exp_mode), int(threads or os.cpu_count() or 1), _f(out))
    if rc:
        raise MemoryError("orc_grid_cell_probs")
    return out


def voxel_downsample(cloud, leaf):
    """pcl::VoxelGrid<PointXYZ> as called by Node.cpp:130-137 (PCL's published algorithm;
    a voxel's points summed in input order).  cloud: (n, 3|4) float32; leaf: scalar or 3.
    Returns (float32 (m, 4) centroids in voxel-key order with w = 1, overflowed flag)."""
    c = np.ascontiguousarray(cloud, dtype=np.float32)
    n = c.shape[0]
    lf = np.broadcast_to(np.asarray(leaf, dtype=np.float32), (3,)).copy()
    out = np.empty((max(n, 1), 4), np.float32)
    m = C.c_uint64(0)
    ovf = orc.orc_voxel_downsample(_f(c), n, c.shape[1] if n else 4, _f(lf), _f(out), C.byref(m))
    return out[: m.value].copy(), bool(ovf)


def philox4x32_10(ctr, key):
    c = (C.c_uint32 * 4)(*[int(v) & 0xFFFFFFFF for v in ctr])
    k = (C.c_uint32 * 2)(*[int(v) & 0xFFFFFFFF for v in key])
    o = (C.c_uint32 * 4)()
    orc.orc_philox4x32_10(c, k, o)
    return tuple(int(v) for v in o)


# ---- map files read by the stand-in octomap ---------------------------------------------------

def write_points_map(path, points, mn, mx, res):
    """AMCLPTS1 file: the occupied leaf centres the stand-in OcTree serves."""
    pts = np.ascontiguousarray(np.asarray(points, np.float32)[:, :3])
    with open(path, "wb") as f:
        f.write(b"AMCLPTS1")
        f.write(struct.pack("<d", float(res)))
        f.write(struct.pack("<3d", *[float(v) for v in mn]))
        f.write(struct.pack("<3d", *[float(v) for v in mx]))
        f.write(struct.pack("<Q", pts.shape[0]))
        f.write(pts.tobytes())


# ---- the verbatim reference (only where it was built) -------------------------------------------

def ref_available() -> bool:
    return _REF_PATH.exists()


_ref = None


def ref():
    global _ref
    if _ref is None:
        if not _REF_PATH.exists():
            raise FileNotFoundError("reference build oracle/_ref/libamcl3d_ref.so is absent")
        L = C.CDLL(str(_REF_PATH))
        vp = C.c_void_p
        sig = {
            "ref_grid_new": ([], vp), "ref_grid_free": ([vp], None),
            "ref_grid_open": ([vp, C.c_char_p, C.c_double], C.c_int),
            "ref_grid_info": ([vp, _u32p, _dp, _dp, _dp], C.c_int),
            "ref_grid_cells": ([vp, C.c_uint64, C.c_uint64, _fp, _fp], C.c_int),
            "ref_grid_slice": ([vp, C.c_double, C.POINTER(C.c_int8), C.c_uint64, C.POINTER(C.c_uint64), _u32p, _u32p],
                               C.c_int),
            "ref_grid_is_into_map": ([vp, C.c_float, C.c_float, C.c_float], C.c_int),
            "ref_cloud_new": ([_fp, C.c_uint64, C.c_uint64], vp), "ref_cloud_free": ([vp], None),
            "ref_cloud_weight": ([vp, vp] + [C.c_float] * 6, C.c_float),
            "ref_pf_new": ([C.c_uint32], vp), "ref_pf_free": ([vp], None),
            "ref_pf_seed": ([vp, C.c_uint32], None), "ref_pf_size": ([vp], C.c_uint64),
            "ref_pf_set_particles": ([vp, _fp, C.c_uint64], None), "ref_pf_get_particles": ([vp, _fp], None),
            "ref_pf_get_mean": ([vp, _fp], None),
            "ref_pf_init": ([vp, C.c_int] + [C.c_float] * 8, None),
            "ref_pf_predict": ([vp] + [C.c_double] * 8, None),
            "ref_pf_update": ([vp, vp, vp, _fp, C.c_uint64] + [C.c_double] * 4, None),
            "ref_pf_peek_uniform": ([vp], C.c_float),
            "ref_pf_resample": ([vp, C.POINTER(C.c_int)], None),
            "ref_pf_range_weight": ([vp, C.c_float, C.c_float, C.c_float, _fp, C.c_uint64, C.c_double], C.c_float),
            "ref_time_update": ([vp, vp, _fp, C.c_uint64, _fp, C.c_uint64] + [C.c_double] * 4 +
                                [C.c_int, C.c_int, C.c_int], C.c_double),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _ref = L
    return _ref


class RefGrid:
    """The reference Grid3d, opened from an occupied-point map through Grid3d::open."""

    def __init__(self, points, mn, mx, res, sensor_dev, workdir=None):
        L = ref()
        self._tmp = tempfile.TemporaryDirectory(dir=workdir)
        self.map_path = os.path.join(self._tmp.name, "map.bt")
        write_points_map(self.map_path, points, mn, mx, res)
        self.h = L.ref_grid_new()
        self.ok = bool(L.ref_grid_open(self.h, self.map_path.encode(), float(sensor_dev)))

    def info(self):
        L = ref()
        size = (C.c_uint32 * 3)()
        mn = (C.c_double * 3)()
        mx = (C.c_double * 3)()
        res = C.c_double()
        L.ref_grid_info(self.h, size, mn, mx, C.byref(res))
        return {"size": tuple(size), "min": tuple(mn), "max": tuple(mx), "resolution": res.value}

    def cells(self, first=0, count=None):
        L = ref()
        inf = self.info()
        tot = inf["size"][0] * inf["size"][1] * inf["size"][2]
        count = tot - first if count is None else count
        d = np.empty(count, np.float32)
        p = np.empty(count, np.float32)
        assert L.ref_grid_cells(self.h, first, count, _f(d), _f(p))
        return d, p

    def cloud_weight(self, cloud, tx, ty, tz, roll, pitch, yaw):
        L = ref()
        pts = np.ascontiguousarray(np.asarray(cloud, np.float32))
        c = L.ref_cloud_new(_f(pts), pts.shape[0], pts.shape[1])
        try:
            return float(L.ref_cloud_weight(self.h, c, tx, ty, tz, roll, pitch, yaw))
        finally:
            L.ref_cloud_free(c)

    def slice(self, z):
        L = ref()
        ln = C.c_uint64()
        w = C.c_uint32()
        h = C.c_uint32()
        if not L.ref_grid_slice(self.h, float(z), None, 0, C.byref(ln), C.byref(w), C.byref(h)):
            return None
        out = np.empty(ln.value, np.int8)
        L.ref_grid_slice(self.h, float(z), out.ctypes.data_as(C.POINTER(C.c_int8)), out.size, C.byref(ln),
                         C.byref(w), C.byref(h))
        return out, w.value, h.value

    def close(self):
        if self.h:
            ref().ref_grid_free(self.h)
            self.h = None
        self._tmp.cleanup()


class RefFilter:
    """The reference ParticleFilter with an injectable particle set and seed."""

    def __init__(self, seed=1):
        self.L = ref()
        self.h = self.L.ref_pf_new(seed)

    def set_particles(self, p7):
        a = np.ascontiguousarray(np.asarray(p7, np.float32).reshape(-1, 7))
        self.L.ref_pf_set_particles(self.h, _f(a), a.shape[0])

    def particles(self):
        n = self.L.ref_pf_size(self.h)
        out = np.empty((n, 7), np.float32)
        self.L.ref_pf_get_particles(self.h, _f(out))
        return out

    def mean(self):
        out = np.empty(7, np.float32)
        self.L.ref_pf_get_mean(self.h, _f(out))
        return out

    def init(self, *args):
        self.L.ref_pf_init(self.h, int(args[0]), *[float(v) for v in args[1:]])

    def predict(self, *args):
        self.L.ref_pf_predict(self.h, *[float(v) for v in args])

    def update(self, grid: RefGrid, cloud, ranges, alpha, sigma, roll, pitch):
        pts = np.ascontiguousarray(np.asarray(cloud, np.float32))
        rg = np.ascontiguousarray(np.asarray(ranges, np.float32).reshape(-1, 4))
        c = self.L.ref_cloud_new(_f(pts), pts.shape[0], pts.shape[1])
        try:
            self.L.ref_pf_update(self.h, grid.h, c, _f(rg) if rg.size else None, rg.shape[0], float(alpha),
                                 float(sigma), float(roll), float(pitch))
        finally:
            self.L.ref_cloud_free(c)

    def peek_uniform(self):
        return float(self.L.ref_pf_peek_uniform(self.h))

    def resample(self):
        over = C.c_int()
        self.L.ref_pf_resample(self.h, C.byref(over))
        return bool(over.value)

    def close(self):
        if self.h:
            self.L.ref_pf_free(self.h)
            self.h = None
