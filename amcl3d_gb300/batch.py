"""Many particle filters stepped together on one GPU (``amcl_batch_*`` in the C ABI).

``FilterBatch`` owns fixed device arenas (the memory budget filters are admitted
against); each added filter is a slot that behaves exactly like a ``ParticleFilter``
with the same seed.  ``stage`` records one filter's next step (predict, update,
resample); ``step`` launches the staged steps of all filters as one CUDA graph.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .filter import Grid3d, Particle, _cloud_array, _ranges_array


class FilterBatch:
    def __init__(self, max_filters: int, max_particles: int, max_points_per_step: int, stream: int | None = None):
        self._h = C.c_void_p()
        N.call("amcl_batch_create", C.byref(self._h), int(max_filters), int(max_particles),
               int(max_points_per_step), C.c_void_p(stream) if stream else None)

    def close(self):
        if self._h:
            N.lib.amcl_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, grid: Grid3d | None, capacity: int, seed: int) -> int:
        """A new filter slot; raises AmclError(AMCL_ENOMEM) when it does not fit."""
        slot = C.c_int()
        N.call("amcl_batch_add", self._h, grid.handle if grid is not None else None, int(capacity),
               int(seed) & (2**64 - 1), C.byref(slot))
        return slot.value

    def try_add(self, grid: Grid3d | None, capacity: int, seed: int) -> int | None:
        slot = C.c_int()
        rc = N.lib.amcl_batch_add(self._h, grid.handle if grid is not None else None, int(capacity),
                                  int(seed) & (2**64 - 1), C.byref(slot))
        return slot.value if rc == N.AMCL_OK else None

    def remove(self, slot: int) -> None:
        N.call("amcl_batch_remove", self._h, int(slot))

    def set_grid(self, slot: int, grid: Grid3d) -> None:
        N.call("amcl_batch_set_grid", self._h, int(slot), grid.handle)

    def init(self, slot, num_particles, x, y, z, a, xd, yd, zd, ad) -> None:
        N.call("amcl_batch_init", self._h, int(slot), int(num_particles), float(x), float(y), float(z), float(a),
               float(xd), float(yd), float(zd), float(ad))

    def set_particles(self, slot: int, p7) -> None:
        a = np.ascontiguousarray(np.asarray(p7, dtype=np.float32).reshape(-1, 7))
        N.call("amcl_batch_set_particles", self._h, int(slot), N.fptr(a), a.shape[0])

    def particles(self, slot: int, n: int) -> np.ndarray:
        out = np.empty((n, 7), np.float32)
        N.call("amcl_batch_get_particles", self._h, int(slot), N.fptr(out), n)
        return out

    def stage(self, slot: int, cloud, range_data, odom=None, alpha=0.5, sigma=0.1, roll=0.0, pitch=0.0,
              resample=True) -> None:
        """odom: (x_mod, y_mod, z_mod, a_mod, dx, dy, dz, da) to predict first, or None."""
        pts, stride = _cloud_array(cloud)
        rg = _ranges_array(range_data)
        od = None if odom is None else np.ascontiguousarray(odom, dtype=np.float64)
        N.call("amcl_batch_stage", self._h, int(slot), N.fptr(pts), pts.shape[0], stride,
               N.fptr(rg) if rg.size else None, rg.shape[0], N.dptr(od) if od is not None else None, float(alpha),
               float(sigma), float(roll), float(pitch), 1 if resample else 0)

    def stage_many(self, slots, clouds, range_data=None, odom=None, alpha=0.5, sigma=0.1, roll=0.0, pitch=0.0,
                   resample=True) -> None:
        """stage() for many filters in one native call: clouds[k] (and range_data[k])
        for slots[k]; odom is one (x_mod, y_mod, z_mod, a_mod, dx, dy, dz, da) for all,
        a (count, 8) array, or None.  The clouds must share their stride (3 or 4 floats)."""
        count = len(slots)
        arrs = [_cloud_array(c) for c in clouds]
        stride = arrs[0][1] if arrs else 4
        if any(st != stride for _, st in arrs):
            raise ValueError("stage_many: the clouds must all have the same stride")
        rgs = [_ranges_array(r) for r in range_data] if range_data is not None else None
        sl = np.ascontiguousarray(slots, dtype=np.int32)
        ptrs = (C.c_void_p * count)(*[a.ctypes.data for a, _ in arrs])
        ns = np.array([a.shape[0] for a, _ in arrs], dtype=np.uint32)
        rptrs = (C.c_void_p * count)(*[r.ctypes.data if r.size else None for r in rgs]) if rgs else None
        nrs = np.array([r.shape[0] for r in rgs], dtype=np.uint32) if rgs else None
        od = None
        if odom is not None:
            o = np.asarray(odom, dtype=np.float64)
            od = np.ascontiguousarray(np.broadcast_to(o, (count, 8)) if o.ndim == 1 else o.reshape(count, 8))
        N.call("amcl_batch_stage_many", self._h, count, sl.ctypes.data_as(C.POINTER(C.c_int)), ptrs,
               ns.ctypes.data_as(C.POINTER(C.c_uint32)), stride, rptrs,
               nrs.ctypes.data_as(C.POINTER(C.c_uint32)) if nrs is not None else None,
               N.dptr(od) if od is not None else None, float(alpha), float(sigma), float(roll), float(pitch),
               1 if resample else 0)

    def stage_packed(self, slots, cloud, counts, range_data=None, range_counts=None, odom=None, alpha=0.5,
                     sigma=0.1, roll=0.0, pitch=0.0, resample=True) -> None:
        """stage() for many filters from one packed cloud: slots[k] takes the next
        counts[k] rows of `cloud` ((total, 3 or 4) float32) and the next range_counts[k]
        rows of range_data ((total, 4)); odom as in stage_many."""
        count = len(slots)
        pts, stride = _cloud_array(cloud)
        sl = np.ascontiguousarray(slots, dtype=np.int32)
        ns = np.ascontiguousarray(counts, dtype=np.uint32)
        if ns.shape[0] != count or int(ns.sum()) != pts.shape[0]:
            raise ValueError("stage_packed: counts must cover the packed cloud, one per slot")
        rg = nrs = None
        if range_data is not None:
            rg = _ranges_array(range_data)
            nrs = np.ascontiguousarray(range_counts, dtype=np.uint32)
            if nrs.shape[0] != count or int(nrs.sum()) != rg.shape[0]:
                raise ValueError("stage_packed: range_counts must cover range_data, one per slot")
        od = None
        if odom is not None:
            o = np.asarray(odom, dtype=np.float64)
            od = np.ascontiguousarray(np.broadcast_to(o, (count, 8)) if o.ndim == 1 else o.reshape(count, 8))
        N.call("amcl_batch_stage_packed", self._h, count, sl.ctypes.data_as(C.POINTER(C.c_int)), N.fptr(pts),
               ns.ctypes.data_as(C.POINTER(C.c_uint32)), stride, N.fptr(rg) if rg is not None and rg.size else None,
               nrs.ctypes.data_as(C.POINTER(C.c_uint32)) if nrs is not None else None,
               N.dptr(od) if od is not None else None, float(alpha), float(sigma), float(roll), float(pitch),
               1 if resample else 0)

    def step(self) -> None:
        N.call("amcl_batch_step", self._h)

    def wait(self) -> None:
        N.call("amcl_batch_wait", self._h)

    def getMean(self, slot: int) -> Particle:
        m = np.zeros(7, np.float32)
        N.call("amcl_batch_get_mean", self._h, int(slot), N.fptr(m), None)
        return Particle(*[float(v) for v in m])

    def mean_var(self, slot: int):
        m = np.zeros(7, np.float32)
        mv = np.zeros(8, np.float64)
        N.call("amcl_batch_get_mean", self._h, int(slot), N.fptr(m), N.dptr(mv))
        return m[:4].copy(), mv[:4].copy(), mv[4:].copy()

    def set_split(self, mode: int, scratch_bytes: int = 0) -> None:
        """Point-parallel weighting of small steps: 0 auto, 1 never, 2 always."""
        N.call("amcl_batch_set_split", self._h, int(mode), int(scratch_bytes))

    def set_tuning(self, threads: int, chunk: int) -> None:
        N.call("amcl_batch_set_tuning", self._h, int(threads), int(chunk))

    def tuning(self) -> tuple[int, int]:
        t, c = C.c_int(), C.c_int()
        N.call("amcl_batch_get_tuning", self._h, C.byref(t), C.byref(c))
        return t.value, c.value

    def autotune(self, reps: int = 3) -> tuple[int, int, float]:
        t, c, ms = C.c_int(), C.c_int(), C.c_double()
        N.call("amcl_batch_autotune", self._h, int(reps), C.byref(t), C.byref(c), C.byref(ms))
        return t.value, c.value, ms.value

    def capacity(self) -> tuple[int, int]:
        fp, fs = C.c_uint64(), C.c_uint32()
        N.call("amcl_batch_capacity", self._h, C.byref(fp), C.byref(fs))
        return int(fp.value), int(fs.value)

    def stream(self) -> int:
        s = C.c_void_p()
        N.call("amcl_batch_stream", self._h, C.byref(s))
        return int(s.value or 0)
