"""Multi-session serving (``amcl_server_*``) and its load generator.

``Server`` wraps the C ABI: sessions are filter slots of a device-resident batch,
requests are scheduled by a native thread with continuous batching.  ``run_load``
drives it open-loop: each session sends update requests as a Poisson process,
sessions join and leave at a fixed rate, new sessions wait in an admission queue
while the memory budget is exhausted; it reports p50/p99 update latency and the
aggregate particle x point weights per second.  ``run_plain`` serves the same kind
of requests one filter per call (predict, update, getMean, resample per request,
one after another) for comparison on the same GPU, closed-loop (its capacity) and
``run_plain_open`` at the served run's offered load (open-loop arrivals, one filter
per session, requests handled first come first served).
"""

from __future__ import annotations

import ctypes as C
import heapq
import math
import time
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .filter import Grid3d, ParticleFilter, _cloud_array, _ranges_array


class ServerResult(C.Structure):
    _fields_ = [
        ("ticket", C.c_uint64),
        ("session", C.c_int64),
        ("status", C.c_int32),
        ("reserved", C.c_int32),
        ("t_submit", C.c_double),
        ("t_done", C.c_double),
        ("mean", C.c_float * 4),
        ("var", C.c_double * 4),
    ]


class Server:
    def __init__(self, max_sessions: int, max_particles: int, max_points_per_step: int, lanes: int = 4):
        self._h = C.c_void_p()
        N.call("amcl_server_create_lanes", C.byref(self._h), int(max_sessions), int(max_particles),
               int(max_points_per_step), int(lanes), None)
        self._buf = (ServerResult * 4096)()

    def close(self):
        if self._h:
            N.lib.amcl_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def open_session(self, grid: Grid3d, capacity: int, seed: int, num_particles: int, init8) -> int | None:
        sid = C.c_int64()
        ini = np.ascontiguousarray(init8, dtype=np.float32)
        rc = N.lib.amcl_server_open_session(self._h, grid.handle, int(capacity), int(seed) & (2**64 - 1),
                                            int(num_particles), N.fptr(ini), C.byref(sid))
        if rc == 2:  # AMCL_ENOMEM: admission refused
            return None
        if rc != 0:
            raise N.AmclError(rc, "amcl_server_open_session", N.lib.amcl_last_error().decode())
        return sid.value

    def close_session(self, sid: int) -> None:
        N.call("amcl_server_close_session", self._h, int(sid))

    def submit(self, sid: int, cloud, range_data, odom=None, alpha=0.5, sigma=0.1, roll=0.0, pitch=0.0,
               resample=True) -> int:
        pts, stride = _cloud_array(cloud)
        rg = _ranges_array(range_data)
        od = None if odom is None else np.ascontiguousarray(odom, dtype=np.float64)
        t = C.c_uint64()
        N.call("amcl_server_submit", self._h, int(sid), N.fptr(pts), pts.shape[0], stride,
               N.fptr(rg) if rg.size else None, rg.shape[0], N.dptr(od) if od is not None else None, float(alpha),
               float(sigma), float(roll), float(pitch), 1 if resample else 0, C.byref(t))
        return t.value

    def prepare(self, sid: int, cloud, range_data, odom=None, alpha=0.5, sigma=0.1, roll=0.0, pitch=0.0,
                resample=True) -> tuple:
        """The arguments of submit() converted once, for a caller that sends the same
        request shape again and again (submit_prepared).  The arrays are kept alive by
        the returned tuple."""
        pts, stride = _cloud_array(cloud)
        rg = _ranges_array(range_data)
        od = None if odom is None else np.ascontiguousarray(odom, dtype=np.float64)
        keep = (pts, rg, od)
        args = (self._h, C.c_int64(int(sid)), pts.ctypes.data_as(N._fp), C.c_uint32(pts.shape[0]),
                C.c_uint32(stride), rg.ctypes.data_as(N._fp) if rg.size else None, C.c_uint32(rg.shape[0]),
                od.ctypes.data_as(N._dp) if od is not None else None, C.c_double(alpha), C.c_double(sigma),
                C.c_double(roll), C.c_double(pitch), C.c_int(1 if resample else 0))
        return keep, args, C.c_uint64()

    def submit_prepared(self, prepared) -> int:
        _keep, args, t = prepared
        rc = N.lib.amcl_server_submit(*args, C.byref(t))
        if rc != 0:
            raise N.AmclError(rc, "amcl_server_submit", N.lib.amcl_last_error().decode())
        return t.value

    def poll(self) -> list:
        out = []
        while True:
            n = C.c_uint32()
            N.call("amcl_server_poll", self._h, self._buf, len(self._buf), C.byref(n))
            for i in range(n.value):
                r = self._buf[i]
                out.append((r.ticket, r.session, r.status, r.t_submit, r.t_done, tuple(r.mean)))
            if n.value < len(self._buf):
                return out

    def counters(self) -> dict:
        g, r = C.c_uint64(), C.c_uint64()
        N.call("amcl_server_counters", self._h, C.byref(g), C.byref(r))
        return {"graphs_built": g.value, "reallocs": r.value}

    def stats(self) -> dict:
        steps, reqs, busy, mb, ns = C.c_uint64(), C.c_uint64(), C.c_double(), C.c_uint32(), C.c_uint32()
        N.call("amcl_server_stats", self._h, C.byref(steps), C.byref(reqs), C.byref(busy), C.byref(mb), C.byref(ns))
        return {"steps": steps.value, "requests": reqs.value, "busy_s": busy.value, "max_batch": mb.value,
                "sessions": ns.value}


# ---- workload of the served configuration -------------------------------------------------------

@dataclass
class SessionSpec:
    grid: int
    P: int
    N: int
    pose: np.ndarray
    seed: int


def log_uniform_int(rng, lo, hi):
    return int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))


def make_scan_pool(maps, seed, n_max_points, per_map=4):
    """Ray-cast scans per map at a few free poses (reused by sessions on that map)."""
    from . import synth as S

    pools = []
    for mi, m in enumerate(maps):
        entries = []
        for k in range(per_map):
            pose = S.free_pose(m, seed + 100 * mi + k, height=min(1.5, m.size_m[2] / 2),
                               clearance=min(0.6, m.size_m[2] / 6))
            scan = S.ray_cast(m, pose, n_elev=48, n_azim=max(32, n_max_points // 48 + 1), elev_deg=(-20, 20),
                              max_range=20.0, n_max=n_max_points, seed=seed + k)
            rg = S.beacons(m, pose, 3, seed=seed + k)
            entries.append((pose, scan, rg))
        pools.append(entries)
    return pools


def run_load(server: Server, grids, pools, n_sessions: int, rate_hz: float, duration_s: float, churn_per_s: float,
             p_range=(1000, 100000), n_range=(500, 10000), seed=0, warmup_s=1.0, odom=None, max_queue=None):
    """Open-loop Poisson load; returns latency percentiles and aggregate throughput.

    A request's latency runs from its scheduled arrival time (not from when this loop
    got round to submitting it) to its result being ready, so a load generator that
    falls behind cannot hide queueing.  max_queue=None serves every scan; an integer
    skips a scan arriving while that many of the session's requests are waiting, as a
    node whose filter is busy does, and counts it in dropped_behind."""
    from . import synth as S

    rng = np.random.default_rng(seed)
    odom = odom if odom is not None else (*S.ODOM_MODS, 0.05, 0.0, 0.0, 0.01)
    specs = {}
    admission = []  # sessions waiting for room
    next_seed = [seed * 1000 + 1]

    def new_spec():
        gi = int(rng.integers(len(grids)))
        pose, scan, rg = pools[gi][int(rng.integers(len(pools[gi])))]
        P = log_uniform_int(rng, *p_range)
        n = min(log_uniform_int(rng, *n_range), scan.shape[0])
        next_seed[0] += 1
        return SessionSpec(gi, P, n, pose, next_seed[0]), scan[:n], rg

    def try_open(spec_scan):
        spec, scan, rg = spec_scan
        init8 = [spec.pose[0], spec.pose[1], spec.pose[2], spec.pose[3], 0.3, 0.3, 0.05, 0.1]
        sid = server.open_session(grids[spec.grid], spec.P, spec.seed, spec.P, init8)
        if sid is None:
            return False
        specs[sid] = (spec, scan, rg, server.prepare(sid, scan, rg, odom, 0.5, 0.1, 0.0, 0.0, True))
        return True

    for _ in range(n_sessions):
        s = new_spec()
        if not try_open(s):
            admission.append(s)
    t0 = time.perf_counter()
    counters0 = None
    events = []  # (time, kind, sid)
    for sid in list(specs):
        heapq.heappush(events, (t0 + rng.exponential(1.0 / rate_hz), 0, sid))
    next_churn = t0 + (1.0 / churn_per_s if churn_per_s > 0 else 1e18)
    outstanding = {}
    per_session = {}
    lat = []
    lat_srv = []  # from the submit call to the result (the server alone)
    weights = 0
    done_req = 0
    t_end = t0 + warmup_s + duration_s
    t_meas = t0 + warmup_s
    submitted = 0
    dropped = 0
    closing = []
    while True:
        now = time.perf_counter()
        if now >= t_end:
            break
        if counters0 is None and now >= t_meas:
            counters0 = server.counters()
        # completions
        for (ticket, sid, status, ts, td, mean) in server.poll():
            info = outstanding.pop(ticket, None)
            if info is None:
                continue
            per_session[sid] = per_session.get(sid, 1) - 1
            if td >= t_meas and status == 0:
                lat.append(td - info[1])
                lat_srv.append(td - ts)
                weights += info[0]
                done_req += 1
        # churn: one session leaves, a new one arrives (waiting for admission)
        if now >= next_churn and specs:
            next_churn += 1.0 / churn_per_s
            victim = list(specs)[int(rng.integers(len(specs)))]
            specs.pop(victim)
            closing.append(victim)
            admission.append(new_spec())
        for sid in list(closing):
            if per_session.get(sid, 0) == 0:  # nothing outstanding: closing does not block
                server.close_session(sid)
                closing.remove(sid)
        while admission and try_open(admission[0]):
            admission.pop(0)
            sid = max(specs)
            heapq.heappush(events, (now + rng.exponential(1.0 / rate_hz), 0, sid))
        # arrivals
        while events and events[0][0] <= now:
            t_arr, _, sid = heapq.heappop(events)
            if sid not in specs:
                continue
            spec, scan, rg, prepared = specs[sid]
            if max_queue is not None and per_session.get(sid, 0) >= max_queue:
                dropped += 1  # the session is that far behind: skip this scan, as the node's threshold gating does
            else:
                ticket = server.submit_prepared(prepared)
                outstanding[ticket] = (spec.P * scan.shape[0], t_arr)
                per_session[sid] = per_session.get(sid, 0) + 1
                submitted += 1
            heapq.heappush(events, (t_arr + rng.exponential(1.0 / rate_hz), 0, sid))
        sleep = min((events[0][0] if events else now + 0.001) - time.perf_counter(), 0.0005)
        if sleep > 0:
            time.sleep(sleep)
    for sid in list(specs):
        try:
            server.close_session(sid)
        except N.AmclError:
            pass
    backlog = len(outstanding)
    counters1 = server.counters()
    counters0 = counters0 or counters1
    lat = np.array(lat)
    lat_srv = np.array(lat_srv)
    st = server.stats()
    return {
        "sessions": n_sessions,
        "rate_hz": rate_hz,
        "duration_s": duration_s,
        "requests_measured": int(done_req),
        "submitted": int(submitted),
        "backlog_at_end": int(backlog),
        "weights_per_s": weights / duration_s,
        "p50_ms": float(np.percentile(lat, 50) * 1e3) if lat.size else None,
        "p99_ms": float(np.percentile(lat, 99) * 1e3) if lat.size else None,
        "server_p50_ms": float(np.percentile(lat_srv, 50) * 1e3) if lat_srv.size else None,
        "server_p99_ms": float(np.percentile(lat_srv, 99) * 1e3) if lat_srv.size else None,
        "mean_batch": st["requests"] / max(st["steps"], 1),
        "graphs_built_measured": counters1["graphs_built"] - counters0["graphs_built"],
        "reallocs_measured": counters1["reallocs"] - counters0["reallocs"],
        "max_batch": st["max_batch"],
        "admission_waiting": len(admission),
        "dropped_behind": int(dropped),
    }


def run_capacity(server: Server, grids, pools, n_sessions: int, duration_s: float, p_range=(1000, 100000),
                 n_range=(500, 10000), seed=0, depth=2, warmup_s=1.0, odom=None):
    """The server's capacity on the session mix: every session keeps `depth` requests
    queued (closed loop, so every step batches every session with work); returns the
    completed particle x point weights per second."""
    from . import synth as S

    rng = np.random.default_rng(seed)
    odom = odom if odom is not None else (*S.ODOM_MODS, 0.05, 0.0, 0.0, 0.01)
    specs = {}
    for _ in range(n_sessions):
        gi = int(rng.integers(len(grids)))
        pose, scan, rg = pools[gi][int(rng.integers(len(pools[gi])))]
        P = log_uniform_int(rng, *p_range)
        n = min(log_uniform_int(rng, *n_range), scan.shape[0])
        init8 = [pose[0], pose[1], pose[2], pose[3], 0.3, 0.3, 0.05, 0.1]
        sid = server.open_session(grids[gi], P, seed * 1000 + len(specs) + 1, P, init8)
        if sid is None:
            break
        specs[sid] = (P * n, server.prepare(sid, scan[:n], rg, odom, 0.5, 0.1, 0.0, 0.0, True))
    outstanding = {}

    def submit(sid):
        w, prepared = specs[sid]
        outstanding[server.submit_prepared(prepared)] = (sid, w)

    for sid in specs:
        for _ in range(depth):
            submit(sid)
    t0 = time.perf_counter()
    t_meas, t_end = t0 + warmup_s, t0 + warmup_s + duration_s
    weights, done = 0, 0
    while True:
        now = time.perf_counter()
        if now >= t_end:
            break
        got = server.poll()
        for (ticket, sid, status, ts, td, mean) in got:
            info = outstanding.pop(ticket, None)
            if info is None:
                continue
            if status == 0 and td >= t_meas:
                weights += info[1]
                done += 1
            submit(info[0])
        if not got:
            time.sleep(0.0002)
    deadline = time.perf_counter() + 60.0
    while outstanding and time.perf_counter() < deadline:  # drain before closing the sessions
        for (ticket, *_rest) in server.poll():
            outstanding.pop(ticket, None)
        time.sleep(0.0005)
    for sid in specs:
        server.close_session(sid)
    return {"sessions": len(specs), "depth": depth, "duration_s": duration_s, "requests": done,
            "weights_per_s": weights / duration_s}


def run_plain(grids, pools, n_requests: int, p_range=(1000, 100000), n_range=(500, 10000), seed=0, odom=None):
    """The same request mix served one filter per call: weights/s and per-call latency."""
    from . import synth as S

    rng = np.random.default_rng(seed)
    odom = odom if odom is not None else (*S.ODOM_MODS, 0.05, 0.0, 0.0, 0.01)
    filters = []
    for k in range(16):
        gi = int(rng.integers(len(grids)))
        pose, scan, rg = pools[gi][int(rng.integers(len(pools[gi])))]
        P = log_uniform_int(rng, *p_range)
        n = min(log_uniform_int(rng, *n_range), scan.shape[0])
        pf = ParticleFilter(seed=k + 1)
        pf.init(P, pose[0], pose[1], pose[2], pose[3], 0.3, 0.3, 0.05, 0.1)
        filters.append((pf, grids[gi], scan[:n], rg, P * n))
    for pf, g, scan, rg, _ in filters:  # warm-up
        pf.predict(*odom)
        pf.update(g, scan, rg, 0.5, 0.1, 0.0, 0.0)
        pf.getMean()
        pf.resample()
    lat = []
    weights = 0
    t0 = time.perf_counter()
    for r in range(n_requests):
        pf, g, scan, rg, w = filters[r % len(filters)]
        ts = time.perf_counter()
        pf.predict(*odom)
        pf.update(g, scan, rg, 0.5, 0.1, 0.0, 0.0)
        pf.getMean()
        pf.resample()
        lat.append(time.perf_counter() - ts)
        weights += w
    dt = time.perf_counter() - t0
    lat = np.array(lat)
    return {"weights_per_s": weights / dt, "p50_ms": float(np.percentile(lat, 50) * 1e3),
            "p99_ms": float(np.percentile(lat, 99) * 1e3), "requests": n_requests}


def run_plain_open(grids, pools, n_sessions: int, rate_hz: float, duration_s: float, p_range=(1000, 100000),
                   n_range=(500, 10000), seed=0, warmup_s=1.0, odom=None, max_queue=4):
    """The served workload without the server: one plain ParticleFilter per session,
    open-loop Poisson arrivals at rate_hz per session, requests handled one at a time
    in arrival order (predict, update, getMean, resample).  Latency runs from the
    request's arrival to its mean being read; a session with max_queue requests
    waiting drops the next scan, as the served run does."""
    import collections

    from . import synth as S

    rng = np.random.default_rng(seed)
    odom = odom if odom is not None else (*S.ODOM_MODS, 0.05, 0.0, 0.0, 0.01)
    sessions = {}
    for sid in range(n_sessions):
        gi = int(rng.integers(len(grids)))
        pose, scan, rg = pools[gi][int(rng.integers(len(pools[gi])))]
        P = log_uniform_int(rng, *p_range)
        n = min(log_uniform_int(rng, *n_range), scan.shape[0])
        pf = ParticleFilter(seed=seed * 1000 + sid + 1)
        pf.init(P, pose[0], pose[1], pose[2], pose[3], 0.3, 0.3, 0.05, 0.1)
        sessions[sid] = (pf, grids[gi], scan[:n], rg, P * n)
    pf, g, sc, rg, _ = sessions[0]
    pf.predict(*odom)
    pf.update(g, sc, rg, 0.5, 0.1, 0.0, 0.0)
    pf.getMean()
    pf.resample()
    t0 = time.perf_counter()
    events = [(t0 + rng.exponential(1.0 / rate_hz), sid) for sid in sessions]
    heapq.heapify(events)
    fifo = collections.deque()
    waiting = collections.Counter()
    lat, weights, done_req, dropped = [], 0, 0, 0
    t_meas, t_end = t0 + warmup_s, t0 + warmup_s + duration_s
    while True:
        now = time.perf_counter()
        if now >= t_end:
            break
        while events and events[0][0] <= now:
            t, sid = heapq.heappop(events)
            if max_queue is not None and waiting[sid] >= max_queue:
                dropped += 1
            else:
                fifo.append((t, sid))
                waiting[sid] += 1
            heapq.heappush(events, (t + rng.exponential(1.0 / rate_hz), sid))
        if not fifo:
            time.sleep(min(max(events[0][0] - now, 0.0), 0.0005))
            continue
        t_arr, sid = fifo.popleft()
        pf, g, sc, rg, w = sessions[sid]
        pf.predict(*odom)
        pf.update(g, sc, rg, 0.5, 0.1, 0.0, 0.0)
        pf.getMean()
        pf.resample()
        td = time.perf_counter()
        waiting[sid] -= 1
        if td >= t_meas:
            lat.append(td - t_arr)
            weights += w
            done_req += 1
    lat = np.array(lat)
    return {"weights_per_s": weights / duration_s, "requests": done_req, "dropped_behind": dropped,
            "backlog_at_end": len(fifo),
            "p50_ms": float(np.percentile(lat, 50) * 1e3) if lat.size else None,
            "p99_ms": float(np.percentile(lat, 99) * 1e3) if lat.size else None}
