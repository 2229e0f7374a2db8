#!/usr/bin/env python
"""Benchmark of the amcl3d particle-filter hot path on GB300.

One step = predict + update (cloud weights, range weights, blend, normalise, mean)
+ getMean + resample of one filter over one synthetic scan, the sequence the ROS
node runs per accepted scan (Node.cpp:154-182).  Metric: particle x point weights
per second (P * N per step / step time), whole job.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--config warehouse|hall|room|served]
                  [--impl ours|reference]

`value` times the steps with the scan already resident in HBM (CUDA events on the
filter's stream); `e2e` times the same steps through the C ABI with host buffers
(the scan copied host->device and the mean read back every step).  The default
workload is the large single-filter configuration (2000x2000x400-cell warehouse,
200k particles, 20k points); `room` is the CPU-runnable 400x400x100 case, `hall`
the warehouse's filter on a 410 MB grid (profiler captures), `served` the
multi-session server under open-loop load.  `--impl reference` times the
reference's CPU update arithmetic (the oracle's C restatement) on the host cores on
the same workload; its grid is built on the host (where the reference's 250 M-cell
limit rules out a full build, only the cells its timed sample reads).
Multi-GPU runs are independent replicas (one filter per GPU, no collective on the
data path), launched one process per GPU by torchrun.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

CONFIGS = {
    "room": dict(
        workload="plain single filter: 20x20x5 m room at 0.05 m (400x400x100 cells), 40 cuboids 0.3-3 m, "
                 "600 particles, 1000-point scan (32x32 beams, 15 m), 3 beacons, alpha 0.5",
        size_m=(20.0, 20.0, 5.0), n_boxes=40, box_range=(0.3, 3.0), max_box_height=None, P=600, n_elev=32,
        n_azim=32, max_range=15.0, N=1000, B=3, elev=(-25.0, 25.0)),
    "warehouse": dict(
        workload="large single filter: 100x100x20 m warehouse at 0.05 m (2000x2000x400 cells, FP32 grid), "
                 "2000 cuboid shelves/pillars, 200000 particles, 20000-point scan (64x312 beams, 40 m), "
                 "6 beacons, alpha 0.5",
        size_m=(100.0, 100.0, 20.0), n_boxes=2000, box_range=(0.3, 3.0), max_box_height=8.0, P=200000, n_elev=64,
        n_azim=312, max_range=40.0, N=20000, B=6, elev=(-20.0, 20.0)),
    # the warehouse's filter and scan over a smaller hall: the same cloud-weight launch
    # shape (200k particles x 20k points) on a 410 MB grid, small enough for a
    # multi-pass profiler capture, still larger than L2
    "hall": dict(
        workload="profiling case: 40x40x8 m hall at 0.05 m (800x800x160 cells, FP32 grid), 320 cuboids, "
                 "200000 particles, 20000-point scan (64x312 beams, 40 m), 6 beacons, alpha 0.5",
        size_m=(40.0, 40.0, 8.0), n_boxes=320, box_range=(0.3, 3.0), max_box_height=6.0, P=200000, n_elev=64,
        n_azim=312, max_range=40.0, N=20000, B=6, elev=(-20.0, 20.0)),
}
METRIC = "particle x point weights/s"
UNIT = "weights/s"
N_SCANS = 4


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---- workload ------------------------------------------------------------------------------------

def make_workload(cfg: dict, seed: int):
    from amcl3d_gb300 import synth as S

    t0 = time.perf_counter()
    m = S.make_map(seed, size_m=cfg["size_m"], res=0.05, n_boxes=cfg["n_boxes"], box_range=cfg["box_range"],
                   max_box_height=cfg["max_box_height"])
    pose = S.free_pose(m, seed + 1)
    scans, poses, odos = [], [], []
    p = pose.copy()
    for k in range(N_SCANS):
        s = S.ray_cast(m, p, n_elev=cfg["n_elev"], n_azim=cfg["n_azim"], elev_deg=cfg["elev"],
                       max_range=cfg["max_range"], n_max=cfg["N"], seed=seed + 10 + k)
        scans.append(s)
        poses.append(p.copy())
        d = S.odometry_step(seed + 100 + k)
        odos.append(d)
        p = p + np.array([math.cos(p[3]) * 0.02, math.sin(p[3]) * 0.02, 0.0, 0.0])
    parts = S.particles_around(pose, cfg["P"], seed + 2)
    ranges = [S.beacons(m, q, cfg["B"], seed=seed + 200 + k) for k, q in enumerate(poses)]
    occ_points = m.points
    info = dict(min=m.min, max=m.max, res=m.res, dims=m.dims, n_points=int(occ_points.shape[0]))
    del m
    log(f"workload generated in {time.perf_counter() - t0:.1f}s: {info['n_points']} occupied voxels, "
        f"scan sizes {[s.shape[0] for s in scans]}")
    return occ_points, info, scans, ranges, odos, parts


def shift_workload(workload, shift):
    """The workload with its map, particles and beacon anchors moved by `shift` (metres);
    the scans are in the sensor frame and stay as they are."""
    occ, info, scans, ranges, odos, parts = workload
    sh = np.asarray(shift, np.float64)
    info = dict(info)
    info["min"] = tuple(float(a + b) for a, b in zip(info["min"], sh))
    info["max"] = tuple(float(a + b) for a, b in zip(info["max"], sh))
    occ = (occ.astype(np.float64) + sh).astype(np.float32)
    parts = parts.copy()
    parts[:, :3] = (parts[:, :3].astype(np.float64) + sh).astype(np.float32)
    moved = []
    for rg in ranges:
        r = rg.copy()
        r[:, 1:4] = (r[:, 1:4].astype(np.float64) + sh).astype(np.float32)
        moved.append(r)
    return occ, info, scans, moved, odos, parts


# ---- clocks sampled during the timed region --------------------------------------------------------

class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ---- CPU baseline: the oracle's restatement of the reference, on host threads --------------------

REF_CELL_LIMIT = 250_000_000  # computeGrid refuses larger grids (PointCloudTools.cpp:103-105)
REF_SAMPLE = 16384             # particles of the reference path's timed sample


def cpu_update_timer(g, scan, rng, threads: int):
    """run(sample[, scan, ranges]): the reference's update arithmetic (oracle restatement,
    float running sums, libm trig/exp) over a particle sample, split over host threads."""
    import oracle as O

    def run(sample: np.ndarray, scan_k=None, rng_k=None):
        sc = scan if scan_k is None else scan_k
        rk = rng if rng_k is None else rng_k
        if threads <= 1:
            O.update_f32(sample, g, sc, rk, 0.5, 0.1, 0.0, 0.0, yaw_trig=0, exp_mode=0)
            return
        chunks = np.array_split(sample, threads)
        with ThreadPoolExecutor(threads) as ex:
            list(ex.map(lambda c: O.update_f32(c, g, sc, rk, 0.5, 0.1, 0.0, 0.0, yaw_trig=0, exp_mode=0)
                        if len(c) else None, chunks))

    return run


def time_sample(run, sample, N, seconds):
    """Repeats the sample until about half of `seconds` has passed; weights/s."""
    reps = 0
    t0 = time.perf_counter()
    while True:
        run(sample)
        reps += 1
        dt = time.perf_counter() - t0
        if dt >= 0.5 * seconds or reps >= 1000:
            break
    return reps * sample.shape[0] * N / dt, reps, dt


def cpu_baseline(g, scans, ranges, parts, seconds: float, threads: int | None = None):
    """Times the reference's update arithmetic on a particle sample, all host cores, on
    the grid read back from the GPU (g: oracle GridData).  Returns (rate, desc)."""
    threads = threads or os.cpu_count() or 1
    scan = scans[0]
    N = scan.shape[0]
    run = cpu_update_timer(g, scan, ranges[0], threads)
    # calibrate on a small sample, then size the timed sample to ~`seconds`
    cal = parts[: max(threads * 4, 64)]
    t0 = time.perf_counter()
    run(cal)
    dt = max(time.perf_counter() - t0, 1e-4)
    rate = cal.shape[0] * N / dt
    n_sample = int(min(parts.shape[0], max(threads * 8, rate * seconds / N)))
    rate, reps, dt = time_sample(run, parts[:n_sample], N, seconds)
    return rate, {
        "cores": threads,
        "kind": "port",
        "sample": f"{reps} x {n_sample} of {parts.shape[0]} particles x {N} points "
                  f"(C restatement of ParticleFilter::update with float running sums), {dt:.1f}s",
    }


def reference_grid(occ_points, info, sample, scan, threads: int, cell_limit: int = REF_CELL_LIMIT):
    """The grid the reference's CPU path reads, built on the host by the oracle's
    restatement of computeGrid: in full where the reference can build it itself, else
    (the warehouse's 1.6 G cells exceed its 250 M limit and would take hours on the
    host) only the cells the sample's weighting reads, every other cell left 0."""
    import oracle as O

    size = tuple(int(v) for v in info["dims"])
    cells = int(np.prod(size))
    if cells <= cell_limit:
        d, p = O.compute_grid(occ_points, info["min"], info["max"], info["res"], 0.05, exp_mode=0, threads=threads)
        return O.GridData(info["min"], info["max"], info["res"], size, p.ravel(), d.ravel()), "full"
    prob = np.zeros(cells, np.float32)  # pages are mapped only where written
    g = O.GridData(info["min"], info["max"], info["res"], size, prob)
    mark = np.zeros(cells, np.uint8)
    chunks = [sample[k:k + 256, :4] for k in range(0, sample.shape[0], 256)]

    def touched(c):
        _, cl = O.cloud_weights(g, c, scan, 0.0, 0.0, yaw_trig=0, cells=True)
        return np.unique(cl[cl >= 0])

    with ThreadPoolExecutor(threads) as ex:
        for u in ex.map(touched, chunks):
            mark[u] = 1
    idx = np.flatnonzero(mark).astype(np.uint64)
    del mark
    prob[idx] = O.grid_cell_probs(occ_points, info["min"], info["res"], 0.05, size, idx, exp_mode=0, threads=threads)
    return g, f"{idx.size} cells read by the sample (of {cells})"


def reference_config(cfg, info, n_points_mean, world):
    """The `config` object of both arms' JSON lines."""
    cells = int(np.prod(info["dims"]))
    return {"workload": cfg["workload"], "particles": cfg["P"], "points": int(n_points_mean), "grid_cells": cells,
            "beacons": cfg["B"], "parallelism": f"replicas x{world}",
            "l2": "flushed between steps (512 MB write)" if cells * 4 < 200 * 2**20 else
                  f"grid larger than L2 ({cells * 4 / 1e9:.2f} GB FP32)"}


# ---- our arm -----------------------------------------------------------------------------------

def load_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic(workload_key: str):
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        d = json.loads(p.read_text())
        v = d.get(workload_key, {}).get("cloud_weight_bytes_per_launch")
        return v
    return None


class FilterTiming:
    """The timed filter steps of one configuration on this GPU: predict + update (cloud
    and range weights, blend, normalise, mean) + getMean + resample per step, as the
    node runs them per accepted scan (Node.cpp:154-182).  `device` times the steps with
    the scans resident in HBM (CUDA events on the filter's stream); `e2e` times the same
    steps through the C ABI with host scans (copied in, the mean read back, every step),
    from the same particle set and generator state.  A grid that fits in L2 is flushed
    (a 512 MB write) before every timed step."""

    def __init__(self, cfg, seed, dev, workload=None):
        import amcl3d_gb300 as A
        from amcl3d_gb300 import synth as S

        self.cfg, self.seed, self.dev = cfg, seed, dev
        self.occ, self.info, self.scans, self.ranges, self.odos, self.parts = workload or make_workload(cfg, seed)
        self.G = A.Grid3d()
        t0 = time.perf_counter()
        self.G.buildGridMap(self.occ, self.info["min"], self.info["max"], self.info["res"], S.SENSOR_DEV)
        self.build_s = time.perf_counter() - t0
        self.pf = A.ParticleFilter(seed=seed)
        self.pf.set_particles(self.parts)

    def run(self, steps, warmup, world=1, barrier_fn=None, clocks_index=0):
        import ctypes as C

        import torch

        from amcl3d_gb300 import _native
        from amcl3d_gb300 import synth as S

        pf, G, dev = self.pf, self.G, self.dev
        stream = torch.cuda.ExternalStream(pf.stream(), device=dev)
        d_scans = [torch.from_numpy(np.ascontiguousarray(s)).to(dev) for s in self.scans]
        torch.cuda.synchronize()
        P = self.cfg["P"]
        cells = int(np.prod(self.info["dims"]))
        flush = torch.empty(512 * 2**20, dtype=torch.uint8, device=dev) if cells * 4 < 200 * 2**20 else None
        scans, ranges, odos = self.scans, self.ranges, self.odos

        def step(k, resident=True):
            i = k % N_SCANS
            pf.predict(*S.ODOM_MODS, *odos[i])
            if resident:
                rg = np.ascontiguousarray(ranges[i])
                _native.call("amcl_pf_update_dev", pf.handle, G.handle, C.c_void_p(d_scans[i].data_ptr()),
                             scans[i].shape[0], _native.fptr(rg), rg.shape[0], 0.5, 0.1, 0.0, 0.0)
            else:
                pf.update(G, scans[i], ranges[i], 0.5, 0.1, 0.0, 0.0)
            pf.getMean()
            pf.resample()

        pf.set_particles(self.parts)
        pf.set_option(4, self.seed)
        for k in range(warmup):
            step(k)
        torch.cuda.synchronize()
        pf.profile(True)
        pf.profile_read(reset=True)
        launches0 = _native.kernel_launches()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        weights = 0
        if barrier_fn:
            barrier_fn()
        torch.cuda.synchronize()
        with ClockSampler(clocks_index) as clocks:
            for k in range(steps):
                if flush is not None:
                    with torch.cuda.stream(stream):
                        flush.fill_(k & 0xFF)
                with torch.cuda.stream(stream):
                    ev[k][0].record(stream)
                step(warmup + k)
                with torch.cuda.stream(stream):
                    ev[k][1].record(stream)
                weights += P * scans[(warmup + k) % N_SCANS].shape[0]
            torch.cuda.synchronize()
        if barrier_fn:
            barrier_fn()
        ms = sum(a.elapsed_time(b) for a, b in ev)
        launches = _native.kernel_launches() - launches0
        prof = pf.profile_read(reset=True)
        pf.profile(False)

        pf.set_particles(self.parts)
        pf.set_option(4, self.seed)
        for k in range(warmup):
            step(k, resident=False)
        torch.cuda.synchronize()
        if barrier_fn:
            barrier_fn()
        e2e_weights = 0
        e2e_s = 0.0
        if flush is None:
            t0 = time.perf_counter()
            for k in range(steps):
                step(warmup + k, resident=False)
                e2e_weights += P * scans[(warmup + k) % N_SCANS].shape[0]
            torch.cuda.synchronize()
            e2e_s = time.perf_counter() - t0
        else:
            for k in range(steps):
                with torch.cuda.stream(stream):
                    flush.fill_((k + 1) & 0xFF)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                step(warmup + k, resident=False)
                torch.cuda.synchronize()
                e2e_s += time.perf_counter() - t0
                e2e_weights += P * scans[(warmup + k) % N_SCANS].shape[0]
        return {"ms": ms, "weights": weights, "launches": launches, "prof": prof, "clocks": clocks.summary(),
                "e2e_s": e2e_s, "e2e_weights": e2e_weights, "flushed": flush is not None}

    def grid_host(self):
        """The grid's probabilities read back (the oracle reads the GPU-built cells)."""
        import oracle as O

        cells = int(np.prod(self.info["dims"]))
        prob = np.empty(cells, np.float32)
        step = 1 << 28
        for first in range(0, cells, step):
            prob[first:first + min(step, cells - first)] = self.G.read_cells(first, min(step, cells - first))[1]
        return O.GridData(self.info["min"], self.info["max"], self.info["res"], self.info["dims"], prob)


def run_ours(args, cfg, rank, world, local_rank):
    import torch

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    seed = 1000 + rank
    ft = FilterTiming(cfg, seed, dev,
                      workload=shift_workload(make_workload(cfg, seed), args.map_shift) if args.map_shift else None)
    log(f"[rank {rank}] grid {ft.info['dims']} built on the GPU in {ft.build_s:.2f}s")
    if args.storage != "f32":
        ft.G.set_storage(args.storage)  # the headline filter gathers the narrower cells
    r = ft.run(args.steps, args.warmup, world, (lambda: barrier(world)) if world > 1 else None, local_rank)
    P = cfg["P"]
    ms_max = allreduce_max(r["ms"], world, dev)
    value = allreduce_sum(r["weights"], world, dev) / (ms_max / 1e3)
    e2e_s = allreduce_max(r["e2e_s"], world, dev)
    e2e_total = allreduce_sum(r["e2e_weights"], world, dev)
    h2d = int(np.mean([s.shape[0] for s in ft.scans]) * 16 + cfg["B"] * 16)
    d2h = 4 + 120  # status word + the mean/variance record
    prof = r["prof"]
    cw_ms, cw_n = prof["cloud_weight"]
    peak, peak_kind = load_peaks()
    N_mean = float(np.mean([s.shape[0] for s in ft.scans]))
    alg_bytes = P * N_mean * 4 + 28 * P + 16 * N_mean + 16 * cfg["B"] * P
    cw_launch_ms = cw_ms / cw_n if cw_n else None
    achieved = alg_bytes / (cw_launch_ms / 1e3) / 1e9 if cw_n else None
    issue = None if args.map_shift else load_issue_profile(args.config)  # profiled on the zero-minimum map
    res = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if args.storage == "f32" else f"{args.storage} grid, f32 arithmetic",
        "data": "synthetic (seeded room/warehouse maps, ray-cast scans; no public dataset)",
        "config": reference_config(cfg, ft.info, N_mean, world), "grid_build_s": round(ft.build_s, 3),
        "e2e": {"value": e2e_total / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": int(r["launches"]),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": None if args.map_shift else load_traffic(args.config),
                     "peak_source": peak_kind, "kernel": "cloud weight (per-particle scan gather)",
                     "kernel_ms_per_launch": cw_launch_ms,
                     "traffic_unit": "DRAM bytes per launch (ncu)",
                     "limiter": "instruction issue and dependent-instruction latency; the cell gathers are "
                                "L2-resident (ncu: >99% L2 hits), so the HBM line is not what binds",
                     "algorithmic_bytes_per_launch": alg_bytes},
        "kernel_ms": {k: (v[0] / v[1] if v[1] else None) for k, v in prof.items()},
        "clocks": r["clocks"],
    }
    if args.map_shift:
        res["config"]["map_minimum"] = ft.info["min"]
    if issue and cw_launch_ms:
        # the issue-side roof: warp instructions per particle x point (ncu) at the SMs'
        # full issue rate (one warp instruction per cycle per scheduler, 4 per SM)
        wpp = issue["warp_inst_per_particle_point"]
        inst = P * N_mean * wpp / 32.0
        mhz = r["clocks"].get("sm_mhz") or issue.get("sm_mhz_max", 2070.0)
        peak_inst = 4 * sm_count() * mhz * 1e6
        achieved_inst = inst / (cw_launch_ms / 1e3)
        res["roofline"]["binding_roof"] = "issue"
        res["roofline"]["issue"] = {
            "achieved_warp_inst_per_s": achieved_inst, "peak_warp_inst_per_s": peak_inst,
            "frac": achieved_inst / peak_inst, "warp_inst_per_particle_point": wpp,
            "ncu_issue_active": issue.get("issue_active"), "source": issue.get("source")}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        g_host = ft.grid_host()
        rate, desc = cpu_baseline(g_host, ft.scans, ft.ranges, ft.parts, seconds=args.cpu_seconds)
        res["cpu_baseline"] = {"value": rate, "unit": UNIT, **desc}
    else:
        g_host = None
    if rank == 0 and world == 1 and args.sections:
        t_sec = time.perf_counter()
        res["voxel_filter"] = voxel_section(seed + 5)
        res["grid_storage"] = storage_section(ft, seed, g_host)
        res["distance_field"] = distance_field_section(ft, seed)
        res["map_minimum"] = map_minimum_section(ft, seed, prof)
        del g_host
        res["room"] = room_section(seed + 3, dev)
        if args.served_sessions > 0:
            grids, maps = four_maps(ft, seed)
            pf_keep = ft.pf
            del pf_keep
            ft.pf = None
            res["batched"] = batched_section(grids, maps, seed + 9)
            res["small_filters"] = small_filters_section(grids[1], maps[1], seed + 11)
            res["served"] = served_section(grids, maps, args.served_sessions, args.served_duration)
        log(f"sections took {time.perf_counter() - t_sec:.1f}s")
    return res


def sm_count():
    import torch

    return torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count


def load_issue_profile(workload_key: str):
    p = ROOT / "profiles" / "issue.json"
    if p.exists():
        return json.loads(p.read_text()).get(workload_key) or json.loads(p.read_text()).get("hall")
    return None


def room_section(seed, dev, steps=100, warmup=3):
    """The plain single filter of the room (400x400x100 cells, 600 particles, ~1k-point
    scans, 3 beacons) for 100 steps: the GPU device-resident and end to end (L2 flushed
    before each step), the reference's CPU update arithmetic on one host thread over the
    same 100 steps, and the distance field built on the GPU against the oracle's
    computeGrid on one host thread (the reference's computeGrid is single-threaded)."""
    import oracle as O
    from amcl3d_gb300 import synth as S

    cfg = CONFIGS["room"]
    ft = FilterTiming(cfg, seed, dev)
    r = ft.run(steps, warmup)
    P = cfg["P"]
    out = {"workload": cfg["workload"], "steps": steps, "value": r["weights"] / (r["ms"] / 1e3),
           "ms_per_step": r["ms"] / steps, "e2e_value": r["e2e_weights"] / r["e2e_s"],
           "e2e_ms_per_step": r["e2e_s"] * 1e3 / steps, "l2": "flushed before each timed step (512 MB write)",
           "kernel_ms": {k: (v[0] / v[1] if v[1] else None) for k, v in r["prof"].items()},
           "gpu_launches": int(r["launches"]), "clocks": r["clocks"]}
    g = ft.grid_host()
    run1 = cpu_update_timer(g, None, None, 1)
    t0 = time.perf_counter()
    w = 0
    for k in range(steps):
        i = k % N_SCANS
        run1(ft.parts, ft.scans[i], ft.ranges[i])
        w += P * ft.scans[i].shape[0]
    cpu_s = time.perf_counter() - t0
    out["reference_cpu"] = {"value": w / cpu_s, "ms_per_step": cpu_s * 1e3 / steps, "cores": 1, "kind": "port",
                            "sample": f"all {steps} steps x {P} particles (C restatement of ParticleFilter::update, "
                                      "float running sums, one thread)"}
    out["gpu_over_reference"] = out["value"] / out["reference_cpu"]["value"]
    out["e2e_over_reference"] = out["e2e_value"] / out["reference_cpu"]["value"]
    # distance field of the whole room: GPU build vs the oracle's computeGrid on one thread
    cells = int(np.prod(ft.info["dims"]))
    t0 = time.perf_counter()
    O.compute_grid(ft.occ, ft.info["min"], ft.info["max"], ft.info["res"], S.SENSOR_DEV, exp_mode=0, threads=1)
    cpu_df = time.perf_counter() - t0
    out["distance_field"] = {"cells": cells, "occupied_points": int(ft.occ.shape[0]), "gpu_s": ft.build_s,
                             "reference_cpu_s": cpu_df, "reference_cores": 1,
                             "gpu_cells_per_s": cells / ft.build_s, "reference_cells_per_s": cells / cpu_df,
                             "gpu_over_reference": cpu_df / ft.build_s}
    return out


def distance_field_section(ft, seed):
    """computeGrid at the large size: the GPU's whole 1.6 G-cell build, and a 4x4x2 m
    (80x80x40-cell) sub-block around the robot built both ways: the GPU builds a grid
    over the sub-block's bounds from every occupied point, the oracle's computeGrid
    (one thread) computes the same cells of the full grid."""
    import amcl3d_gb300 as A
    import oracle as O
    from amcl3d_gb300 import synth as S

    info, occ, parts = ft.info, ft.occ, ft.parts
    sx, sy, sz = info["dims"]
    c = [int((float(np.mean(parts[:, a])) - info["min"][a]) / info["res"]) for a in range(3)]
    lo = (max(0, c[0] - 40), max(0, c[1] - 40), max(0, c[2] - 20))
    hi = (min(sx, lo[0] + 80), min(sy, lo[1] + 80), min(sz, lo[2] + 40))
    sub_cells = (hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2])
    t0 = time.perf_counter()
    O.compute_grid(occ, info["min"], info["max"], info["res"], S.SENSOR_DEV, lo=lo, hi=hi, exp_mode=0, threads=1)
    cpu_s = time.perf_counter() - t0
    res = info["res"]
    smin = tuple(info["min"][a] + lo[a] * res for a in range(3))
    smax = tuple(info["min"][a] + hi[a] * res for a in range(3))
    G2 = A.Grid3d()
    G2.buildGridMap(occ, smin, smax, res, S.SENSOR_DEV)  # warm (point upload path)
    t0 = time.perf_counter()
    G2.buildGridMap(occ, smin, smax, res, S.SENSOR_DEV)
    gpu_s = time.perf_counter() - t0
    del G2
    cells = sx * sy * sz
    return {"warehouse": {"cells": cells, "occupied_points": int(occ.shape[0]), "gpu_s": ft.build_s,
                          "gpu_cells_per_s": cells / ft.build_s,
                          "reference": "none: computeGrid refuses grids above 250 M cells (PointCloudTools.cpp:103-105)"},
            "subblock_4x4x2m": {"cells": sub_cells, "reference_cpu_s": cpu_s, "reference_cores": 1,
                                "reference_cells_per_s": sub_cells / cpu_s,
                                "gpu_s_at_full_build_rate": sub_cells / (cells / ft.build_s),
                                "gpu_over_reference_per_cell": (cells / ft.build_s) / (sub_cells / cpu_s),
                                "gpu_standalone_s": gpu_s,
                                "note": "the reference's computeGrid builds whole maps; the GPU's per-cell rate is "
                                        "its whole-warehouse build.  The standalone GPU build of a grid over just "
                                        "the sub-block's bounds is slow: all 22.8 M occupied points lie outside "
                                        "it and are bucketed into its edge buckets (exact, but every edge cell "
                                        "scans them)"}}


def map_minimum_section(ft, seed, zero_min_prof, steps=5, warmup=3, shift=(-17.35, -9.5, -1.4)):
    """The headline filter on its map moved so that the minimum is not zero, as a real
    octomap map's bounds are: the offsets double(t) - min are then no floats, and the cloud
    weighting takes the general yaw loop.  The same scans, particles and steps, the map,
    particles and beacon anchors moved by `shift`; cloud-weighting ms per launch against
    the headline's (zero minimum)."""
    import torch

    wl = shift_workload((ft.occ, ft.info, ft.scans, ft.ranges, ft.odos, ft.parts), shift)
    moved = FilterTiming(ft.cfg, seed, ft.dev, workload=wl)
    r = moved.run(steps, warmup)
    cw_ms, cw_n = r["prof"]["cloud_weight"]
    z_ms, z_n = zero_min_prof["cloud_weight"]
    out = {"minimum": wl[1]["min"], "cloud_weight_ms_per_launch": cw_ms / cw_n,
           "zero_minimum_ms_per_launch": z_ms / z_n, "ratio_to_zero_minimum": (cw_ms / cw_n) / (z_ms / z_n),
           "weights_per_s": r["weights"] / (r["ms"] / 1e3), "steps": steps,
           "loop": "general yaw loop: float estimate, floors widened 2^-22, float two-sum for open points"}
    del moved
    torch.cuda.empty_cache()
    return out


def four_maps(ft, seed):
    """The four maps of the batched and served configurations (200^3, 400x400x100,
    1000x1000x200 and the 2000x2000x400 warehouse, 0.05 m); the warehouse is the one
    already built."""
    import amcl3d_gb300 as A
    from amcl3d_gb300 import synth as S

    specs = [((10.0, 10.0, 10.0), 20, 6.0), ((20.0, 20.0, 5.0), 40, None), ((50.0, 50.0, 10.0), 400, 8.0)]
    maps, grids = [], []
    for k, (size, nb, hmax) in enumerate(specs):
        m = S.make_map(300 + k, size_m=size, n_boxes=nb, max_box_height=hmax)
        G = A.Grid3d()
        G.buildGridMap(m.points, m.min, m.max, m.res, S.SENSOR_DEV)
        maps.append(m)
        grids.append(G)
    cfg = ft.cfg
    wh = S.make_map(ft.seed, size_m=cfg["size_m"], res=0.05, n_boxes=cfg["n_boxes"], box_range=cfg["box_range"],
                    max_box_height=cfg["max_box_height"])
    maps.append(wh)
    grids.append(ft.G)
    return grids, maps


def small_filters_section(G, m, seed, n_filters=512, P=1000, N=500, steps=5):
    """Many small filters (1k particles, 500 points each, one room map): one batched
    step for all of them (scans staged from one packed host array) against the plain
    path stepping them one call at a time."""
    import amcl3d_gb300 as A
    from amcl3d_gb300 import synth as S
    from amcl3d_gb300.batch import FilterBatch

    pose = S.free_pose(m, seed)
    scan = S.ray_cast(m, pose, n_max=N, max_range=15.0, seed=seed + 1)
    rg = S.beacons(m, pose, 3, seed=seed + 2)
    odom = (*S.ODOM_MODS, 0.05, 0.0, 0.0, 0.01)
    B = FilterBatch(max_filters=n_filters, max_particles=n_filters * (P + 256), max_points_per_step=n_filters * N)
    slots = [B.add(G, P, seed * 1000 + f) for f in range(n_filters)]
    for sl in slots:
        B.init(sl, P, pose[0], pose[1], pose[2], pose[3], 0.3, 0.3, 0.05, 0.1)
    packed = np.ascontiguousarray(np.concatenate([scan] * n_filters))
    packed_rg = np.ascontiguousarray(np.concatenate([rg] * n_filters))
    counts = [scan.shape[0]] * n_filters
    rcounts = [rg.shape[0]] * n_filters
    t_stage = t_step = 0.0

    def bstep():
        nonlocal t_stage, t_step
        t0 = time.perf_counter()
        B.stage_packed(slots, packed, counts, packed_rg, rcounts, odom)
        t1 = time.perf_counter()
        B.step()
        B.wait()
        t_stage += t1 - t0
        t_step += time.perf_counter() - t1

    bstep()
    t_stage = t_step = 0.0
    for _ in range(steps):
        bstep()
    batched_s = (t_stage + t_step) / steps
    step_s = t_step / steps
    B.close()
    filters = [A.ParticleFilter(seed=seed * 1000 + f) for f in range(64)]
    for pf in filters:
        pf.init(P, pose[0], pose[1], pose[2], pose[3], 0.3, 0.3, 0.05, 0.1)

    def pstep(pf):
        pf.predict(*odom)
        pf.update(G, scan, rg, 0.5, 0.1, 0.0, 0.0)
        pf.getMean()
        pf.resample()

    for pf in filters:
        pstep(pf)
    t0 = time.perf_counter()
    for _ in range(steps):
        for pf in filters:
            pstep(pf)
    plain_per_filter = (time.perf_counter() - t0) / (steps * len(filters))
    w = P * scan.shape[0]
    return {"filters": n_filters, "particles": P, "points": int(scan.shape[0]),
            "batched_ms_per_step": batched_s * 1e3, "batched_weights_per_s": n_filters * w / batched_s,
            "batched_launch_and_wait_ms": step_s * 1e3, "batched_staging_ms": (batched_s - step_s) * 1e3,
            "batched_over_plain_launch_and_wait": (n_filters * w / step_s) / (w / plain_per_filter),
            "plain_ms_per_filter_step": plain_per_filter * 1e3, "plain_weights_per_s": w / plain_per_filter,
            "batched_over_plain": (n_filters * w / batched_s) / (w / plain_per_filter),
            "timing": "host wall clock per step, end to end: the batched step stages the 512 scans from one packed "
                      "host array (amcl_batch_stage_packed) and waits for the step; the plain steps copy their "
                      "scan inside update and read the mean back"}


def storage_section(ft, seed, g_host, steps=5, sample=64):
    """The large filter's step with the grid's probabilities gathered as FP32, FP16 and
    uint8 (amcl_grid_set_storage): cloud-weight kernel time, the gather bytes per second
    those cells amount to, the L1/L2 hit rates of an ncu capture per storage (hall map),
    and at every step the per-particle weights of a particle sample against the FP64
    oracle (the mean in double of the FP64 probabilities of the cells the reference's
    arithmetic selects)."""
    import amcl3d_gb300 as A
    import oracle as O
    from amcl3d_gb300 import synth as S

    pf, G, parts, scans, ranges, odos = ft.pf, ft.G, ft.parts, ft.scans, ft.ranges, ft.odos
    prof_cache = ROOT / "profiles" / "storage.json"
    ncu = json.loads(prof_cache.read_text()) if prof_cache.exists() else {}
    p64 = g_host.prob.astype(np.float64) if g_host is not None else None
    out = {}
    P = parts.shape[0]
    rng = np.random.default_rng(seed)
    for storage in ("f32", "f16", "u8"):
        G.set_storage(storage)
        pf.set_particles(parts)
        pf.set_option(4, seed)
        for k in range(2):
            pf.predict(*S.ODOM_MODS, *odos[k % N_SCANS])
            pf.update(G, scans[k % N_SCANS], ranges[k % N_SCANS], 0.5, 0.1, 0.0, 0.0)
            pf.resample()
        pf.profile(True)
        pf.profile_read(reset=True)
        weights, errs, errs_c = 0, [], []
        for k in range(steps):
            i = (2 + k) % N_SCANS
            pf.predict(*S.ODOM_MODS, *odos[i])
            if p64 is not None:
                # the sample: particles of this step's (predicted) set; their weights with the
                # reference's float running sum (computeCloudWeight) and with the compensated sum
                samp = pf.particles()[rng.choice(P, sample, replace=False)]
                pose4 = samp[:, :4]
                _, cells = O.cloud_weights(g_host, pose4, scans[i], 0.0, 0.0, yaw_trig=1, cells=True)
                exact = np.array([p64[c[c >= 0]].mean() if (c >= 0).sum() > 10 else 0.0 for c in cells])
                got = G.computeCloudWeights(pose4, scans[i]).astype(np.float64)
                mask = exact > 0
                errs.append(np.abs(got[mask] - exact[mask]) / exact[mask])
                side = A.ParticleFilter(seed=1)
                side.set_option(1, 1)
                side.set_particles(samp)
                side.update(G, scans[i], np.zeros((0, 4), np.float32), 1.0, 0.1, 0.0, 0.0)
                gotc = side.particles()[:, 5].astype(np.float64)  # normalised by the sample's exact sum
                want = exact / exact.sum()
                errs_c.append(np.abs(gotc[mask] - want[mask]) / want[mask])
                del side
            pf.update(G, scans[i], ranges[i], 0.5, 0.1, 0.0, 0.0)
            pf.getMean()
            pf.resample()
            weights += P * scans[i].shape[0]
        prof = pf.profile_read(reset=True)
        pf.profile(False)
        ms, n = prof["cloud_weight"]
        bpc = {"f32": 4, "f16": 2, "u8": 1}[storage]
        e = np.concatenate(errs) if errs else np.zeros(0)
        ec = np.concatenate(errs_c) if errs_c else np.zeros(0)
        out[storage] = {"cloud_weight_ms": ms / n, "weights_per_s": weights / (ms / 1e3), "bytes_per_cell": bpc,
                        "gather_bytes_per_s": weights * bpc / (ms / 1e3),
                        "ncu_hall": ncu.get(storage),
                        "weight_rel_err_vs_fp64": {
                            "running_sum_max": float(e.max()) if e.size else None,
                            "running_sum_mean": float(e.mean()) if e.size else None,
                            "compensated_sum_max": float(ec.max()) if ec.size else None,
                            "compensated_sum_mean": float(ec.mean()) if ec.size else None,
                            "particles": int(e.size), "steps": steps,
                            "note": "running sum: the reference's float sum in cloud order (computeCloudWeight); "
                                    "compensated: AMCL_OPT_CLOUD_SUM=1 (normalised weights of the sample, "
                                    "within 2x the per-particle error)"}}
    G.set_storage("f32")
    return out


def batched_section(grids, maps, seed, n_filters=256, p_range=(1000, 200000), n_range=(500, 20000), steps=100):
    """Batched uneven filters (amcl_batch_*): 256 filters over the four maps, P
    log-uniform 1k-200k, N log-uniform 500-20k, the batch autotuned once, then 100 steps,
    each timed by CUDA events around the graph launch on the batch's stream (device) and
    by the host clock including the staging of the 256 host scans (wall)."""
    import torch

    from amcl3d_gb300 import serve as SV
    from amcl3d_gb300 import synth as S
    from amcl3d_gb300.batch import FilterBatch

    rng = np.random.default_rng(seed)
    pools = SV.make_scan_pool(maps, seed, n_range[1])
    specs = []
    for f in range(n_filters):
        gi = int(rng.integers(len(grids)))
        pose, scan, rg = pools[gi][int(rng.integers(len(pools[gi])))]
        P = SV.log_uniform_int(rng, *p_range)
        n = min(SV.log_uniform_int(rng, *n_range), scan.shape[0])
        specs.append((gi, P, pose, scan[:n], rg))
    B = FilterBatch(max_filters=n_filters, max_particles=sum(s[1] for s in specs) + 256 * n_filters,
                    max_points_per_step=sum(s[3].shape[0] for s in specs))
    slots = []
    for f, (gi, P, pose, scan, rg) in enumerate(specs):
        sl = B.add(grids[gi], P, seed * 1000 + f)
        B.init(sl, P, pose[0], pose[1], pose[2], pose[3], 0.3, 0.3, 0.05, 0.1)
        slots.append(sl)
    odom = (*S.ODOM_MODS, 0.05, 0.0, 0.0, 0.01)
    packed = np.ascontiguousarray(np.concatenate([sp[3] for sp in specs]))
    packed_rg = np.ascontiguousarray(np.concatenate([sp[4] for sp in specs]))
    counts = [sp[3].shape[0] for sp in specs]
    rcounts = [sp[4].shape[0] for sp in specs]
    stream = torch.cuda.ExternalStream(B.stream())

    def step(ev=None):
        B.stage_packed(slots, packed, counts, packed_rg, rcounts, odom)
        if ev:
            ev[0].record(stream)
        B.step()
        if ev:
            ev[1].record(stream)
        B.wait()

    step()
    tuned = B.autotune(reps=2)
    step()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    t0 = time.perf_counter()
    for k in range(steps):
        step(evs[k])
    wall = (time.perf_counter() - t0) / steps
    dev_ms = sum(a.elapsed_time(b) for a, b in evs) / steps
    weights = sum(P * scan.shape[0] for (gi, P, pose, scan, rg) in specs)
    B.close()
    return {"filters": n_filters, "maps": [list(m.dims) for m in maps], "steps": steps,
            "particles": f"log-uniform {p_range}", "points": f"log-uniform {n_range}",
            "particles_total": int(sum(s[1] for s in specs)), "weights_per_step": int(weights),
            "device_ms_per_step": dev_ms, "weights_per_s": weights / (dev_ms / 1e3),
            "wall_ms_per_step": wall * 1e3, "wall_weights_per_s": weights / wall,
            "tuning": {"threads": tuned[0], "chunk": tuned[1]},
            "timing": "device: CUDA events around each step's graph launch on the batch stream (the graph "
                      "includes the step's host-to-device copies); wall: host clock per step including the "
                      "staging of the 256 host scans from one packed array and the wait"}


def voxel_section(seed: int, leaf: float = 0.1, reps: int = 20):
    """The scan filter the node runs before every update (pcl::VoxelGrid, Node.cpp:130-137)
    on a raw 64x2048-beam scan: GPU (host scan in, host centroids out, per call) against
    the oracle's single-threaded restatement of PCL's algorithm on the host."""
    import oracle as O

    import amcl3d_gb300 as A
    from amcl3d_gb300 import synth as S

    m = S.make_map(seed, size_m=(40.0, 40.0, 8.0), n_boxes=320, max_box_height=6.0)
    raw = S.ray_cast(m, S.free_pose(m, seed + 1), n_elev=64, n_azim=2048, max_range=40.0, n_max=64 * 2048,
                     seed=seed + 2)
    v = A.VoxelGrid()
    for _ in range(3):
        out = v.downsample(raw, leaf)
    t0 = time.perf_counter()
    for _ in range(reps):
        out = v.downsample(raw, leaf)
    gpu_ms = (time.perf_counter() - t0) / reps * 1e3
    exp, _ = O.voxel_downsample(raw, leaf)
    assert np.array_equal(out, exp), "voxel filter differs from the oracle"
    t0 = time.perf_counter()
    for _ in range(3):
        O.voxel_downsample(raw, leaf)
    cpu_ms = (time.perf_counter() - t0) / 3 * 1e3
    v.close()
    return {"points_in": int(raw.shape[0]), "points_out": int(out.shape[0]), "leaf_m": leaf,
            "gpu_ms_per_scan_e2e": gpu_ms, "cpu_port_ms_per_scan": cpu_ms, "cpu_cores": 1,
            "gpu_points_per_s": raw.shape[0] / (gpu_ms / 1e3)}


PLAIN_OPEN_MAX_SESSIONS = 400  # one plain filter (with its own weighting scratch) per session


def served_section(grids, maps, n_sessions, duration_s, rate_hz=10.0, churn_per_s=5.0, seed=7,
                   p_range=(1000, 100000), n_range=(500, 10000), lanes=4, storages=("f32", "f16")):
    """The served multi-session configuration on the four maps: n_sessions sessions at
    Poisson rate_hz each, churn_per_s joining and leaving, every scan served (nothing
    skipped), latency from each request's scheduled arrival to its result; per grid
    storage.  Beside it the server's capacity on the same mix (closed loop, every
    session always queued) and the plain one-filter-per-call path's closed-loop
    capacity on the same mix."""
    from amcl3d_gb300 import serve as SV

    pools = SV.make_scan_pool(maps, seed, n_range[1])
    mean_p = (p_range[1] - p_range[0]) / math.log(p_range[1] / p_range[0])
    mean_n = (n_range[1] - n_range[0]) / math.log(n_range[1] / n_range[0])

    def server(n):
        return SV.Server(max_sessions=n + 64, max_particles=int(n * mean_p * 4),
                         max_points_per_step=(n + 64) * n_range[1], lanes=lanes)

    out = {"sessions": n_sessions, "rate_hz_per_session": rate_hz, "duration_s": duration_s,
           "duration_note": f"{duration_s:.0f} s measured after 1 s of warm-up per storage (the configuration "
                            "names 5 minutes)", "churn_per_s": churn_per_s,
           "particles": f"log-uniform {p_range}", "points": f"log-uniform {n_range}", "lanes": lanes,
           "maps": [list(m.dims) for m in maps], "policy": "every scan served (no skipping)",
           "offered_weights_per_s": n_sessions * rate_hz * mean_p * mean_n}
    for storage in storages:
        for G in grids:
            G.set_storage(storage)
        srv = server(n_sessions)
        t0 = time.perf_counter()
        r = SV.run_load(srv, grids, pools, n_sessions, rate_hz, duration_s, churn_per_s, p_range, n_range, seed=seed)
        srv.close()
        log(f"served {n_sessions} sessions ({storage}) in {time.perf_counter() - t0:.1f}s: {r}")
        out[storage] = {k: r[k] for k in ("weights_per_s", "p50_ms", "p99_ms", "requests_measured", "submitted",
                                          "backlog_at_end", "mean_batch", "max_batch", "dropped_behind",
                                          "admission_waiting")}
        out[storage]["p99_within_15ms"] = bool(r["p99_ms"] is not None and r["p99_ms"] <= 15.0)
    for G in grids:
        G.set_storage("f32")
    srv = server(n_sessions)
    cap = SV.run_capacity(srv, grids, pools, n_sessions, 8.0, p_range, n_range, seed=seed)
    srv.close()
    plain = SV.run_plain(grids, pools, 400, p_range, n_range, seed=seed)
    log(f"served capacity {cap}; plain closed loop {plain}")
    out["capacity_weights_per_s"] = cap["weights_per_s"]
    out["capacity_note"] = ("closed loop: every session keeps 2 requests queued, FP32 grids, "
                            f"{cap['duration_s']:.0f} s")
    out["plain_capacity_weights_per_s"] = plain["weights_per_s"]
    out["plain_closed_loop_p50_ms"] = plain["p50_ms"]
    out["plain_closed_loop_p99_ms"] = plain["p99_ms"]
    out["served_over_plain_capacity"] = cap["weights_per_s"] / plain["weights_per_s"]
    return out


def run_served(args, rank, world, local_rank):
    """Served multi-session localization alone (--config served): sessions spread over
    the four maps (200^3, 400x400x100, 1000x1000x200, 2000x2000x400 cells)."""
    import torch

    import amcl3d_gb300 as A
    from amcl3d_gb300 import synth as S

    torch.cuda.set_device(local_rank)
    specs = [((10.0, 10.0, 10.0), 20, 6.0), ((20.0, 20.0, 5.0), 40, None), ((50.0, 50.0, 10.0), 400, 8.0),
             ((100.0, 100.0, 20.0), 2000, 8.0)]
    maps, grids = [], []
    for k, (size, nb, hmax) in enumerate(specs):
        m = S.make_map(300 + k, size_m=size, n_boxes=nb, max_box_height=hmax)
        G = A.Grid3d()
        G.buildGridMap(m.points, m.min, m.max, m.res, S.SENSOR_DEV)
        maps.append(m)
        grids.append(G)
    res = served_section(grids, maps, args.sessions, args.duration, args.rate, args.churn, lanes=args.lanes,
                         storages=(args.storage,))
    r = res[args.storage]
    return {"metric": METRIC + " (served)", "value": r["weights_per_s"], "unit": UNIT, "n_gpus": world,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {"f32": "f32", "f16": "f16 grid, f32 arithmetic", "u8": "u8 grid, f32 arithmetic"}[args.storage],
            "data": "synthetic", "config": {"workload": "served multi-session localization", "grid_storage": args.storage},
            "served": res}


def run_reference(args, cfg, rank, world):
    """The reference's CPU path (its arithmetic, restated in C: the reference tree
    cannot travel to this host) on all host cores, a bounded sample per step, on the
    same workload as our arm (same seeds); ms_per_step is the full filter's step at that
    rate, and the single-thread rate (the reference itself runs on one thread) is
    measured beside it."""
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    occ_points, info, scans, ranges, odos, parts = make_workload(cfg, 1000)
    sample = parts[: min(parts.shape[0], REF_SAMPLE)]
    t0 = time.perf_counter()
    g, grid_desc = reference_grid(occ_points, info, sample, scans[0], threads)
    log(f"reference grid ({grid_desc}) in {time.perf_counter() - t0:.1f}s")
    N = scans[0].shape[0]
    run = cpu_update_timer(g, scans[0], ranges[0], threads)
    rates, reps_total, dt_total = [], 0, 0.0
    for k in range(args.warmup + args.steps):
        rate, reps, dt = time_sample(run, sample, N, args.cpu_seconds / 4)
        if k >= args.warmup:
            rates.append(rate)
            reps_total += reps
            dt_total += dt
    value = float(np.mean(rates))
    # one thread, as the reference runs: a smaller sample
    one = sample[: min(sample.shape[0], 1024)]
    rate1, reps1, dt1 = time_sample(cpu_update_timer(g, scans[0], ranges[0], 1), one, N, 4.0)
    full_step_ms = parts.shape[0] * N / value * 1e3
    desc = {"cores": threads, "kind": "port",
            "sample": f"{args.steps} steps x {reps_total // max(args.steps, 1)} x {sample.shape[0]} of "
                      f"{parts.shape[0]} particles x {N} points (C restatement of ParticleFilter::update with "
                      f"float running sums), {dt_total:.1f}s; grid: {grid_desc}",
            "single_thread": {"value": rate1, "unit": UNIT,
                              "full_step_ms": parts.shape[0] * N / rate1 * 1e3,
                              "sample": f"{reps1} x {one.shape[0]} particles x {N} points, {dt1:.1f}s"}}
    return {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": full_step_ms,
        "ms_per_step_note": f"the full {parts.shape[0]}-particle step at the measured rate (each timed step ran "
                            f"a {sample.shape[0]}-particle sample)",
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded room/warehouse maps, ray-cast scans; no public dataset)",
        "config": reference_config(cfg, info, float(np.mean([sc.shape[0] for sc in scans])), world),
        "cpu_baseline": {"value": value, "unit": UNIT, **desc},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


# ---- distributed helpers ------------------------------------------------------------------------------

def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def allreduce_max(v, world, dev):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(v)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(v, world, dev):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(v)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", choices=sorted(CONFIGS) + ["served"], default="warehouse")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sessions", type=int, default=1000, help="served config: concurrent sessions")
    ap.add_argument("--rate", type=float, default=10.0, help="served config: requests/s per session")
    ap.add_argument("--duration", type=float, default=20.0, help="served config: measured seconds")
    ap.add_argument("--churn", type=float, default=5.0, help="served config: sessions joining/leaving per s")
    ap.add_argument("--lanes", type=int, default=4, help="served config: concurrent server lanes")
    ap.add_argument("--storage", choices=["f32", "f16", "u8"], default="f32",
                    help="grid storage the headline filter (or the served config) gathers")
    ap.add_argument("--map-shift", type=lambda t: tuple(float(v) for v in t.split(",")), default=None,
                    help="dx,dy,dz: move the map (and particles, beacons) so that its minimum is not zero, as a "
                         "real map's is; the cloud weighting then takes the general yaw loop")
    ap.add_argument("--served-sessions", type=int, default=1000,
                    help="sessions of the served section of the default line (0: skip the batched, small-filter "
                         "and served sections)")
    ap.add_argument("--served-duration", type=float, default=20.0,
                    help="measured seconds per grid storage of the served section of the default line")
    ap.add_argument("--no-sections", dest="sections", action="store_false",
                    help="only the headline measurement (no voxel, storage, distance-field, room, batched, "
                         "small-filter or served sections)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.config == "served":
        if rank == 0:
            out = ({"impl": "reference", "unavailable": "the reference serves one filter per ROS node; it has no "
                    "multi-session server to time"} if args.impl == "reference" else
                   run_served(args, rank, 1, local_rank))
            print(json.dumps(out), flush=True)
        return
    cfg = CONFIGS[args.config]
    if args.impl == "reference":
        res = run_reference(args, cfg, rank, world)
        if rank == 0 and res:
            print(json.dumps(res), flush=True)
        return
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    res = run_ours(args, cfg, rank, world, local_rank)
    if rank == 0:
        print(json.dumps(res), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
