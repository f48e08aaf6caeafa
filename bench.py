#!/usr/bin/env python3
"""Benchmark of the ProbabilisticMap scan path on one GB300.

Workload (default ``multimap``): 64 independent ProbabilisticMaps of uneven
size, each receiving one insertPointCloud scan per tick -- points per map
log-uniform in [10k, 500k], drawn from the room and LiDAR generators,
resolutions cycling 0.02 / 0.05 / 0.1 m, max range 10 m, default Options --
for 50 ticks (``--steps``). Every tick runs through the batched form (one
graph-replayed persistent launch for all 64 scans) and through the plain
per-scan path (64 synchronous insertPointCloud calls) on identical inputs; the
two sets of maps are compared bit-exactly after the run.

Metric: ray-cell updates/s, V / t with V = points + sum of cast ray lengths
(the count the reference's own loop performs, identical on CPU and GPU).

* ``value``: batched ticks, device time (CUDA events around the tick on the
  batch's stream), points resident in HBM, L2 flushed (256 MiB write) before
  every tick. ``plain_per_scan_value`` is the same for the per-scan path
  (summed device time of its scans) and ``batched_over_plain`` their ratio;
  ``wall`` gives both timed on the host around the calls.
* ``e2e``: the batched ticks from pinned host memory through the C ABI
  (host->device copy of the points and read-back of the counters inside).
* ``tick_ms_p50`` / ``tick_ms_p99``: latency of one batched tick call.
* ``roofline``: k_tick, algorithmic bytes per tick over its event-timed
  duration, against the measured HBM copy bandwidth.
* ``cpu_baseline``: the CPU path (the oracle restatement, timed against the
  reference in profiles/cpu_port_vs_ref.md) on all host cores, whole maps
  per process, one tick or more.

Other workloads (``--workload``): ``lidar`` (one map, 64x2048 LiDAR scans),
``depth`` (640x480 depth frames, then 1 M isOccupied), ``room``
(VoxelGrid<float> create/update/iterate), ``serve`` (32 Poisson clients).

``--impl reference`` times the CPU path alone on the same workload (all host
cores for ``multimap``). Under torchrun with N > 1 the maps are sharded
across ranks (``multimap``) or each rank runs a replica (``lidar``); ``value``
sums the ranks' ray-cell updates over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

L2_FLUSH_BYTES = 256 << 20
RAY_LIST_BYTES = 16          # one int4 per cast ray
CELL_RMW_BYTES = 8           # 4-byte cell word read + written
LEAF_MASK_BYTES = 64         # new leaf: its 512-bit mask is written by the kernel


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during a region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
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
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        loaded = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def lidar_scans(n_scans=20):
    from bonxai_gb300 import synth
    scene = synth.LidarScene()
    scans = [scene.scan(k) for k in range(n_scans)]
    return scene, scans


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic():
    """Per-scan DRAM bytes of the ray phase from the committed ncu summary."""
    p = ROOT / "profiles" / "ray_phase_lidar_traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            return None
    return None


def cpu_sample(scene, scans, seconds=10.0):
    """CPU oracle (single thread): passes over the 20-scan sequence, each on a
    fresh map, until about `seconds` of CPU work (at least one pass).
    Returns (ray-cell updates, seconds, scans)."""
    from oracle import oracle as O
    port = O.port()
    V, dt, n = 0, 0.0, 0
    while dt < seconds or n == 0:
        m = port.pmap(scene.resolution)
        for pts, o in scans:
            t0 = time.perf_counter()
            V += m.insert(pts, o, scene.max_range)
            dt += time.perf_counter() - t0
            n += 1
            if dt >= seconds and n >= len(scans):
                break
        del m
    return V, dt, n


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    scene, scans = lidar_scans(max(args.steps, args.warmup, 1) if args.steps < 20 else 20)
    from oracle import oracle as O
    port = O.port()
    m = port.pmap(scene.resolution)
    for k in range(args.warmup):
        pts, o = scans[k % len(scans)]
        m.insert(pts, o, scene.max_range)
    m = port.pmap(scene.resolution)
    V, t = 0, 0.0
    for k in range(args.steps):
        if k and k % len(scans) == 0:
            m = port.pmap(scene.resolution)
        pts, o = scans[k % len(scans)]
        t0 = time.perf_counter()
        V += m.insert(pts, o, scene.max_range)
        t += time.perf_counter() - t0
    value = V / t
    line = {
        "impl": "reference", "metric": "ray-cell updates/s", "value": value,
        "unit": "ray-cell updates/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": workload_config(scene),
        "cpu_baseline": {"value": value, "unit": "ray-cell updates/s", "cores": 1,
                         "kind": "port",
                         "sample": f"{args.steps} scans of the 20-scan sequence, one thread "
                                   "(the reference's scan is single-threaded per map)"},
        "e2e": {"value": value, "unit": "ray-cell updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def unique_ray_updates(bx, cfg, resolution, scans, max_range):
    """Cells the ray phase of each scan updates, counted once per cell (the
    kernel's own counter also counts racing lanes that both store the same
    word). A cell changes update_id to the scan's u exactly when the scan
    updates it; the endpoint phase updates one cell per cast ray. Replays the
    sequence on a fresh map outside any timed region."""
    m = bx.ProbabilisticMap(resolution, cfg)
    out = []
    _, cells = m.dump(sort=False)
    for pts, o in scans:
        u = m.update_count
        before = int(np.count_nonzero((cells & 0xF) == u))
        m.insert_point_cloud(pts, o, max_range)
        rays = m.last_stats()["cast_rays"]
        _, cells = m.dump(sort=False)
        after = int(np.count_nonzero((cells & 0xF) == u))
        out.append(after - before - rays)
    m.close()
    return out


def workload_config(scene):
    return {"workload": "lidar_64x2048_20scan", "points_per_scan": 131072,
            "resolution_m": scene.resolution, "max_range_m": scene.max_range,
            "scene": "40x40x8 m, 200 boxes, floor", "map": "one ProbabilisticMap",
            "l2": "flushed before every timed scan (256 MiB write)"}


def run_ours(args):
    import torch
    import bonxai_gb300 as bx

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.device("cuda", torch.cuda.current_device())

    scene, scans = lidar_scans(20)
    d_scans = [(torch.from_numpy(p).to(dev), o) for p, o in scans]
    h_scans = [(torch.from_numpy(p).pin_memory(), o) for p, o in scans]
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=dev)

    cfg = bx.Config(flags=bx.FLAG_TIMING | args.flags, rays_per_warp=args.rays_per_warp,
                    ray_unroll=args.ray_unroll, block_size=args.block_size,
                    initial_leaves=1 << 19, initial_inners=1 << 15, hash_buckets=1 << 15)
    m = bx.ProbabilisticMap(scene.resolution, cfg)
    mr = scene.max_range

    # warm-up
    for k in range(args.warmup):
        pts, o = d_scans[k % 20]
        m.insert_point_cloud(pts, o, mr)
    m.clear()

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    # ---------------- value: device-resident inputs
    launches0 = m.last_stats()["launches"]
    V_total, dev_ms, ray_ms, per_scan = 0, 0.0, [], []
    leaves_prev = 0
    barrier()
    t_wall0 = time.perf_counter()
    with ClockSampler(dev.index) as clk:
        for k in range(args.steps):
            if k and k % 20 == 0:
                m.clear()
                leaves_prev = 0
            flush.fill_(k)
            torch.cuda.synchronize()
            pts, o = d_scans[k % 20]
            V = m.insert_point_cloud(pts, o, mr)
            t = m.kernel_times()
            st = m.last_stats()
            V_total += V
            dev_ms += sum(t)
            ray_ms.append(t[3])
            new_leaves = st["leaves"] - leaves_prev
            leaves_prev = st["leaves"]
            per_scan.append((k % 20, st["cast_rays"], max(new_leaves, 0)))
    barrier()
    t_wall = time.perf_counter() - t_wall0
    launches = m.last_stats()["launches"] - launches0
    clocks = clk.summary()

    if ws > 1:
        import torch.distributed as dist
        tt = torch.tensor([dev_ms, float(V_total)], dtype=torch.float64, device=dev)
        mx = tt.clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        sm = tt.clone()
        dist.all_reduce(sm, op=dist.ReduceOp.SUM)
        dev_ms_all, V_all = float(mx[0]), float(sm[1])
    else:
        dev_ms_all, V_all = dev_ms, float(V_total)
    value = V_all / (dev_ms_all / 1e3)

    # ---------------- e2e: host buffers through the C ABI, on a map configured
    # as a user's would be (no per-kernel timing events)
    if args.no_e2e:
        h_scans = h_scans[:0]
    m.close()
    m = bx.ProbabilisticMap(scene.resolution, bx.Config(
        flags=args.flags, rays_per_warp=args.rays_per_warp, ray_unroll=args.ray_unroll,
        block_size=args.block_size, initial_leaves=1 << 19, initial_inners=1 << 15,
        hash_buckets=1 << 15))
    for k in range(min(3, args.warmup) if h_scans else 0):
        m.insert_point_cloud(h_scans[k][0].numpy(), h_scans[k][1], mr)
    m.clear()
    barrier()
    V_e2e, t_e2e = 0, 1e-30
    for k in range(args.steps if h_scans else 0):
        if k and k % 20 == 0:
            m.clear()
        flush.fill_(k)
        torch.cuda.synchronize()
        pts, o = h_scans[k % 20]
        arr = pts.numpy()
        t0 = time.perf_counter()
        V_e2e += m.insert_point_cloud(arr, o, mr)
        t_e2e += time.perf_counter() - t0
    barrier()
    if ws > 1:
        import torch.distributed as dist
        tt = torch.tensor([t_e2e, float(V_e2e)], dtype=torch.float64, device=dev)
        mx = tt.clone()
        dist.all_reduce(mx, op=dist.ReduceOp.MAX)
        sm = tt.clone()
        dist.all_reduce(sm, op=dist.ReduceOp.SUM)
        t_e2e, V_e2e = float(mx[0]), float(sm[1])
    e2e = V_e2e / t_e2e

    if rank != 0:
        return 0

    # algorithmic bytes of each timed ray phase, with the cells it updates
    # counted once (replayed on a fresh map after the timed regions)
    uniq = unique_ray_updates(bx, cfg, scene.resolution, d_scans, mr)
    ray_bytes = sum(RAY_LIST_BYTES * r + CELL_RMW_BYTES * uniq[j] + LEAF_MASK_BYTES * nl
                    for j, r, nl in per_scan)
    ray_bytes_ra = sum(16 * r + 64 * uniq[j] for j, r, nl in per_scan)
    peak, peak_kind = peaks()
    avg_ray_ms = sum(ray_ms) / len(ray_ms)
    bytes_per_launch = ray_bytes / len(ray_ms)
    achieved = bytes_per_launch / (avg_ray_ms / 1e3) / 1e9
    tr = ncu_traffic()
    roofline = {
        "kernel": "k_mark + k_apply_rays (ray phase: mark the ray cells, apply per leaf)",
        "bound": "hbm", "achieved": achieved,
        "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
        "traffic": tr.get("dram_bytes_per_launch") if tr else None,
        "algorithmic_bytes_per_launch": bytes_per_launch,
        "random_access_bytes_per_launch": ray_bytes_ra / len(ray_ms),
        "ray_kernel_ms": avg_ray_ms,
        "ray_kernel_share_of_scan": sum(ray_ms) / dev_ms,
        "unique_ray_cells_updated_per_scan": float(np.mean(uniq)),
    }
    cpu = None
    if not args.no_cpu:
        Vc, tc, nc = cpu_sample(scene, scans, args.cpu_seconds)
        cpu = {"value": Vc / tc, "unit": "ray-cell updates/s", "cores": 1, "kind": "port",
               "sample": f"{nc} scans (passes over the 20-scan sequence, fresh map per "
                         f"pass), one thread, {tc:.1f} s"}
    line = {
        "metric": "ray-cell updates/s", "value": value, "unit": "ray-cell updates/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dev_ms_all / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": dict(workload_config(scene), parallelism=f"replicas x{ws}",
                       rays_per_warp=args.rays_per_warp, ray_unroll=args.ray_unroll),
        "roofline": roofline, "cpu_baseline": cpu,
        "e2e": None if args.no_e2e else {"value": e2e, "unit": "ray-cell updates/s",
                "h2d_bytes_per_step": 131072 * 12, "d2h_bytes_per_step": 128,
                "ms_per_step": 1e3 * t_e2e / args.steps},
        "gpu_launches": launches, "clocks": clocks,
        "wall_s_timed_region": t_wall,
        "ray_cells_per_step": V_all / args.steps / ws,
    }
    print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


# ----------------------------------------------------------------------------
# room workload: VoxelGrid<float> create / update / iterate (300k points)
# ----------------------------------------------------------------------------
def run_room(args):
    """VoxelGrid<float> at 0.02 m, (2,3) bits, 300,000 points of a 6x4x3 m room
    with 20 spheres: create (setValue of U[0,1) values at posToCoord of the
    points on a cleared grid), update (setValue of new values), iterate
    (forEachCell as a dump of coordinates and values into device buffers).
    One step = the three phases; metric = grid items/s = (2 x points + cells
    dumped) / device time."""
    import ctypes as C
    import torch
    import bonxai_gb300 as bx
    from bonxai_gb300 import synth
    ws, rank, local = dist_env()
    torch.cuda.set_device(local if ws > 1 else 0)
    dev = torch.device("cuda", torch.cuda.current_device())
    s = torch.cuda.Stream()
    pts = synth.room_cloud(300_000, seed=1000)
    g0 = bx.VoxelGrid(0.02, 2, 3, np.float32)
    coords = torch.from_numpy(g0.pos_to_coord(pts)).to(dev)
    g0.close()
    vals = [torch.from_numpy(synth.room_values(len(pts), seed=1000 + k)).to(dev)
            for k in range(2)]
    g = bx.VoxelGrid(0.02, 2, 3, np.float32,
                     bx.Config(stream=s.cuda_stream, initial_leaves=1 << 14))
    lib = g.lib
    n = len(pts)
    out_xyz = torch.empty((n, 3), dtype=torch.int32, device=dev)
    out_val = torch.empty(n, dtype=torch.float32, device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=dev)
    got = C.c_size_t()

    def step(k):
        g.clear()
        flush.fill_(k)
        torch.cuda.synchronize()
        e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        e[0].record(s)
        g._check(lib.bxg_grid_set_values(g.h, C.c_void_p(coords.data_ptr()),
                                         C.c_void_p(vals[0].data_ptr()), n, None))
        e[1].record(s)
        g._check(lib.bxg_grid_set_values(g.h, C.c_void_p(coords.data_ptr()),
                                         C.c_void_p(vals[1].data_ptr()), n, None))
        e[2].record(s)
        g._check(lib.bxg_grid_dump(g.h, C.c_void_p(out_xyz.data_ptr()),
                                   C.c_void_p(out_val.data_ptr()), n, C.byref(got)))
        e[3].record(s)
        torch.cuda.synchronize()
        return [e[i].elapsed_time(e[i + 1]) for i in range(3)], got.value

    for k in range(args.warmup):
        step(k)
    phase = np.zeros(3)
    cells = 0
    with ClockSampler(dev.index) as clk:
        for k in range(args.steps):
            t, c = step(k)
            phase += t
            cells = c
    clocks = clk.summary()
    ms = float(phase.sum()) / args.steps
    items = 2 * n + cells
    value = items / (ms / 1e3)
    roots, leaves = g.node_counts()
    # algorithmic bytes: create 16 B/point in + 4 B/cell written + 64 B mask per
    # leaf; update 16 B/point + 4 B/cell; iterate 64 B mask per leaf + 4 B per
    # cell read + 16 B per cell out
    b_create = 16 * n + 4 * cells + 64 * leaves
    b_update = 16 * n + 4 * cells
    b_iter = 64 * leaves + 20 * cells
    pk, pkind = peaks()
    ph = phase / args.steps
    dom = int(np.argmax(ph))
    b_dom = [b_create, b_update, b_iter][dom]
    ach = b_dom / (ph[dom] / 1e3) / 1e9
    # e2e: host coordinates and values through the C ABI, dump to host
    h_coords = coords.cpu().numpy()
    h_vals = [v.cpu().numpy() for v in vals]
    h_xyz = np.empty((n, 3), np.int32)
    h_out = np.empty(n, np.float32)
    t_e2e = 0.0
    for k in range(args.steps):
        g.clear()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g._check(lib.bxg_grid_set_values(g.h, h_coords.ctypes.data_as(C.c_void_p),
                                         h_vals[0].ctypes.data_as(C.c_void_p), n, None))
        g._check(lib.bxg_grid_set_values(g.h, h_coords.ctypes.data_as(C.c_void_p),
                                         h_vals[1].ctypes.data_as(C.c_void_p), n, None))
        g._check(lib.bxg_grid_dump(g.h, h_xyz.ctypes.data_as(C.c_void_p),
                                   h_out.ctypes.data_as(C.c_void_p), n, C.byref(got)))
        t_e2e += time.perf_counter() - t0
    e2e = items * args.steps / t_e2e
    cpu = None
    if not args.no_cpu:
        from oracle import oracle as O
        port = O.port()
        og = port.grid(0.02, 2, 3, O.ORC_F32)
        t0 = time.perf_counter()
        og.set_values(h_coords, h_vals[0])
        og.set_values(h_coords, h_vals[1])
        xyz_c, _ = og.dump()
        tc = time.perf_counter() - t0
        cpu = {"value": (2 * n + len(xyz_c)) / tc, "unit": "grid items/s", "cores": 1,
               "kind": "port", "sample": f"one create+update+iterate, one thread, {tc:.2f} s"}
    if rank != 0:
        return 0
    line = {
        "metric": "grid items/s (setValue create + update + forEachCell)", "value": value,
        "unit": "grid items/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "room_300k_voxelgrid_float", "points": n, "resolution_m": 0.02,
                   "inner_bits": 2, "leaf_bits": 3, "room": "6x4x3 m, 20 spheres",
                   "l2": "flushed before every step (256 MiB write); the grid (~"
                         f"{(leaves * 2112) >> 20} MiB) fits L2, so phases 2-3 hit it",
                   "parallelism": f"replicas x{ws}"},
        "phase_ms": {"create": ph[0], "update": ph[1], "iterate": ph[2]},
        "cells": cells, "leaves": leaves, "roots": roots,
        "roofline": {"kernel": ["create", "update", "iterate"][dom], "bound": "hbm",
                     "achieved": ach, "peak": pk, "unit": "GB/s", "frac": ach / pk,
                     "peak_kind": pkind, "traffic": None,
                     "algorithmic_bytes_per_launch": b_dom},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e, "unit": "grid items/s",
                "h2d_bytes_per_step": 2 * n * 16, "d2h_bytes_per_step": cells * 16},
        "gpu_launches": None, "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    g.close()
    return 0


# ----------------------------------------------------------------------------
# depth workload: 640x480 camera frames, then 1 M isOccupied lookups
# ----------------------------------------------------------------------------
def run_depth(args):
    """ProbabilisticMap at 0.02 m, max_range 5 m: 640x480 pinhole depth frames
    (fx = fy = 525) of an 8x6x3 m room with 50 boxes along a 6-DoF random walk
    (one step = one frame, invalid pixels dropped), then isOccupied on 1 M
    coordinates drawn uniformly in the final map's cell box. value = ray-cell
    updates/s of the frames; "lookup" = the lookups, device-resident."""
    import ctypes as C
    import torch
    import bonxai_gb300 as bx
    from bonxai_gb300 import synth
    ws, rank, local = dist_env()
    torch.cuda.set_device(local if ws > 1 else 0)
    dev = torch.device("cuda", torch.cuda.current_device())
    room = synth.DepthRoom()
    n_frames = min(max(args.steps, 1), 20) + args.warmup  # timed frames cycle through 20
    frames = [room.frame(k) for k in range(n_frames)]
    d_frames = [(torch.from_numpy(p).to(dev), o) for p, o in frames]
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=dev)
    m = bx.ProbabilisticMap(room.resolution,
                            bx.Config(flags=bx.FLAG_TIMING | args.flags,
                                      rays_per_warp=args.rays_per_warp,
                                      ray_unroll=args.ray_unroll, block_size=args.block_size,
                                      initial_leaves=1 << 18))
    for k in range(args.warmup):
        m.insert_point_cloud(*d_frames[k], room.max_range)
    m.clear()
    V, ms, ray_ms = 0, 0.0, []
    with ClockSampler(dev.index) as clk:
        for k in range(args.steps):
            flush.fill_(k)
            torch.cuda.synchronize()
            if k and k % 20 == 0:
                m.clear()
            V += m.insert_point_cloud(*d_frames[args.warmup + k % 20], room.max_range)
            t = m.kernel_times()
            ms += sum(t)
            ray_ms.append(t[3])
    clocks = clk.summary()
    value = V / (ms / 1e3)
    xyz, _ = m.dump(sort=False)
    q = torch.from_numpy(synth.lookup_coords(xyz.min(0), xyz.max(0), 1 << 20, seed=3)).to(dev)
    out = torch.empty(q.shape[0], dtype=torch.uint8, device=dev)
    s = torch.cuda.ExternalStream(m.stream)
    lib = m.lib
    look, call = [], []
    for k in range(args.warmup + args.steps):
        flush.fill_(k)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        m._check(lib.bxg_pmap_is_occupied(m.h, C.c_void_p(q.data_ptr()), q.shape[0],
                                          C.c_void_p(out.data_ptr())))
        b.record(s)
        torch.cuda.synchronize()
        if k >= args.warmup:
            look.append(m.last_query_ms())  # the lookup kernel alone
            call.append(a.elapsed_time(b))  # the synchronous call on the stream
    lk_ms = float(np.median(look))
    nq = q.shape[0]
    pk, pkind = peaks()
    lk_ach = 17.0 * nq / (lk_ms / 1e3) / 1e9
    # e2e: host points through the C ABI
    t_e2e, V_e2e = 0.0, 0
    m.clear()
    for k in range(args.steps):
        if k and k % 20 == 0:
            m.clear()
        p, o = frames[args.warmup + k % 20]
        t0 = time.perf_counter()
        V_e2e += m.insert_point_cloud(p, o, room.max_range)
        t_e2e += time.perf_counter() - t0
    cpu = None
    if not args.no_cpu:
        from oracle import oracle as O
        om = O.port().pmap(room.resolution)
        t0 = time.perf_counter()
        Vc = sum(om.insert(*frames[args.warmup + k], room.max_range)
                 for k in range(min(3, args.steps, 20)))
        tc = time.perf_counter() - t0
        cpu = {"value": Vc / tc, "unit": "ray-cell updates/s", "cores": 1, "kind": "port",
               "sample": f"{min(3, args.steps)} frames, one thread, {tc:.2f} s"}
    if rank != 0:
        return 0
    line = {
        "metric": "ray-cell updates/s", "value": value, "unit": "ray-cell updates/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": {"workload": "depth_640x480_room", "resolution_m": room.resolution,
                   "max_range_m": room.max_range, "camera": "640x480, fx=fy=525",
                   "room": "8x6x3 m, 50 boxes", "frames": args.steps,
                   "l2": "flushed before every timed frame and lookup batch",
                   "parallelism": f"replicas x{ws}"},
        "lookup": {"lookups_per_s": nq / (lk_ms / 1e3), "n": nq, "ms": lk_ms,
                   "call_ms": float(np.median(call)),
                   "call_lookups_per_s": nq / (float(np.median(call)) / 1e3),
                   "roofline": {"bound": "hbm", "achieved": lk_ach, "peak": pk, "unit": "GB/s",
                                "frac": lk_ach / pk, "peak_kind": pkind,
                                "algorithmic_bytes_per_lookup": 17,
                                "random_access_achieved_gbs": 109.0 * nq / (lk_ms / 1e3) / 1e9}},
        "roofline": None, "ray_kernel_ms": float(np.mean(ray_ms)),
        "cpu_baseline": cpu,
        "e2e": {"value": V_e2e / t_e2e, "unit": "ray-cell updates/s",
                "h2d_bytes_per_step": int(np.mean([len(f[0]) for f in frames])) * 12,
                "d2h_bytes_per_step": 128},
        "gpu_launches": None, "clocks": clocks,
    }
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------------------
# multi-map workload: 64 maps per tick, batched vs plain per-scan path
# ----------------------------------------------------------------------------
MM_RANGE = 10.0


def multimap_inputs(n_maps: int, only=None, max_points=None):
    """Base scan per map (log-uniform 10k..500k points, room or LiDAR
    generator, resolution cycling 0.02/0.05/0.1 m). Tick t moves a LiDAR
    sensor 0.5 m along +x (five poses, cycling) and re-observes a room from
    its centre. `only`: indices of the maps to generate (None: all); the
    others get None. `max_points` caps the points per map (small test runs)."""
    from bonxai_gb300 import synth
    specs = synth.multi_map_specs(n_maps)
    if max_points:
        for sp in specs:
            sp.n_points = min(sp.n_points, int(max_points))
    base = []
    for sp in specs:
        if only is not None and sp.index not in only:
            base.append(None)
            continue
        if sp.kind == "lidar":
            n_az = max(16, -(-sp.n_points // 64))
            scene = synth.LidarScene(seed=sp.seed, n_az=n_az, max_range=MM_RANGE)
            pts, o = scene.scan(0, n_points=sp.n_points)
        else:
            pts = synth.room_cloud(sp.n_points, seed=sp.seed)
            o = ((synth.ROOM_LO + synth.ROOM_HI) / 2).astype(np.float32)
        base.append((pts, o))
    return specs, base


def multimap_scan(sp, base_scan, t):
    pts, o = base_scan
    if sp.kind == "lidar":
        d = np.array([0.5 * (t % 5), 0.0, 0.0], np.float32)
        return pts + d, o + d
    return pts, o


def multimap_tick(specs, base, t):
    return [multimap_scan(sp, b, t) for sp, b in zip(specs, base)]


def _farm_worker(conn, n_maps, mine, max_points):
    """One CPU process of the map-parallel CPU path: owns the maps `mine`
    (oracle maps, single-threaded each, persistent across ticks) and inserts
    their scans of the ticks it is sent."""
    from oracle import oracle as O
    port = O.port()
    specs, base = multimap_inputs(n_maps, only=set(mine), max_points=max_points)
    maps = {i: port.pmap(specs[i].resolution) for i in mine}
    ticks = {i: 0 for i in mine}
    conn.send(("ready", 0, 0.0))
    while True:
        msg = conn.recv()
        if msg is None:
            break
        V, dt = 0, 0.0
        for i in msg:
            if i not in maps:
                continue
            pts, o = multimap_scan(specs[i], base[i], ticks[i])
            t0 = time.perf_counter()
            V += maps[i].insert(pts, o, MM_RANGE)
            dt += time.perf_counter() - t0
            ticks[i] += 1
        conn.send(("done", V, dt))


class MapFarm:
    """The multi-map workload on the host cores: `cores` spawned processes,
    whole maps assigned by longest-processing-time on their point counts
    (bonxai_gb300.sharding), each map's scans inserted in order by the CPU
    oracle (the reference's scan is single-threaded per map; maps are
    independent, so they run in parallel)."""

    def __init__(self, n_maps: int, cores: int, max_points=None):
        import multiprocessing as mp
        from bonxai_gb300 import sharding, synth
        specs = synth.multi_map_specs(n_maps)
        ranks = sharding.assign_maps([sp.n_points for sp in specs], cores)
        ctx = mp.get_context("spawn")  # the GPU may be in use in this process
        self.procs, self.conns = [], []
        self.n_maps = n_maps
        for r in range(cores):
            mine = [i for i, k in enumerate(ranks) if k == r]
            if not mine:
                continue
            a, b = ctx.Pipe()
            p = ctx.Process(target=_farm_worker, args=(b, n_maps, mine, max_points), daemon=True)
            p.start()
            self.procs.append(p)
            self.conns.append(a)
        for c in self.conns:
            c.recv()
        self.cores = len(self.procs)

    def tick(self, maps=None):
        """Inserts the next scan of each map in `maps` (default all); returns
        (ray-cell updates, wall seconds, summed single-core seconds)."""
        ids = list(range(self.n_maps)) if maps is None else list(maps)
        t0 = time.perf_counter()
        for c in self.conns:
            c.send(ids)
        res = [c.recv() for c in self.conns]
        wall = time.perf_counter() - t0
        return sum(r[1] for r in res), wall, sum(r[2] for r in res)

    def close(self):
        for c in self.conns:
            try:
                c.send(None)
            except (BrokenPipeError, OSError):
                pass
        for p in self.procs:
            p.join(timeout=10)


def mm_cpu_baseline(n_maps, cores, seconds, max_points=None):
    """cpu_baseline of the multi-map workload: whole ticks of all maps on the
    host cores until about `seconds` of wall time (at least one tick)."""
    farm = MapFarm(n_maps, cores, max_points)
    try:
        V, wall, busy, ticks = 0, 0.0, 0.0, 0
        while wall < seconds or ticks == 0:
            v, w, b = farm.tick()
            V, wall, busy, ticks = V + v, wall + w, busy + b, ticks + 1
    finally:
        farm.close()
    return {"value": V / wall, "unit": "ray-cell updates/s", "cores": farm.cores,
            "kind": "port",
            "sample": f"{ticks} tick(s) of all {n_maps} maps, maps spread over {farm.cores} "
                      f"processes, {wall:.1f} s wall; single-core rate "
                      f"{V / busy:.4g} ray-cell updates/s ({busy:.1f} s of one-core work). "
                      "The port's timing is within 10 % of the reference compiled unmodified "
                      "(profiles/cpu_port_vs_ref.md)"}


def run_reference_multimap(args):
    """The multi-map workload on the host's CPU cores through the CPU path
    (the reference's algorithm as the oracle restates it): rank 0 only. Each
    step is one tick of a rotating subset of the maps, sized so that the whole
    run stays within a few minutes; every map still gets its scans in order."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    cores = os.cpu_count() or 1
    farm = MapFarm(args.maps, cores, args.max_points)
    try:
        _, w0, _ = farm.tick()  # one full tick: also sizes the per-step sample
        n_steps = args.steps + args.warmup
        per_step = max(1, min(args.maps, int(args.maps * 150.0 / max(w0 * n_steps, 1e-9))))
        order = list(range(args.maps))
        cursor = 0

        def subset():
            nonlocal cursor
            ids = [order[(cursor + k) % args.maps] for k in range(per_step)]
            cursor = (cursor + per_step) % args.maps
            return ids

        for _ in range(args.warmup):
            farm.tick(subset())
        V, wall, busy = 0, 0.0, 0.0
        for _ in range(args.steps):
            v, w, b = farm.tick(subset())
            V, wall, busy = V + v, wall + w, busy + b
    finally:
        farm.close()
    value = V / wall
    line = {
        "impl": "reference", "metric": "ray-cell updates/s (64-map batched tick)",
        "value": value, "unit": "ray-cell updates/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": multimap_config(args, ws),
        "cpu_baseline": {"value": value, "unit": "ray-cell updates/s", "cores": farm.cores,
                         "kind": "port",
                         "sample": f"each step one tick of {per_step} of the {args.maps} maps "
                                   f"(rotating), maps spread over {farm.cores} processes; "
                                   f"single-core rate {V / busy:.4g} ray-cell updates/s"},
        "e2e": {"value": value, "unit": "ray-cell updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def multimap_config(args, ws):
    return {"workload": "multimap_64_uneven", "maps": args.maps,
            "points_per_map": "log-uniform 10k..500k (room / LiDAR generators)",
            "resolutions_m": [0.02, 0.05, 0.1], "max_range_m": MM_RANGE,
            "ticks": args.steps, "parallelism": f"maps sharded over {ws} rank(s)",
            "l2": "flushed before every timed tick (256 MiB write)"}


def mm_traffic():
    """Per-tick DRAM and L2 figures of k_tick from the committed ncu summary."""
    p = ROOT / "profiles" / "k_tick_multimap_traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            return None
    return None


def run_multimap(args):
    """The 64-map uneven workload: every tick, one insertPointCloud scan per
    map, through the batched form (one graph-replayed persistent launch for
    all maps) and through the plain per-scan path (one synchronous
    insertPointCloud call per map) on identical inputs; the maps of the two
    paths are compared bit-exactly after the run. Under torchrun each rank
    takes whole maps (longest-processing-time assignment by points,
    bonxai_gb300.sharding); no collective touches the data, and rank 0 reports
    units summed over ranks over the slowest rank's time."""
    import torch
    import bonxai_gb300 as bx
    from bonxai_gb300 import sharding

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.device("cuda", torch.cuda.current_device())
    t0 = time.perf_counter()
    specs, base = multimap_inputs(args.maps, max_points=args.max_points)
    mine = sharding.my_maps([len(b[0]) for b in base], ws, rank)
    specs = [specs[i] for i in mine]
    base = [base[i] for i in mine]
    n_maps = len(specs)
    log(f"rank {rank}: generated {args.maps} base scans in {time.perf_counter() - t0:.1f} s, "
        f"{sum(len(b[0]) for b in base)} of its points per tick")
    ticks = args.warmup + args.steps
    big = bx.Config(flags=args.flags, initial_leaves=1 << 16, initial_inners=1 << 12,
                    hash_buckets=1 << 14)
    timed_cfg = bx.Config(flags=bx.FLAG_TIMING | args.flags, initial_leaves=1 << 16,
                          initial_inners=1 << 12, hash_buckets=1 << 14)
    bmaps = [bx.ProbabilisticMap(sp.resolution, big) for sp in specs]
    pmaps = [bx.ProbabilisticMap(sp.resolution, timed_cfg) for sp in specs]
    batch = bx.Batch(bx.Config(rays_per_warp=args.rays_per_warp, ray_unroll=args.ray_unroll))
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=dev)

    t_b, t_p, dev_b, dev_p, V_b, V_p = 0.0, 0.0, 0.0, 0.0, 0, 0
    lat_b, lat_p, dev_ticks = [], [], []
    phases = {}
    alg = {"points": 0, "rays": 0, "ray_cells_updated": 0, "new_leaves": 0}
    leaves_prev = [0] * n_maps
    launches0 = batch.stats()["launches"]
    clk = ClockSampler(dev.index)
    clk.__enter__()
    for t in range(ticks):
        scans = multimap_tick(specs, base, t)
        pts = torch.from_numpy(np.concatenate([s[0] for s in scans])).to(dev)
        off = np.concatenate([[0], np.cumsum([len(s[0]) for s in scans])]).astype(np.uint64)
        org = np.stack([s[1] for s in scans])
        dev_scans = [pts[int(off[i]):int(off[i + 1])] for i in range(n_maps)]
        timed = t >= args.warmup
        # batched tick
        flush.fill_(t)
        torch.cuda.synchronize()
        a = time.perf_counter()
        rc = batch.insert(bmaps, pts, off, org, MM_RANGE)
        dt = time.perf_counter() - a
        if timed:
            t_b += dt
            bst = batch.stats()
            dev_b += bst["device_ms"] / 1e3
            dev_ticks.append(bst["device_ms"])
            for k, v in bst["phase_ms"].items():
                phases[k] = phases.get(k, 0.0) + v / args.steps
            V_b += int(rc.sum())
            lat_b.append(dt * 1e3)
            for i, m in enumerate(bmaps):
                st = m.last_stats()
                alg["points"] += st["points"]
                alg["rays"] += st["cast_rays"]
                alg["ray_cells_updated"] += st["ray_cells_updated"]
                alg["new_leaves"] += max(st["leaves"] - leaves_prev[i], 0)
        for i, m in enumerate(bmaps):
            leaves_prev[i] = m.last_stats()["leaves"]
        # plain per-scan path, same inputs
        flush.fill_(t)
        torch.cuda.synchronize()
        a = time.perf_counter()
        vp, dp = 0, 0.0
        for i in range(n_maps):
            vp += pmaps[i].insert_point_cloud(dev_scans[i], org[i], MM_RANGE)
            dp += sum(pmaps[i].kernel_times())
        dt = time.perf_counter() - a
        if timed:
            t_p += dt
            dev_p += dp / 1e3
            V_p += vp
            lat_p.append(dt * 1e3)
        if rc.sum() != vp:
            raise SystemExit(f"tick {t}: batched {int(rc.sum())} != plain {vp} ray cells")
    clk.__exit__(None, None, None)
    launches = batch.stats()["launches"] - launches0
    # bit-exact check of every map after the run
    same = all(np.array_equal(bmaps[i].dump()[1], pmaps[i].dump()[1]) for i in range(n_maps))
    if ws > 1:
        import torch.distributed as dist
        V_b, dev_b = sharding.aggregate(V_b, dev_b)
        V_p, dev_p = sharding.aggregate(V_p, dev_p)
        _, t_b = sharding.aggregate(0, t_b)
        _, t_p = sharding.aggregate(0, t_p)
        ok = torch.tensor([1.0 if same else 0.0], device=dev)
        dist.all_reduce(ok, op=dist.ReduceOp.MIN)
        same = bool(ok.item())
    value = V_b / dev_b           # batched, device-timed (inputs resident in HBM)
    plain_dev = V_p / dev_p       # plain per-scan, summed device time of its scans
    batched_wall = V_b / t_b      # both paths timed on the host around the calls
    plain_wall = V_p / t_p
    # e2e: the same ticks from pinned host memory through the C ABI (the batch
    # copies the points to the device inside the call)
    e2e = None
    if not args.no_e2e:
        emaps = [bx.ProbabilisticMap(sp.resolution, big) for sp in specs]
        t_e, V_e, h2d = 0.0, 0, 0
        for t in range(ticks):
            scans = multimap_tick(specs, base, t)
            hp = torch.from_numpy(np.concatenate([s[0] for s in scans])).pin_memory().numpy()
            off = np.concatenate([[0], np.cumsum([len(s[0]) for s in scans])]).astype(np.uint64)
            org = np.stack([s[1] for s in scans])
            torch.cuda.synchronize()
            a = time.perf_counter()
            rc = batch.insert(emaps, hp, off, org, MM_RANGE)
            dt = time.perf_counter() - a
            if t >= args.warmup:
                t_e += dt
                V_e += int(rc.sum())
                h2d += int(off[-1]) * 12
        if ws > 1:
            V_e, t_e = sharding.aggregate(V_e, t_e)
        e2e = {"value": V_e / t_e, "unit": "ray-cell updates/s",
               "h2d_bytes_per_step": h2d // args.steps,
               "d2h_bytes_per_step": n_maps * (8 + 4 * 32),
               "ms_per_step": 1e3 * t_e / args.steps}
        for m in emaps:
            m.close()
    if rank != 0:
        dist.destroy_process_group()
        return 0
    # roofline of k_tick: algorithmic bytes of the timed ticks over their
    # event-timed device duration
    pk, pkind = peaks()
    tick_bytes = (12 * alg["points"] + RAY_LIST_BYTES * alg["rays"] +
                  CELL_RMW_BYTES * (alg["rays"] + alg["ray_cells_updated"]) +
                  LEAF_MASK_BYTES * alg["new_leaves"]) / args.steps
    tick_ms = float(np.mean(dev_ticks))
    ach = tick_bytes / (tick_ms / 1e3) / 1e9
    tr = mm_traffic() or {}
    roofline = {"kernel": "k_tick (one launch per tick)", "bound": "hbm", "achieved": ach,
                "peak": pk, "unit": "GB/s", "frac": ach / pk, "peak_kind": pkind,
                "traffic": tr.get("dram_bytes_per_tick"),
                "algorithmic_bytes_per_launch": tick_bytes, "launch_ms": tick_ms,
                "l2": tr.get("l2")}
    cpu = None
    if not args.no_cpu and ws == 1:
        cpu = mm_cpu_baseline(args.maps, os.cpu_count() or 1, args.cpu_seconds,
                              args.max_points)
    lat_b.sort()
    lat_p.sort()

    def pct(v, q):
        return v[min(len(v) - 1, int(q * len(v)))]

    line = {
        "metric": "ray-cell updates/s (64-map batched tick)", "value": value,
        "unit": "ray-cell updates/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * dev_b / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": dict(multimap_config(args, ws), points_per_tick_rank0=int(off[-1]),
                       rays_per_warp=args.rays_per_warp, graph=batch.stats()["graph"]),
        "plain_per_scan_value": plain_dev, "batched_over_plain": value / plain_dev,
        "wall": {"batched": batched_wall, "plain_per_scan": plain_wall,
                 "batched_over_plain": batched_wall / plain_wall},
        "tick_ms_p50": pct(lat_b, 0.5), "tick_ms_p99": pct(lat_b, 0.99),
        "plain_tick_ms_p50": pct(lat_p, 0.5), "plain_tick_ms_p99": pct(lat_p, 0.99),
        "maps_bit_identical_batched_vs_plain": same,
        "tick_phase_ms": phases, "roofline": roofline,
        "e2e": e2e, "cpu_baseline": cpu, "gpu_launches": launches, "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()
    return 0


# ----------------------------------------------------------------------------
# serving workload: 32 clients, Poisson arrivals, mixed requests
# ----------------------------------------------------------------------------
def run_serve(args):
    import threading
    import bonxai_gb300 as bx
    from bonxai_gb300 import synth

    n_clients = args.clients
    rate = args.rate
    duration = args.duration
    rng0 = np.random.default_rng(5000)
    # request payloads: slices of a few large base scans, shifted per client
    t0 = time.perf_counter()
    lidar = synth.LidarScene(seed=5001, n_az=4800, max_range=MM_RANGE)  # 307,200 rays
    lid_pts, lid_o = lidar.scan(0, n_points=300_000)
    room_pts = synth.room_cloud(300_000, seed=5002)
    room_o = ((synth.ROOM_LO + synth.ROOM_HI) / 2).astype(np.float32)
    coords_pool = rng0.integers([-100, -100, -20], [100, 100, 60], (1_000_000, 3)).astype(np.int32)
    log(f"serving inputs ready in {time.perf_counter() - t0:.1f} s")
    res = [0.1 if c % 2 == 0 else 0.05 for c in range(n_clients)]
    cfg = bx.ServerConfig(pool_budget_bytes=args.budget_gb << 30, rays_per_warp=args.rays_per_warp,
                          ray_unroll=args.ray_unroll, initial_leaves=1 << 14)
    srv = bx.Server(res, cfg)

    def client_stream(cid, rng, t_end, counts):
        shift = np.array([0.7 * cid, -0.3 * cid, 0.0], np.float32)
        t = time.perf_counter()
        k = 0
        while True:
            t += rng.exponential(n_clients / rate)
            if t > t_end:
                return
            d = t - time.perf_counter()
            if d > 0:
                time.sleep(d)
            u = rng.random()
            if u < 0.70:
                n = int(np.exp(rng.uniform(np.log(10_000), np.log(300_000))))
                if cid % 2 == 0:
                    pts, o = lid_pts[:n] + shift, lid_o + shift
                else:
                    pts, o = room_pts[:n], room_o
                srv.insert(cid, pts, o, MM_RANGE, discard=True)
                counts[0] += 1
            elif u < 0.95:
                n = int(np.exp(rng.uniform(np.log(1_000), np.log(1_000_000))))
                srv.query(cid, coords_pool[:n], mode=0, discard=True)
                counts[1] += 1
            else:
                srv.get_occupied(cid, discard=True)
                counts[2] += 1
            k += 1

    # warm-up: one insert per client
    for cid in range(n_clients):
        srv.insert(cid, lid_pts[:20000] if cid % 2 == 0 else room_pts[:20000],
                   lid_o if cid % 2 == 0 else room_o, MM_RANGE, discard=True)
    srv.drain()
    base = srv.stats()
    t_start = time.perf_counter()
    t_end = t_start + duration
    counts = [[0, 0, 0] for _ in range(n_clients)]
    threads = [threading.Thread(target=client_stream,
                                args=(c, np.random.default_rng(5100 + c), t_end, counts[c]))
               for c in range(n_clients)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    srv.drain(600)
    wall = time.perf_counter() - t_start
    st = srv.stats()
    done = st["completed"] - base["completed"]
    line = {
        "metric": "served requests/s (32-client mixed stream)", "value": done / wall,
        "unit": "requests/s", "n_gpus": 1, "steps": int(done), "warmup": n_clients,
        "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "int32", "data": "synthetic",
        "config": {"workload": "serve_32", "clients": n_clients, "offered_rate_rps": rate,
                   "duration_s": duration, "mix": "70% insert 10k-300k pts, 25% isOccupied "
                   "1k-1M coords, 5% getOccupiedVoxels", "budget_gb": args.budget_gb,
                   "resolutions_m": [0.1, 0.05], "max_range_m": MM_RANGE},
        "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
        "insert_p50_ms": st["insert_p50_ms"], "insert_p99_ms": st["insert_p99_ms"],
        "lookup_p50_ms": st["lookup_p50_ms"], "lookup_p99_ms": st["lookup_p99_ms"],
        "occupied_p50_ms": st["occupied_p50_ms"], "occupied_p99_ms": st["occupied_p99_ms"],
        "ray_cell_updates_per_s": (st["ray_cells"] - base["ray_cells"]) / wall,
        "lookups_per_s": (st["lookup_coords"] - base["lookup_coords"]) / wall,
        "ticks": st["ticks"] - base["ticks"], "rejected": st["rejected"],
        "gpu_busy_frac": (st["busy_s"] - base["busy_s"]) / wall,
        "submitted": [sum(c[i] for c in counts) for i in range(3)],
        "pool_bytes": st["pool_bytes"],
    }
    srv.close()
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="multimap",
                    choices=["lidar", "multimap", "serve", "room", "depth"])
    ap.add_argument("--maps", type=int, default=64)
    ap.add_argument("--max-points", type=int, default=0,
                    help="cap on points per map of the multimap workload (small test runs)")
    ap.add_argument("--clients", type=int, default=32)
    ap.add_argument("--rate", type=float, default=2000.0, help="offered requests/s (serve)")
    ap.add_argument("--duration", type=float, default=60.0, help="seconds of load (serve)")
    ap.add_argument("--budget-gb", type=int, default=40)
    ap.add_argument("--rays-per-warp", type=int, default=1)
    ap.add_argument("--ray-unroll", type=int, default=1)
    ap.add_argument("--block-size", type=int, default=0)
    ap.add_argument("--flags", type=int, default=0, help="extra BXG_FLAG_* bits for the maps")
    ap.add_argument("--cpu-seconds", type=float, default=10.0,
                    help="CPU baseline sample length (seconds of single-thread work)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true",
                    help="skip the host-buffer pass (short runs for profiling)")
    args = ap.parse_args()
    if args.warmup < 3:
        log("warmup raised to 3")
        args.warmup = 3
    if args.impl == "reference":
        if args.workload == "multimap":
            return run_reference_multimap(args)
        return run_reference(args)
    if args.workload == "room":
        return run_room(args)
    if args.workload == "depth":
        return run_depth(args)
    if args.workload == "multimap":
        return run_multimap(args)
    if args.workload == "serve":
        return run_serve(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
