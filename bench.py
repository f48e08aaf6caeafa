#!/usr/bin/env python3
"""Benchmark of the ProbabilisticMap scan path on one GB300.

Workload (default ``lidar``): ProbabilisticMap::insertPointCloud of a 64-beam x
2048-column LiDAR (131,072 float32 points per scan, elevation -25..+15 deg) in a
seeded 40x40x8 m scene of 200 boxes, 20 scans along a straight trajectory
(0.5 m steps), resolution 0.1 m, max range 30 m, default Options. One step is
one scan; the map is cleared every 20 scans (outside the timed region) so the
timed steps replay the 20-scan sequence.

Metric: ray-cell updates/s, V / t with V = points + sum of cast ray lengths
(the count the reference's own loop performs, identical on CPU and GPU).

* ``value``: device time of the whole scan (first to last kernel, CUDA events
  on the library's stream) with the points already in HBM; L2 is flushed
  (256 MiB write) before every timed scan.
* ``e2e``: the same scans through the C ABI with pinned host buffers: the
  host->device copy of the points, all kernels, and the device->host read of
  the scan's counters, timed on the host around the call.
* ``roofline``: the ray kernel (dominant), algorithmic bytes per launch over its
  CUDA-event duration, against the measured HBM copy bandwidth.
* ``cpu_baseline``: the CPU oracle (a restatement of the reference, one thread)
  on a bounded sample of the same sequence.

``--impl reference`` times that CPU implementation alone on this workload.
Under torchrun with N > 1 each rank runs an independent replica of the map
(the scan of one map does not shard); ``value`` sums the ranks' ray-cell
updates over the slowest rank's time.
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
                 "--format=csv,noheader,nounits", "-lms", "100"],
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
    """Per-launch DRAM bytes of the ray kernel from the committed ncu summary."""
    p = ROOT / "profiles" / "k_rays_lidar_traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            return None
    return None


def cpu_sample(scene, scans, n_scans=3):
    """CPU oracle (single thread) on the first n_scans of the sequence."""
    from oracle import oracle as O
    port = O.port()
    m = port.pmap(scene.resolution)
    V = 0
    t0 = time.perf_counter()
    for k in range(n_scans):
        pts, o = scans[k]
        V += m.insert(pts, o, scene.max_range)
    dt = time.perf_counter() - t0
    return V, dt


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

    cfg = bx.Config(flags=bx.FLAG_TIMING, rays_per_warp=args.rays_per_warp,
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
    V_total, dev_ms, ray_ms, ray_bytes, ray_bytes_ra = 0, 0.0, [], 0.0, 0.0
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
            ray_bytes += (RAY_LIST_BYTES * st["cast_rays"] + CELL_RMW_BYTES * st["ray_cells_updated"]
                          + LEAF_MASK_BYTES * max(new_leaves, 0))
            ray_bytes_ra += 16 * st["cast_rays"] + 64 * st["ray_cells_updated"]
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

    # ---------------- e2e: host buffers through the C ABI
    if args.no_e2e:
        h_scans = h_scans[:0]
    m.clear()
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

    peak, peak_kind = peaks()
    avg_ray_ms = sum(ray_ms) / len(ray_ms)
    bytes_per_launch = ray_bytes / len(ray_ms)
    achieved = bytes_per_launch / (avg_ray_ms / 1e3) / 1e9
    tr = ncu_traffic()
    roofline = {
        "kernel": "k_rays<32> (ray phase)", "bound": "hbm", "achieved": achieved,
        "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
        "traffic": tr.get("dram_bytes_per_launch") if tr else None,
        "algorithmic_bytes_per_launch": bytes_per_launch,
        "random_access_bytes_per_launch": ray_bytes_ra / len(ray_ms),
        "ray_kernel_ms": avg_ray_ms,
        "ray_kernel_share_of_scan": sum(ray_ms) / dev_ms,
    }
    cpu = None
    if not args.no_cpu:
        Vc, tc = cpu_sample(scene, scans, args.cpu_scans)
        cpu = {"value": Vc / tc, "unit": "ray-cell updates/s", "cores": 1, "kind": "port",
               "sample": f"scans 0-{args.cpu_scans - 1} of the sequence on a fresh map, "
                         f"one thread, {tc:.1f} s"}
    line = {
        "metric": "ray-cell updates/s", "value": value, "unit": "ray-cell updates/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dev_ms_all / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "config": dict(workload_config(scene), parallelism=f"replicas x{ws}",
                       rays_per_warp=args.rays_per_warp),
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--rays-per-warp", type=int, default=1)
    ap.add_argument("--cpu-scans", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-e2e", action="store_true",
                    help="skip the host-buffer pass (short runs for profiling)")
    args = ap.parse_args()
    if args.warmup < 3:
        log("warmup raised to 3")
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
