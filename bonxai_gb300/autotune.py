"""Autotuner for the ray-phase launch shape and the root-hash load factor.

Tunable knobs (none changes a result, only speed):
  ray phase       two phases (mark the ray cells, then apply per leaf) or one
                  pass (BXG_FLAG_RAYS_SINGLE_PASS); the knobs below shape the
                  one-pass walk
  rays_per_warp   1, 2, 4   lanes per ray = 32 / rays_per_warp
  ray_unroll      1, 2      cells per lane per step
  block_size      0, 256, 1024  threads per block of the per-map ray kernel
                  (0: 1024 for large scans, 256 for small ones)
  hash_load_factor 0.25, 0.5, 0.75  root-hash growth threshold

For each candidate the tuner replays a short sample of the workload on fresh
maps and times it with the library's own CUDA events (per-map path: the ray
kernel; batched path: the whole tick). It writes the winners to a JSON file
that bench.py and callers pass back through bxg_config:

    python -m bonxai_gb300.autotune --out autotune.json
"""
from __future__ import annotations

import argparse
import itertools
import json
import sys
import time
from pathlib import Path

import numpy as np

DEFAULT_OUT = Path(__file__).resolve().parent / "_build" / "autotune.json"


def _lidar_sample(n_scans=6, n_points=131072):
    from bonxai_gb300 import synth
    scene = synth.LidarScene()
    return scene, [scene.scan(k, n_points=n_points) for k in range(n_scans)]


def tune_per_map(scans, resolution, max_range, repeats=2):
    """Best (ray-phase form, rays_per_warp, ray_unroll, block_size,
    hash_load_factor) for the per-map scan, by the summed scan time over the
    sample."""
    import torch
    import bonxai_gb300 as bx
    dev = [(torch.from_numpy(p).cuda(), o) for p, o in scans]
    results = []
    cands = [(0, 1, 1, 0, lf) for lf in (0.25, 0.5, 0.75)]  # two phases
    cands += [(bx.FLAG_RAYS_SINGLE_PASS,) + c for c in
              itertools.product((1, 2, 4), (1, 2), (0, 256, 1024), (0.25, 0.5, 0.75))]
    for form, rpw, unroll, bs, lf in cands:
        best = None
        for _ in range(repeats):
            cfg = bx.Config(rays_per_warp=rpw, ray_unroll=unroll, block_size=bs,
                            hash_load_factor=lf, flags=bx.FLAG_TIMING | form,
                            initial_leaves=1 << 18, hash_buckets=1 << 12)
            m = bx.ProbabilisticMap(resolution, cfg)
            t_ray = t_all = 0.0
            for p, o in dev:
                m.insert_point_cloud(p, o, max_range)
                kt = m.kernel_times()
                t_ray += kt[3]
                t_all += sum(kt)
            m.close()
            best = t_all if best is None else min(best, t_all)
        results.append({"flags": form, "rays_per_warp": rpw, "ray_unroll": unroll,
                        "block_size": bs, "hash_load_factor": lf, "scan_ms": best / len(dev)})
    results.sort(key=lambda r: r["scan_ms"])
    return results


def tune_batched(n_maps=16, ticks=3):
    """Best (ray-phase form, rays_per_warp, ray_unroll) for the batched tick on a
    multi-map sample, by device time per tick."""
    import torch
    import bonxai_gb300 as bx
    from bonxai_gb300 import synth
    specs = synth.multi_map_specs(n_maps)
    scans = []
    for sp in specs:
        n = min(sp.n_points, 100_000)
        if sp.kind == "lidar":
            pts, o = synth.LidarScene(seed=sp.seed, max_range=10.0).scan(0, n_points=n)
        else:
            pts = synth.room_cloud(n, seed=sp.seed)
            o = ((synth.ROOM_LO + synth.ROOM_HI) / 2).astype(np.float32)
        scans.append((pts, o))
    pts = torch.from_numpy(np.concatenate([s[0] for s in scans])).cuda()
    off = np.concatenate([[0], np.cumsum([len(s[0]) for s in scans])]).astype(np.uint64)
    org = np.stack([s[1] for s in scans])
    results = []
    cands = [(0, 1, 1)] + [(bx.FLAG_RAYS_SINGLE_PASS, rpw, unroll)
                           for rpw, unroll in itertools.product((1, 2, 4), (1, 2))]
    for form, rpw, unroll in cands:
        b = bx.Batch(bx.Config(rays_per_warp=rpw, ray_unroll=unroll))
        maps = [bx.ProbabilisticMap(sp.resolution, bx.Config(flags=form)) for sp in specs]
        times = []
        for _ in range(ticks):
            b.insert(maps, pts, off, org, 10.0)
            times.append(b.stats()["device_ms"])
        results.append({"flags": form, "rays_per_warp": rpw, "ray_unroll": unroll,
                        "tick_ms": float(np.median(times[1:] if len(times) > 1 else times))})
        for m in maps:
            m.close()
        b.close()
    results.sort(key=lambda r: r["tick_ms"])
    return results


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(DEFAULT_OUT))
    ap.add_argument("--quick", action="store_true")
    args = ap.parse_args(argv)
    import torch
    torch.cuda.set_device(0)
    t0 = time.time()
    scene, scans = _lidar_sample(3 if args.quick else 6)
    per_map = tune_per_map(scans, scene.resolution, scene.max_range, repeats=1 if args.quick else 2)
    batched = tune_batched(8 if args.quick else 16)
    out = {"per_map": per_map[0], "batched": batched[0], "per_map_all": per_map,
           "batched_all": batched, "device": torch.cuda.get_device_name(0),
           "seconds": time.time() - t0}
    Path(args.out).parent.mkdir(parents=True, exist_ok=True)
    Path(args.out).write_text(json.dumps(out, indent=1))
    print(json.dumps({"per_map": per_map[0], "batched": batched[0]}))
    return 0


def load(path: str | Path = DEFAULT_OUT) -> dict | None:
    p = Path(path)
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            return None
    return None


if __name__ == "__main__":
    sys.exit(main())
