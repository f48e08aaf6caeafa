"""Times the oracle restatement (oracle/bonxai_oracle.cpp) against the
reference compiled unmodified (oracle/_ref, built by oracle/build_ref.sh where
the reference sources are mounted) on the same inputs, one thread each,
interleaved, best of `--reps` runs. Test infrastructure: it measures the CPU
baseline's fidelity and is not part of the library.

    python oracle/time_port_vs_ref.py [--reps 4]
"""
from __future__ import annotations

import argparse
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reps", type=int, default=4)
    args = ap.parse_args()
    import bench
    from bonxai_gb300 import synth
    from oracle import oracle as O
    port, ref = O.port(), O.ref()
    if ref is None:
        print("the reference build is not available here (oracle/_ref)")
        return 1
    scene = synth.LidarScene()
    scans = [scene.scan(k) for k in range(20)]
    specs, base = bench.multimap_inputs(64)
    mm = bench.multimap_tick(specs, base, 0)
    sel = list(range(0, 64, 4))

    def lidar(L):
        m = L.pmap(scene.resolution)
        t0 = time.perf_counter()
        V = sum(m.insert(p, o, scene.max_range) for p, o in scans)
        return time.perf_counter() - t0, V

    def multimap(L):
        t, V = 0.0, 0
        for i in sel:
            m = L.pmap(specs[i].resolution)
            t0 = time.perf_counter()
            V += m.insert(*mm[i], bench.MM_RANGE)
            t += time.perf_counter() - t0
        return t, V

    res = {}
    for _ in range(args.reps):
        for name, L in (("port", port), ("reference", ref)):
            for wl, f in (("lidar_20_scans", lidar), ("multimap_tick0_16_maps", multimap)):
                res.setdefault((wl, name), []).append(f(L))
    for wl in ("lidar_20_scans", "multimap_tick0_16_maps"):
        tp = min(t for t, _ in res[(wl, "port")])
        tr = min(t for t, _ in res[(wl, "reference")])
        vp, vr = res[(wl, "port")][0][1], res[(wl, "reference")][0][1]
        print(f"{wl}: port {tp:.3f} s, reference {tr:.3f} s, port/reference {tp / tr:.3f}, "
              f"ray-cell updates {vp} / {vr}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
