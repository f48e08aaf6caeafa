"""The CPU legs of bench.py (no GPU): the single-thread baseline sample and
the map-parallel multi-map baseline run the oracle and report consistent
fields; --help parses."""
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def test_help_parses():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--help"], capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0 and "--workload" in r.stdout


def test_cpu_sample_counts_ray_cells(port):
    import bench
    from bonxai_gb300 import synth
    scene = synth.LidarScene()
    scans = [scene.scan(k, n_points=2048) for k in range(3)]
    V, dt, n = bench.cpu_sample(scene, scans, seconds=0.0)
    assert n == 3 and dt > 0
    m = port.pmap(scene.resolution)
    assert V == sum(m.insert(p, o, scene.max_range) for p, o in scans)


def test_multimap_cpu_baseline_spreads_maps(port):
    import bench
    from bonxai_gb300 import synth
    specs = synth.multi_map_specs(3)
    scans = []
    for sp in specs:
        pts = synth.room_cloud(3000, seed=sp.seed)
        scans.append((pts, ((synth.ROOM_LO + synth.ROOM_HI) / 2).astype(np.float32)))
    cpu = bench.mm_cpu_baseline(specs, scans, 2)
    assert cpu["kind"] == "port" and cpu["cores"] == 2 and cpu["value"] > 0
    assert "3 maps" in cpu["sample"] and "one core" in cpu["sample"]
