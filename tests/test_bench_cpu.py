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


def test_multimap_farm_matches_single_process(port):
    """The map-parallel CPU path (spawned processes owning whole maps) gives the
    same ray-cell counts as inserting the same scans in one process, tick
    after tick."""
    import bench
    specs, base = bench.multimap_inputs(3, max_points=3000)
    maps = [port.pmap(sp.resolution) for sp in specs]
    farm = bench.MapFarm(3, 2, max_points=3000)
    try:
        assert farm.cores == 2
        for t in range(2):
            want = sum(m.insert(*bench.multimap_scan(sp, b, t), bench.MM_RANGE)
                       for m, sp, b in zip(maps, specs, base))
            V, wall, busy = farm.tick()
            assert V == want and wall > 0 and busy > 0
    finally:
        farm.close()


def test_multimap_cpu_baseline_fields():
    import bench
    cpu = bench.mm_cpu_baseline(3, 2, 0.0, max_points=2000)
    assert cpu["kind"] == "port" and cpu["cores"] == 2 and cpu["value"] > 0
    assert "3 maps" in cpu["sample"] and "single-core" in cpu["sample"]


def test_reference_arm_multimap_line():
    import json
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                        "--maps", "3", "--max-points", "2000", "--steps", "2", "--warmup", "3"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["config"]["workload"] == "multimap_64_uneven"
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["cores"] >= 1
