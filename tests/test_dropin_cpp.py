"""Caller code written against the reference's C++ API (tests/cpp/dropin_main.cpp)
compiles unchanged against include/bonxai/*.hpp + include/bonxai_map/*.hpp,
runs on the GPU library, and matches the CPU oracle."""
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from bonxai_gb300 import synth

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def dropin_exe(tmp_path_factory, cuda_lib):
    out = tmp_path_factory.mktemp("dropin") / "dropin_main"
    lib_dir = ROOT / "bonxai_gb300" / "_build"
    # -ffp-contract=off: the program computes its own test points (e.g.
    # -0.5 + 0.3 * a); GCC on aarch64 would fuse those into FMAs by default and
    # the points would differ by an ulp from the oracle replay below.
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-Wall", "-Wextra",
                           "-Werror",
                           f"-I{ROOT / 'include'}", str(ROOT / "tests" / "cpp" / "dropin_main.cpp"),
                           f"-L{lib_dir}", "-lbonxai_gb300", f"-Wl,-rpath,{lib_dir}", "-o", str(out)])
    return out


def test_dropin_program_matches_oracle(dropin_exe, tmp_path, port):
    scene = synth.LidarScene()
    n_scans, n_pts = 3, 8192
    scans = [scene.scan(k, n_points=n_pts) for k in range(n_scans)]
    with open(tmp_path / "scans.bin", "wb") as f:
        np.array([n_scans, n_pts], np.int32).tofile(f)
        np.array([scene.resolution, scene.max_range], np.float64).tofile(f)
        for pts, o in scans:
            o.astype(np.float32).tofile(f)
            pts.astype(np.float32).tofile(f)
    r = subprocess.run([str(dropin_exe), str(tmp_path / "scans.bin"), str(tmp_path)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr

    # --- tutorial flow, replayed on the oracle
    g = port.grid(0.1, 2, 3, 4)  # int64 ("long")
    b = port.grid(0.1, 2, 3, 1)
    xs = []
    x = -1.0
    while x < 1.0:
        xs.append(x)
        x += 0.1
    P = np.array([(a, bb, c) for a in xs for bb in xs for c in xs], np.float64)
    coords = g.pos_to_coord(P)
    g.set_values(coords, np.arange(len(P), dtype=np.int64))
    b.set_cells_on(coords, 0)
    c555 = g.pos_to_coord([[0.55, 0.55, 0.55]])
    g.set_values(c555, np.array([77], np.int64))
    b.set_cells_on(c555, 0)
    lines = dict(l.split(" ", 1) for l in (tmp_path / "tutorial.txt").read_text().splitlines())
    assert lines["cells"] == f"{g.active_cells()} {b.active_cells()}"
    assert lines["origin"] == "500" and lines["far"] == "1"
    o = g.pos_to_coord([[0.0, 0.0, 0.0]])
    g.set_values(o, np.array([500], np.int64))
    g.get_values(g.pos_to_coord([[10.0, 10.0, 10.0]]), create=True)
    xyz, v = g.dump()
    below = (xyz[:, 2].astype(np.float64) * 0.1) < -0.1
    g.set_cells_off(xyz[below])
    assert lines["after_visit"] == f"{g.active_cells()} sum {g.active_cells()}"
    assert lines["const_origin"] == "1"
    assert lines["const_below"] == "nullptr"
    assert lines["binary_on"] == "1"
    assert lines["serialization"] == "long 2 3 round_trip_ok"
    assert (tmp_path / "node.txt").read_text().split() == ["ingest", "same", "export", "same"]

    # --- tree walk through rootMap() / getLeafGrid(), replayed on the oracle
    t = dict(l.split(" ", 1) for l in (tmp_path / "tree.txt").read_text().splitlines())
    tg = port.grid(0.05, 2, 3, 1)  # int32
    i = np.arange(3000)
    tc = np.stack([(i * 37) % 211 - 100, (i * 53) % 97 - 40, (i * 11) % 61 - 30], 1)
    tg.set_values(tc.astype(np.int32), (i * 7 + 1).astype(np.int32))
    walk = t["walk"].split()
    assert walk[0] == "same"
    assert [int(x) for x in walk[1:]] == [tg.root_count(), tg.leaf_count(), tg.active_cells()]
    assert t["leaf_copies"] == "same" and t["missing_leaf"] == "nullptr"
    assert t["pointers"] == "stable stored"
    assert t["leaf_create"] == "empty 4242"

    # --- probabilistic map flow
    m = port.pmap(scene.resolution)
    for pts, org in scans:
        m.insert(pts, org, scene.max_range)
    for i in range(200):
        a = 0.01 * i
        m.add_hit(np.array([[1.0 + a, -0.5 + 0.3 * a, 0.8]]))
        if i % 3 == 0:
            m.add_miss(np.array([[-2.0 - a, 0.5, 1.2 + 0.1 * a]]))
    m.update_free_cells([0.05, 0.05, 1.0])
    ox, oc = m.dump()
    raw = np.fromfile(tmp_path / "cells.bin", np.int32).reshape(-1, 4)
    order = np.lexsort((raw[:, 2], raw[:, 1], raw[:, 0]))
    assert np.array_equal(raw[order, :3], ox) and np.array_equal(raw[order, 3], oc)
    occ = np.fromfile(tmp_path / "occupied.bin", np.int32).reshape(-1, 3)
    occ = occ[np.lexsort((occ[:, 2], occ[:, 1], occ[:, 0]))]
    assert np.array_equal(occ, m.occupied())
    summ = (tmp_path / "summary.txt").read_text().split()
    assert summ[3] == summ[5]  # every probed occupied voxel answers isOccupied
