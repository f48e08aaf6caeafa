"""Parity at the full sizes of the depth-camera and multi-map workloads.

* Depth camera: 100 frames of 640x480 depth (fx = fy = 525) into one map at
  0.02 m and a 5 m range, then isOccupied / isUnknown / isFree on 1 M
  coordinates drawn in the final map's cell box.
* Multi-map: the 64 maps of the uneven workload (10k-500k points each, room
  and LiDAR scenes, 0.02 / 0.05 / 0.1 m, 10 m range) for three ticks, through
  the batched tick and through the per-scan path.

Every cell coordinate, every packed cell word and every query answer is
compared with the CPU oracle (bit-exact). The oracle's maps are built in
spawned processes while the GPU works; they report a digest of each sorted
map (SHA-256 of the coordinates and words) rather than the maps themselves.
"""
from __future__ import annotations

import hashlib
import multiprocessing as mp

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TICKS = 3
N_MAPS = 64
LOOKUPS = 1 << 20


def _digest(xyz: np.ndarray, cells: np.ndarray) -> str:
    o = np.lexsort((xyz[:, 2], xyz[:, 1], xyz[:, 0]))
    h = hashlib.sha256()
    h.update(np.ascontiguousarray(xyz[o], np.int32).tobytes())
    h.update(np.ascontiguousarray(cells[o], np.int32).tobytes())
    return f"{len(cells)}:{h.hexdigest()}"


def _depth_oracle(frames: int, seed_coords: int):
    """Oracle side of the depth workload: ray cells per frame, map digest,
    query answers."""
    from bonxai_gb300 import synth
    from oracle import oracle as O
    room = synth.DepthRoom()
    m = O.port().pmap(room.resolution)
    V = [m.insert(*room.frame(k), room.max_range) for k in range(frames)]
    xyz, cells = m.dump()
    q = synth.lookup_coords(xyz.min(0), xyz.max(0), LOOKUPS, seed=seed_coords)
    occ, unk, fre = m.query(q)
    return V, _digest(xyz, cells), occ, unk, fre


def _multimap_oracle(mine):
    """Oracle side of the multi-map workload for the maps `mine`."""
    import bench
    from oracle import oracle as O
    specs, base = bench.multimap_inputs(N_MAPS, only=set(mine))
    port = O.port()
    out = {}
    for i in mine:
        m = port.pmap(specs[i].resolution)
        V = [m.insert(*bench.multimap_scan(specs[i], base[i], t), bench.MM_RANGE)
             for t in range(TICKS)]
        out[i] = (V, _digest(*m.dump()))
    return out


def test_depth_100_frames_and_1m_queries(gpu):
    import torch
    from bonxai_gb300 import synth
    ctx = mp.get_context("spawn")
    with ctx.Pool(1) as pool:
        want = pool.apply_async(_depth_oracle, (100, 3))
        room = synth.DepthRoom()
        m = gpu.ProbabilisticMap(room.resolution, gpu.Config(initial_leaves=1 << 17))
        V = []
        for k in range(100):
            pts, org = room.frame(k)
            V.append(m.insert_point_cloud(torch.from_numpy(pts).cuda(), org, room.max_range))
        xyz, cells = m.dump()
        q = synth.lookup_coords(xyz.min(0), xyz.max(0), LOOKUPS, seed=3)
        occ, unk, fre = m.is_occupied(q), m.is_unknown(q), m.is_free(q)
        oV, odig, oocc, ounk, ofre = want.get(timeout=1800)
    assert V == oV
    assert _digest(xyz, cells) == odig
    assert np.array_equal(occ, oocc) and np.array_equal(unk, ounk)
    assert np.array_equal(fre, ofre)
    assert occ.any() and unk.any() and fre.any()


def test_multimap_64_full_size_three_ticks(gpu):
    import torch
    import bench
    from bonxai_gb300 import sharding
    specs, base = bench.multimap_inputs(N_MAPS)
    cores = max(1, min(16, mp.cpu_count()))
    ranks = sharding.assign_maps([sp.n_points for sp in specs], cores)
    jobs = [[i for i, r in enumerate(ranks) if r == k] for k in range(cores)]
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        pending = [pool.apply_async(_multimap_oracle, (j,)) for j in jobs if j]
        cfg = gpu.Config(initial_leaves=1 << 16, initial_inners=1 << 12, hash_buckets=1 << 14)
        bmaps = [gpu.ProbabilisticMap(sp.resolution, cfg) for sp in specs]
        pmaps = [gpu.ProbabilisticMap(sp.resolution, cfg) for sp in specs]
        batch = gpu.Batch()
        Vb = [[] for _ in specs]
        Vp = [[] for _ in specs]
        for t in range(TICKS):
            scans = bench.multimap_tick(specs, base, t)
            pts = torch.from_numpy(np.concatenate([s[0] for s in scans])).cuda()
            off = np.concatenate([[0], np.cumsum([len(s[0]) for s in scans])]).astype(np.uint64)
            org = np.stack([s[1] for s in scans])
            rc = batch.insert(bmaps, pts, off, org, bench.MM_RANGE)
            for i in range(N_MAPS):
                Vb[i].append(int(rc[i]))
                Vp[i].append(pmaps[i].insert_point_cloud(pts[int(off[i]):int(off[i + 1])],
                                                         org[i], bench.MM_RANGE))
        got_b = [_digest(*m.dump()) for m in bmaps]
        got_p = [_digest(*m.dump()) for m in pmaps]
        want = {}
        for r in pending:
            want.update(r.get(timeout=1800))
    for i in range(N_MAPS):
        V, dig = want[i]
        assert Vb[i] == V and Vp[i] == V, (i, specs[i])
        assert got_b[i] == dig, (i, specs[i])
        assert got_p[i] == dig, (i, specs[i])
