"""Batched ticks (many maps per persistent launch) vs the per-map path and the
CPU oracle: every map bit-identical after every tick."""
import numpy as np
import pytest

from bonxai_gb300 import synth

pytestmark = pytest.mark.gpu


def _specs():
    # mixed sizes, resolutions and generators, as in the multi-map workload
    return [("lidar", 0.1, 20000), ("room", 0.02, 15000), ("lidar", 0.05, 5000),
            ("room", 0.1, 30000), ("lidar", 0.02, 12000), ("room", 0.05, 3000),
            ("lidar", 0.1, 40000), ("room", 0.02, 8000)]


def _scan(kind, n, seed, tick):
    if kind == "lidar":
        return synth.LidarScene(seed=seed).scan(tick, n_points=n)
    pts = synth.room_cloud(n, seed=seed * 10 + tick)
    return pts, ((synth.ROOM_LO + synth.ROOM_HI) / 2).astype(np.float32)


@pytest.mark.parametrize("rpw,unroll,flags", [(1, 1, 0), (2, 1, 0), (1, 1, 4), (1, 2, 0), (4, 2, 0)])
def test_batch_matches_per_map_and_oracle(gpu, port, rpw, unroll, flags):
    specs = _specs()
    cfg = gpu.Config(rays_per_warp=rpw, ray_unroll=unroll, flags=flags)
    batch = gpu.Batch(cfg)
    bmaps = [gpu.ProbabilisticMap(r) for _, r, _ in specs]
    pmaps = [gpu.ProbabilisticMap(r) for _, r, _ in specs]
    omaps = [port.pmap(r) for _, r, _ in specs]
    for tick in range(4):
        scans = [_scan(k, n, 7000 + i, tick) for i, (k, _, n) in enumerate(specs)]
        pts = np.concatenate([s[0] for s in scans])
        off = np.concatenate([[0], np.cumsum([len(s[0]) for s in scans])])
        origins = np.stack([s[1] for s in scans])
        rc = batch.insert(bmaps, pts, off, origins, 6.0)
        for i, (p, o) in enumerate(scans):
            v1 = pmaps[i].insert_point_cloud(p, o, 6.0)
            v2 = omaps[i].insert(p, o, 6.0)
            assert rc[i] == v1 == v2, (tick, i)
    assert batch.stats()["ticks"] == 4
    for i in range(len(specs)):
        bx_, bc = bmaps[i].dump()
        px, pc = pmaps[i].dump()
        ox, oc = omaps[i].dump()
        assert np.array_equal(bx_, ox) and np.array_equal(bc, oc), i
        assert np.array_equal(px, ox) and np.array_equal(pc, oc), i
        assert bmaps[i].update_count == omaps[i].update_count


def test_batch_pool_exhaustion_is_completed(gpu, port):
    """Maps created with tiny pools run out during the tick and are completed
    by the per-map path after growing."""
    tiny = gpu.Config(initial_leaves=16, initial_inners=4, hash_buckets=16)
    scene = synth.LidarScene()
    batch = gpu.Batch()
    maps = [gpu.ProbabilisticMap(0.1, tiny) for _ in range(3)]
    om = [port.pmap(0.1) for _ in range(3)]
    for tick in range(2):
        scans = [scene.scan(tick + 3 * i, n_points=20000) for i in range(3)]
        pts = np.concatenate([s[0] for s in scans])
        off = np.concatenate([[0], np.cumsum([len(s[0]) for s in scans])])
        rc = batch.insert(maps, pts, off, np.stack([s[1] for s in scans]), 30.0)
        for i, (p, o) in enumerate(scans):
            assert rc[i] == om[i].insert(p, o, 30.0)
    for i in range(3):
        a, ac = maps[i].dump()
        b, bc = om[i].dump()
        assert np.array_equal(a, b) and np.array_equal(ac, bc)


def test_batch_rejects_duplicate_maps(gpu):
    batch = gpu.Batch()
    m = gpu.ProbabilisticMap(0.1)
    pts = np.zeros((4, 3), np.float32)
    with pytest.raises(gpu.BonxaiError):
        batch.insert([m, m], pts, [0, 2, 4], np.zeros((2, 3), np.float32), 5.0)
