"""GPU ProbabilisticMap vs the CPU oracle, bit-exact (cells, packed CellT
words, ray-cell totals, query answers)."""
import numpy as np
import pytest
import torch

from conftest import golden
from bonxai_gb300 import synth

pytestmark = pytest.mark.gpu


def assert_same_map(gmap, omap):
    gx, gc = gmap.dump()
    ox, oc = omap.dump()
    assert len(gx) == len(ox), (len(gx), len(ox))
    assert np.array_equal(gx, ox)
    bad = np.nonzero(gc != oc)[0]
    assert len(bad) == 0, (len(bad), gx[bad[:5]], gc[bad[:5]], oc[bad[:5]])


def test_golden_lidar(gpu):
    g = golden("pmap_lidar.npz")
    m = gpu.ProbabilisticMap(float(g["resolution"]))
    for k in range(len(g["points"])):
        v = m.insert_point_cloud(g["points"][k], g["origins"][k], float(g["max_range"]))
        assert v == g["v"][k]
        if k == 2:
            xyz, c = m.dump()
            assert np.array_equal(xyz, g["xyz3"]) and np.array_equal(c, g["cells3"])
    xyz, c = m.dump()
    assert np.array_equal(xyz, g["xyz8"]) and np.array_equal(c, g["cells8"])
    assert np.array_equal(m.is_occupied(g["query"]), g["occ"])
    assert np.array_equal(m.is_unknown(g["query"]), g["unk"])
    assert np.array_equal(m.is_free(g["query"]), g["fre"])
    assert np.array_equal(m.get_occupied_voxels(), g["occupied"])
    assert np.array_equal(m.get_free_voxels(), g["free"])


def test_golden_repeat(gpu):
    g = golden("pmap_repeat.npz")
    m = gpu.ProbabilisticMap(float(g["resolution"]))
    vs = [m.insert_point_cloud(g["points"], g["origin"], float(g["max_range"]))
          for _ in range(7)]
    assert vs == list(g["v"])
    assert m.update_count == 1 + 7 % 3
    xyz, c = m.dump()
    assert np.array_equal(xyz, g["xyz"]) and np.array_equal(c, g["cells"])


def test_golden_add_points(gpu):
    g = golden("pmap_addpts.npz")
    m = gpu.ProbabilisticMap(float(g["resolution"]))
    for k in range(len(g["hits"])):
        m.add_hit_points(g["hits"][k])
        m.add_miss_points(g["misses"][k])
        assert m.update_free_cells(g["origins"][k]) == g["ray_cells"][k]
    xyz, c = m.dump()
    assert np.array_equal(xyz, g["xyz"]) and np.array_equal(c, g["cells"])


@pytest.mark.parametrize("rpw,unroll", [(1, 1), (2, 1), (4, 1), (1, 2), (2, 2), (4, 2)])
def test_lidar_scans_vs_oracle(gpu, port, rpw, unroll):
    scene = synth.LidarScene()
    m = gpu.ProbabilisticMap(scene.resolution, gpu.Config(rays_per_warp=rpw, ray_unroll=unroll))
    o = port.pmap(scene.resolution)
    for k in range(5):
        pts, org = scene.scan(k, n_points=16384)
        assert m.insert_point_cloud(pts, org, scene.max_range) == o.insert(pts, org, scene.max_range)
    assert_same_map(m, o)


def test_scans_interleaved_with_grid_writes_and_added_points(gpu, port):
    """Scans share a scratch table with the grid-view batch calls and with
    addHitPoint/addMissPoint batches (the ray kernel leaves it empty for the
    next scan); interleaving all three must not change any result."""
    scene = synth.LidarScene()
    m = gpu.ProbabilisticMap(0.1)
    o = port.pmap(0.1)
    lib = gpu.load_library()
    rng = np.random.default_rng(12)
    for k in range(5):
        pts, org = scene.scan(k, n_points=20000 + 3000 * k)
        assert m.insert_point_cloud(pts, org, 30.0) == o.insert(pts, org, 30.0)
        if k % 2 == 0:
            # rewrite a third of the cells with their own words: the map is
            # unchanged, the scratch table is not
            xyz, cells = m.dump()
            c = np.ascontiguousarray(xyz[::3])
            w = np.ascontiguousarray(cells[::3])
            assert lib.bxg_grid_set_values(lib.bxg_pmap_grid(m.h), c.ctypes.data, w.ctypes.data,
                                           len(c), None) == 0
        else:
            h = (org + rng.normal(0, 3, (500, 3))).astype(np.float64)
            mi = (org + rng.normal(0, 3, (300, 3))).astype(np.float64)
            m.add_hit_points(h)
            o.add_hit(h)
            m.add_miss_points(mi)
            o.add_miss(mi)
            assert m.update_free_cells(org.astype(np.float64)) == o.update_free_cells(
                org.astype(np.float64))
    assert_same_map(m, o)


def test_leaf_directory_vs_oracle(gpu, port):
    """The leaf directory of the ray walk gives the oracle's maps: 20 LiDAR scans
    (the 4-bit epoch wraps), a clear in between, tiny pools that grow
    mid-scan, depth frames at 0.02 m, and scans after queued hit/miss points."""
    F = 0
    scene = synth.LidarScene()
    m = gpu.ProbabilisticMap(scene.resolution, gpu.Config(flags=F))
    o = port.pmap(scene.resolution)
    for k in range(20):
        pts, org = scene.scan(k, n_points=8192)
        assert m.insert_point_cloud(pts, org, scene.max_range) == o.insert(pts, org, scene.max_range)
        if k == 9:
            # grid().clear() keeps the scan counter (as in the reference): a
            # fresh oracle map is advanced to the same counter by empty
            # updateFreeCells calls
            assert_same_map(m, o)
            m.clear()
            o = port.pmap(scene.resolution)
            while o.update_count != m.update_count:
                o.update_free_cells(np.zeros(3))
    assert_same_map(m, o)
    tiny = gpu.Config(flags=F, initial_leaves=16, initial_inners=4, hash_buckets=16)
    m2 = gpu.ProbabilisticMap(scene.resolution, tiny)
    o2 = port.pmap(scene.resolution)
    for k in range(3):
        pts, org = scene.scan(k, n_points=20000)
        assert m2.insert_point_cloud(pts, org, 30.0) == o2.insert(pts, org, 30.0)
        h = (org + np.random.default_rng(k).normal(0, 40, (200, 3))).astype(np.float64)
        m2.add_hit_points(h)
        o2.add_hit(h)
    pts, org = scene.scan(5, n_points=20000)
    assert m2.insert_point_cloud(pts, org, 30.0) == o2.insert(pts, org, 30.0)
    assert_same_map(m2, o2)
    room = synth.DepthRoom()
    m3 = gpu.ProbabilisticMap(room.resolution, gpu.Config(flags=F))
    o3 = port.pmap(room.resolution)
    for k in range(3):
        pts, org = room.frame(k, subsample=8)
        assert m3.insert_point_cloud(pts, org, room.max_range) == o3.insert(pts, org, room.max_range)
    assert_same_map(m3, o3)


def test_leaf_directory_across_scans(gpu, port):
    """The leaf directory kept across scans. 20 scans of a sensor moving 9.5 m
    (its cube is re-centred once the origin leaves the margin) match the
    oracle. Then cells are switched off and their leaves released through
    grid(): later scans, whose new leaves reuse the released slots, match a
    twin map rebuilt from the same state with a fresh directory."""
    scene = synth.LidarScene()
    m = gpu.ProbabilisticMap(scene.resolution)
    o = port.pmap(scene.resolution)
    for k in range(20):
        pts, org = scene.scan(k, n_points=8192)
        assert m.insert_point_cloud(pts, org, scene.max_range) == o.insert(pts, org, scene.max_range)
    assert_same_map(m, o)

    m2 = gpu.ProbabilisticMap(scene.resolution)
    for k in range(5):
        pts, org = scene.scan(k, n_points=8192)
        m2.insert_point_cloud(pts, org, scene.max_range)
    xyz, _ = m2.dump()
    # every on-cell of the leaves within 7 leaves of the next origin: those
    # leaves empty out and are released
    _, org5 = scene.scan(5, n_points=8192)
    c5 = np.floor(np.asarray(org5, np.float64) / scene.resolution).astype(np.int64) >> 3
    sel = np.all(np.abs((xyz.astype(np.int64) >> 3) - c5) <= 7, axis=1)
    assert sel.sum() > 1000
    g = m2.grid()
    roots0, leaves0 = g.node_counts()
    g.set_cells_off(xyz[sel])
    g.release_unused_memory()
    assert g.node_counts()[1] < leaves0
    twin = gpu.ProbabilisticMap(scene.resolution)
    twin.grid().deserialize(g.serialize("int"))
    while twin.update_count != m2.update_count:
        twin.update_free_cells(np.zeros(3))
    for k in range(5, 10):
        pts, org = scene.scan(k, n_points=8192)
        assert m2.insert_point_cloud(pts, org, scene.max_range) == \
            twin.insert_point_cloud(pts, org, scene.max_range)
    a, b = m2.dump(), twin.dump()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_depth_frames_vs_oracle(gpu, port):
    room = synth.DepthRoom()
    m = gpu.ProbabilisticMap(room.resolution)
    o = port.pmap(room.resolution)
    for k in range(4):
        pts, org = room.frame(k, subsample=16)
        assert m.insert_point_cloud(pts, org, room.max_range) == o.insert(pts, org, room.max_range)
    assert_same_map(m, o)
    xyz, _ = o.dump()
    q = synth.lookup_coords(xyz.min(0), xyz.max(0), 200000, seed=1)
    occ, unk, fre = o.query(q)
    assert np.array_equal(m.is_occupied(q), occ)
    assert np.array_equal(m.is_unknown(q), unk)
    assert np.array_equal(m.is_free(q), fre)


def test_device_resident_points_and_stride(gpu, port):
    scene = synth.LidarScene()
    pts, org = scene.scan(1, n_points=8192)
    m1 = gpu.ProbabilisticMap(0.1)
    m1.insert_point_cloud(torch.from_numpy(pts).cuda(), org, 30.0)
    # pcl::PointXYZ layout: x, y, z, padding (16-byte stride)
    padded = np.zeros((len(pts), 4), np.float32)
    padded[:, :3] = pts
    m2 = gpu.ProbabilisticMap(0.1)
    m2.insert_point_cloud(padded, org, 30.0, stride=16)
    o = port.pmap(0.1)
    o.insert(pts, org, 30.0)
    assert_same_map(m1, o)
    assert_same_map(m2, o)


def test_double_points(gpu, port):
    rng = np.random.default_rng(3)
    org = np.array([0.013, -0.27, 0.5])
    pts = org + rng.normal(0, 3.0, (20000, 3))
    m = gpu.ProbabilisticMap(0.05)
    o = port.pmap(0.05)
    for _ in range(4):
        assert m.insert_point_cloud(pts, org, 4.0) == o.insert(pts, org, 4.0)
    assert_same_map(m, o)


def test_custom_options_and_clamps(gpu, port):
    rng = np.random.default_rng(4)
    opts = [-900000, 1300000, -2500000, 2000000, 100000]
    m = gpu.ProbabilisticMap(0.1)
    o = port.pmap(0.1)
    m.options = opts
    o.options = opts
    assert list(m.options) == opts
    org = np.zeros(3, np.float32)
    for k in range(6):
        pts = rng.normal(0, 1.5, (6000, 3)).astype(np.float32)
        assert m.insert_point_cloud(pts, org, 2.0) == o.insert(pts, org, 2.0)
    assert_same_map(m, o)
    q = rng.integers(-40, 40, (50000, 3)).astype(np.int32)
    assert np.array_equal(m.is_occupied(q), o.query(q)[0])
    assert np.array_equal(m.is_free(q), o.query(q)[2])


def test_edge_cases(gpu, port):
    m = gpu.ProbabilisticMap(0.1)
    o = port.pmap(0.1)
    org = np.array([0.05, 0.05, 0.05], np.float32)
    empty = np.zeros((0, 3), np.float32)
    assert m.insert_point_cloud(empty, org, 5.0) == o.insert(empty, org, 5.0) == 0
    assert m.update_count == o.update_count == 2
    # points in the origin cell: no ray; duplicates; a point exactly at max range
    pts = np.array([[0.06, 0.07, 0.08], [0.06, 0.07, 0.08], [5.05, 0.05, 0.05],
                    [0.05, 5.05, 0.05], [-3.0, 2.0, 1.0]], np.float32)
    for _ in range(4):
        assert m.insert_point_cloud(pts, org, 5.0) == o.insert(pts, org, 5.0)
    assert_same_map(m, o)


def test_nonfinite_points_are_dropped(gpu, port):
    rng = np.random.default_rng(5)
    pts = rng.normal(0, 2, (5000, 3)).astype(np.float32)
    bad = pts.copy()
    bad[::17, 1] = np.nan
    bad[::23, 2] = np.inf
    keep = np.isfinite(bad).all(1)
    m = gpu.ProbabilisticMap(0.1)
    o = port.pmap(0.1)
    org = np.zeros(3, np.float32)
    m.insert_point_cloud(bad, org, 3.0)
    o.insert(bad[keep], org, 3.0)
    assert_same_map(m, o)


def test_full_size_lidar_20_scans(gpu, port):
    """The 64 x 2048 LiDAR workload at full size, all 20 scans, bit-exact."""
    scene = synth.LidarScene()
    m = gpu.ProbabilisticMap(scene.resolution)
    o = port.pmap(scene.resolution)
    total = 0
    for k in range(20):
        pts, org = scene.scan(k)
        v = m.insert_point_cloud(pts, org, scene.max_range)
        assert v == o.insert(pts, org, scene.max_range)
        total += v
    assert_same_map(m, o)
    assert total > 20 * 131072


def test_growth_from_tiny_pools(gpu, port):
    cfg = gpu.Config(initial_leaves=16, initial_inners=4, hash_buckets=16)
    scene = synth.LidarScene()
    m = gpu.ProbabilisticMap(0.1, cfg)
    o = port.pmap(0.1)
    for k in range(3):
        pts, org = scene.scan(k, n_points=30000)
        assert m.insert_point_cloud(pts, org, 30.0) == o.insert(pts, org, 30.0)
    assert_same_map(m, o)


def test_pool_budget_exhaustion_reports_and_recovers(gpu):
    cfg = gpu.Config(initial_leaves=16, initial_inners=4, hash_buckets=16,
                     pool_budget_bytes=1 << 20)
    scene = synth.LidarScene()
    m = gpu.ProbabilisticMap(0.1, cfg)
    pts, org = scene.scan(0, n_points=30000)
    with pytest.raises(gpu.BonxaiError) as ei:
        m.insert_point_cloud(pts, org, 30.0)
    assert ei.value.status in (2, 3)
    # the handle stays usable
    q = np.zeros((10, 3), np.int32)
    m.is_occupied(q)
    m.clear()
    small = np.array([[0.5, 0.5, 0.5]], np.float32)
    m.insert_point_cloud(small, np.zeros(3, np.float32), 30.0)


def test_kernel_timing_and_stats(gpu, port):
    scene = synth.LidarScene()
    m = gpu.ProbabilisticMap(0.1, gpu.Config(flags=gpu.FLAG_TIMING))
    pts, org = scene.scan(0, n_points=20000)
    v = m.insert_point_cloud(pts, org, 30.0)
    st = m.last_stats()
    assert st["points"] == 20000 and st["ray_cells_visited"] == v - 20000
    t = m.kernel_times()
    assert all(x >= 0 for x in t) and t[3] > 0
    m.is_occupied(np.zeros((50000, 3), np.int32))
    assert m.last_query_ms() > 0


def _adversarial_points(res, origin, max_range, n, seed):
    """Points that sit on or within a few ulps of cell boundaries, and at
    distances within a few ulps of max_range from the origin: the cases where
    a float computation of the endpoint could round differently from the
    reference's double computation."""
    rng = np.random.default_rng(seed)
    o = origin.astype(np.float64)
    k = rng.integers(-400, 400, (n, 3)).astype(np.float64)
    on_grid = (k * res).astype(np.float32)
    ulps = rng.integers(-3, 4, (n, 3)).astype(np.float32)
    toward = np.where(ulps < 0, -np.inf, np.inf).astype(np.float32)
    near_grid = np.where(ulps == 0, on_grid, np.nextafter(on_grid, toward)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    scale = max_range * (1.0 + rng.integers(-8, 9, (n, 1)) * 2.0 ** -23)
    near_range = (o + d * scale).astype(np.float32)
    # misses whose endpoint lands near a cell boundary: directions toward grid points
    tgt = (rng.integers(-300, 300, (n, 3)) * res).astype(np.float64)
    dd = tgt - o
    dd /= np.linalg.norm(dd, axis=1, keepdims=True)
    far = (o + dd * (max_range * rng.uniform(1.0, 3.0, (n, 1)))).astype(np.float32)
    zeros = near_grid.copy()
    zeros[:, rng.integers(0, 3)] = 0.0
    return np.concatenate([on_grid, near_grid, near_range, far, zeros])


@pytest.mark.parametrize("res,origin,max_range", [
    (0.1, np.array([0.0, 0.0, 0.0], np.float32), 30.0),
    (0.1, np.array([1.25, -3.5, 1.7], np.float32), 30.0),
    (0.05, np.array([0.3, 0.1, 0.0], np.float32), 12.5),
    (0.02, np.array([-2.0, 4.0, 1.0], np.float32), 5.0),
    (0.3, np.array([100.0, -50.0, 3.0], np.float32), 60.0),
])
def test_endpoint_filter_adversarial(gpu, port, res, origin, max_range):
    """The float filter of the endpoint math falls back to double wherever the
    result could differ: points on and next to cell boundaries and at max_range,
    per map path and batched, bit-exact with the oracle."""
    pts = _adversarial_points(res, origin, max_range, 4000, seed=int(res * 1000))
    m = gpu.ProbabilisticMap(res)
    o = port.pmap(res)
    for k in range(3):
        p = pts[k::3]
        assert m.insert_point_cloud(p, origin, max_range) == o.insert(p, origin, max_range)
    assert_same_map(m, o)
    b = gpu.Batch()
    bm = gpu.ProbabilisticMap(res)
    o2 = port.pmap(res)
    for k in range(3):
        p = np.ascontiguousarray(pts[k::3])
        rc = b.insert([bm], p, np.array([0, len(p)]), origin.reshape(1, 3), max_range)
        assert rc[0] == o2.insert(p, origin, max_range)
    bx_, bc = bm.dump()
    ox, oc = o.dump()
    assert np.array_equal(bx_, ox) and np.array_equal(bc, oc)


def test_queries_on_cells_with_zero_words(gpu):
    """isOccupied/isUnknown/isFree read the cell word first and the mask only
    for a zero word: cells turned on with a zero word through the grid view
    (and a negative threshold, so that 0 counts as occupied) still answer as
    probabilistic_map.cpp:56-75 does for an existing cell."""
    scene = synth.LidarScene()
    m = gpu.ProbabilisticMap(0.1)
    pts, org = scene.scan(0, n_points=20000)
    m.insert_point_cloud(pts, org, 30.0)
    lib = gpu.load_library()
    xyz, cells = m.dump()
    zero_on = np.ascontiguousarray(xyz[::5])
    fresh = np.ascontiguousarray(np.array([[9000 + k, -9000, 5] for k in range(50)], np.int32))
    both = np.ascontiguousarray(np.concatenate([zero_on, fresh]))
    zeros = np.zeros(len(both), np.int32)
    assert lib.bxg_grid_set_values(lib.bxg_pmap_grid(m.h), both.ctypes.data, zeros.ctypes.data,
                                   len(both), None) == 0
    opts = m.options
    opts[4] = -5
    m.options = opts
    xyz, cells = m.dump()
    on = {tuple(c): int(w) >> 4 for c, w in zip(xyz, cells)}
    q = np.concatenate([xyz[::3], fresh, fresh + 1, synth.lookup_coords(xyz.min(0), xyz.max(0),
                                                                          20000, seed=9)])
    q = np.ascontiguousarray(q.astype(np.int32))
    want_occ = np.array([tuple(c) in on and on[tuple(c)] > -5 for c in q], np.uint8)
    want_unk = np.array([tuple(c) not in on or on[tuple(c)] == -5 for c in q], np.uint8)
    want_fre = np.array([tuple(c) in on and on[tuple(c)] < -5 for c in q], np.uint8)
    assert np.array_equal(m.is_occupied(q), want_occ)
    assert np.array_equal(m.is_unknown(q), want_unk)
    assert np.array_equal(m.is_free(q), want_fre)


def test_ray_phase_counts_each_updated_cell_once(gpu):
    """The two-phase ray update (mark the ray cells, then apply per leaf)
    updates each cell once, so its counter is the exact number of cells the
    ray phase changed: cells whose update_id became the scan's counter, minus
    the endpoint cells (one per cast ray)."""
    scene = synth.LidarScene()
    m = gpu.ProbabilisticMap(0.1)
    for k in range(5):
        pts, org = scene.scan(k, n_points=40000)
        u = m.update_count
        _, before = m.dump(sort=False)
        n_before = int(np.count_nonzero((before & 0xF) == u))
        m.insert_point_cloud(pts, org, 30.0)
        _, after = m.dump(sort=False)
        st = m.last_stats()
        changed = int(np.count_nonzero((after & 0xF) == u)) - n_before
        assert st["ray_cells_updated"] == changed - st["cast_rays"]


def test_single_pass_and_two_phase_ray_update_agree(gpu, port):
    """Maps with FLAG_RAYS_SINGLE_PASS (or KEEP_NONFINITE) walk rays in one pass
    (k_rays); default maps mark and apply. On finite points all give the
    oracle's map."""
    scene = synth.LidarScene()
    a = gpu.ProbabilisticMap(0.1)
    b = gpu.ProbabilisticMap(0.1, gpu.Config(flags=gpu.FLAG_KEEP_NONFINITE))
    c = gpu.ProbabilisticMap(0.1, gpu.Config(flags=gpu.FLAG_RAYS_SINGLE_PASS))
    o = port.pmap(0.1)
    for k in range(4):
        pts, org = scene.scan(k, n_points=25000)
        va = a.insert_point_cloud(pts, org, 30.0)
        vb = b.insert_point_cloud(pts, org, 30.0)
        vc = c.insert_point_cloud(pts, org, 30.0)
        assert va == vb == vc == o.insert(pts, org, 30.0)
    for m in (a, b, c):
        assert_same_map(m, o)
