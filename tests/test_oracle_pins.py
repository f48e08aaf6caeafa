"""Pins the CPU restatement (oracle/bonxai_oracle.cpp) to the reference.

Two anchors: the golden fixtures made by the reference's own code
(tests/golden/make_golden.py), replayable anywhere; and, where the reference
sources are mounted, direct comparison with the reference compiled unmodified
on random cases.
"""
import numpy as np
import pytest

from conftest import golden
from bonxai_gb300 import synth


def test_default_options_constants(port):
    # logods(0.4f), logods(0.7f), logods(0.12f), logods(0.97f), logods(0.5)
    # (probabilistic_map.hpp:56-64)
    g = golden("constants.npz")["options"]
    assert list(g) == [-405465, 847297, -1992430, 3476099, 0]
    assert list(port.pmap(0.1).options) == list(g)


def test_rays_golden(port):
    g = golden("rays.npz")
    off = 0
    for (pair, n) in zip(g["pairs"], g["lens"]):
        ray = port.compute_ray(pair[:3], pair[3:])
        assert len(ray) == n
        assert np.array_equal(ray, g["cells"][off:off + n])
        off += n


def test_ray_sample_from_survey(port):
    # (0,0,0) -> (5,2,-3): the end cell is excluded
    ray = port.compute_ray([0, 0, 0], [5, 2, -3])
    assert ray.tolist() == [[0, 0, 0], [1, 0, -1], [2, 1, -1], [3, 1, -2], [4, 2, -2]]
    assert len(port.compute_ray([1, 1, 1], [1, 1, 1])) == 0
    assert port.compute_ray([1, 1, 1], [2, 1, 1]).tolist() == [[1, 1, 1]]


def test_pmap_lidar_golden(port):
    g = golden("pmap_lidar.npz")
    m = port.pmap(float(g["resolution"]))
    for k in range(len(g["points"])):
        v = m.insert(g["points"][k], g["origins"][k], float(g["max_range"]))
        assert v == g["v"][k]
        if k == 2:
            xyz, c = m.dump()
            assert np.array_equal(xyz, g["xyz3"]) and np.array_equal(c, g["cells3"])
    xyz, c = m.dump()
    assert np.array_equal(xyz, g["xyz8"]) and np.array_equal(c, g["cells8"])
    occ, unk, fre = m.query(g["query"])
    assert np.array_equal(occ, g["occ"]) and np.array_equal(unk, g["unk"])
    assert np.array_equal(fre, g["fre"])
    assert np.array_equal(m.occupied(), g["occupied"])
    assert np.array_equal(m.free(), g["free"])


def test_pmap_repeat_golden(port):
    g = golden("pmap_repeat.npz")
    m = port.pmap(float(g["resolution"]))
    vs = [m.insert(g["points"], g["origin"], float(g["max_range"])) for _ in range(7)]
    assert vs == list(g["v"])
    xyz, c = m.dump()
    assert np.array_equal(xyz, g["xyz"]) and np.array_equal(c, g["cells"])


def test_pmap_addpts_golden(port):
    g = golden("pmap_addpts.npz")
    m = port.pmap(float(g["resolution"]))
    for k in range(len(g["hits"])):
        m.add_hit(g["hits"][k])
        m.add_miss(g["misses"][k])
        assert m.update_free_cells(g["origins"][k]) == g["ray_cells"][k]
    xyz, c = m.dump()
    assert np.array_equal(xyz, g["xyz"]) and np.array_equal(c, g["cells"])


@pytest.mark.parametrize("name,dt,odt", [("f32", np.float32, 0), ("i32", np.int32, 1)])
def test_grid_golden(port, name, dt, odt):
    g = golden("grid_setvalue.npz")
    G = port.grid(0.05, 2, 3, odt)
    coords = G.pos_to_coord(g["points"])
    assert np.array_equal(coords, g[f"{name}_coords"])
    assert np.array_equal(G.set_values(coords, g[f"{name}_vals"]), g[f"{name}_was"])
    v, f = G.get_values(g[f"{name}_q"], create=False)
    assert np.array_equal(v, g[f"{name}_qv"]) and np.array_equal(f, g[f"{name}_qf"])
    assert np.array_equal(G.set_cells_off(g[f"{name}_off"]), g[f"{name}_was_off"])
    assert np.array_equal(G.set_cells_on(g[f"{name}_on"], default=dt(7)), g[f"{name}_was_on2"])
    v, f = G.get_values(g[f"{name}_cq"], create=True)
    assert np.array_equal(v, g[f"{name}_cv"]) and np.array_equal(f, g[f"{name}_cf"])
    xyz, v = G.dump()
    assert np.array_equal(xyz, g[f"{name}_xyz"]) and np.array_equal(v, g[f"{name}_v"])
    assert G.active_cells() == int(g[f"{name}_active"])


# ---------------------------------------------------------------- direct pins
def _random_scans(rng, n_scans, n_pts, spread):
    out = []
    for _ in range(n_scans):
        o = rng.uniform(-0.5, 0.5, 3).astype(np.float32)
        pts = (o + rng.normal(0, spread, (n_pts, 3))).astype(np.float32)
        out.append((pts, o))
    return out


@pytest.mark.parametrize("seed,res,mr", [(0, 0.1, 3.0), (1, 0.05, 1.5), (2, 0.2, 100.0)])
def test_port_matches_reference_random(port, ref, seed, res, mr):
    rng = np.random.default_rng(seed)
    scans = _random_scans(rng, 7, 2500, 2.0)
    a, b = port.pmap(res), ref.pmap(res)
    for pts, o in scans:
        assert a.insert(pts, o, mr) == b.insert(pts, o, mr)
    xa, ca = a.dump()
    xb, cb = b.dump()
    assert np.array_equal(xa, xb) and np.array_equal(ca, cb)


def test_reference_count_path_equals_reference_insert(ref):
    """The harness's counting path leaves the same map as insertPointCloud."""
    rng = np.random.default_rng(9)
    scans = _random_scans(rng, 5, 2000, 1.5)
    a, b = ref.pmap(0.1), ref.pmap(0.1)
    for pts, o in scans:
        a.insert(pts, o, 2.5)
        b.insert_reference_path(pts, o, 2.5)
    xa, ca = a.dump()
    xb, cb = b.dump()
    assert np.array_equal(xa, xb) and np.array_equal(ca, cb)


def test_port_matches_reference_lidar(port, ref):
    scene = synth.LidarScene()
    a, b = port.pmap(0.1), ref.pmap(0.1)
    for k in range(4):
        pts, o = scene.scan(k, n_points=20000)
        assert a.insert(pts, o, 30.0) == b.insert(pts, o, 30.0)
    xa, ca = a.dump()
    xb, cb = b.dump()
    assert np.array_equal(xa, xb) and np.array_equal(ca, cb)


# leaf_bits <= 3 only: with leaf_bits >= 4 the reference double-frees a pooled
# leaf on destruction (the deleter of bonxai.hpp:577-581 runs ~LeafGrid() and
# then `delete ptr`, destroying the heap-allocated mask words twice).
@pytest.mark.parametrize("ib,lb", [(2, 3), (1, 1), (3, 2), (4, 3)])
def test_port_grid_matches_reference(port, ref, ib, lb):
    rng = np.random.default_rng(ib * 10 + lb)
    coords = rng.integers(-300, 300, (20000, 3)).astype(np.int32)
    coords = np.concatenate([coords, coords[:5000]])  # duplicates: last writer wins
    vals = rng.random(len(coords)).astype(np.float32)
    a, b = port.grid(0.1, ib, lb, 0), ref.grid(0.1, ib, lb, 0)
    assert np.array_equal(a.set_values(coords, vals), b.set_values(coords, vals))
    off = coords[::7]
    assert np.array_equal(a.set_cells_off(off), b.set_cells_off(off))
    assert np.array_equal(a.set_cells_on(off[::3], 5.0), b.set_cells_on(off[::3], 5.0))
    a.release_unused()
    b.release_unused()
    assert a.leaf_count() == b.leaf_count() and a.root_count() == b.root_count()
    xa, va = a.dump()
    xb, vb = b.dump()
    assert np.array_equal(xa, xb) and np.array_equal(va, vb)
    a.clear(1)
    b.clear(1)
    assert a.active_cells() == b.active_cells() == 0
    assert a.leaf_count() == b.leaf_count()


def test_pos_to_coord_edges(port, ref):
    pts = np.array([[0.0, -0.0, 1e-300], [-1e-9, 0.1, 0.3], [0.29999999999999993, -0.2, 7.0],
                    [123.456, -987.65, 0.05]], np.float64)
    for res in (0.02, 0.05, 0.1, 0.3):
        assert np.array_equal(port.grid(res).pos_to_coord(pts), ref.grid(res).pos_to_coord(pts))


def test_serialized_streams_golden(port):
    """The reference's Serialize streams hold exactly the cells the restatement
    builds from the same inputs (format read by tests/serial_format.py)."""
    import serial_format as sf
    g = golden("serialized.npz")
    header, xyz, vals = sf.parse(g["grid_f32"].tobytes(), 4)
    assert header == "Bonxai::VoxelGrid<float,2,3>(0.050000)"
    G = port.grid(0.05, 2, 3, 0)
    G.set_values(g["grid_coords"], g["grid_values"])
    ox, ov = G.dump()
    assert np.array_equal(xyz, ox) and np.array_equal(vals.view(np.float32).ravel(), ov)
    header, xyz, vals = sf.parse(g["pmap"].tobytes(), 4)
    assert header == "Bonxai::VoxelGrid<Bonxai::ProbabilisticMap::CellT,2,3>(0.100000)"
    lid = golden("pmap_lidar.npz")
    m = port.pmap(0.1)
    for k in range(3):
        m.insert(lid["points"][k], lid["origins"][k], float(lid["max_range"]))
    ox, oc = m.dump()
    assert np.array_equal(xyz, ox) and np.array_equal(vals.view(np.int32).ravel(), oc)


@pytest.mark.parametrize("zband", [(-np.inf, np.inf), (0.0, 2.0), (0.35, 0.35)])
def test_port_export_occupied_matches_reference(port, ref, zband):
    """The restated occupied-point export equals the reference's PointT
    getOccupiedVoxels (coordToPos) with the ROS node's z band applied."""
    scene = synth.LidarScene()
    a, b = port.pmap(0.1), ref.pmap(0.1)
    for k in range(3):
        pts, o = scene.scan(k, n_points=20000)
        a.insert(pts, o, 30.0)
        b.insert(pts, o, 30.0)
    ea, eb = a.export_occupied(*zband), b.export_occupied(*zband)
    assert len(ea) > 0 or zband == (0.35, 0.35)
    assert np.array_equal(ea.view(np.uint32), eb.view(np.uint32))


def test_sensor_to_world_restatement(port):
    """Non-finite points are dropped in order; the transform is float with the
    stated order ((r0*x + r1*y) + r2*z) + t, checked against numpy float32."""
    rng = np.random.default_rng(3)
    p = rng.normal(0, 10, (5000, 3)).astype(np.float32)
    p[7, 1] = np.nan
    p[11, 2] = np.inf
    p[12, 0] = -np.inf
    c, s = np.cos(0.3), np.sin(0.3)
    m = np.array([[c, -s, 0.0, 1.25], [s, c, 0.0, -3.5], [0.0, 0.0, 1.0, 1.7]], np.float32)
    got = port.sensor_to_world(m, p)
    keep = np.isfinite(p).all(axis=1)
    q = p[keep]
    want = np.empty_like(q)
    for r in range(3):
        v = m[r, 0] * q[:, 0]
        v = v + m[r, 1] * q[:, 1]
        v = v + m[r, 2] * q[:, 2]
        want[:, r] = v + m[r, 3]
    assert got.dtype == np.float32 and len(got) == keep.sum()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
