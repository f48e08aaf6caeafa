"""GPU VoxelGrid<T> vs the CPU oracle."""
import numpy as np
import pytest

from conftest import golden
from bonxai_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,dt,odt", [("f32", np.float32, 0), ("i32", np.int32, 1)])
def test_grid_golden(gpu, name, dt, odt):
    g = golden("grid_setvalue.npz")
    G = gpu.VoxelGrid(0.05, dtype=dt)
    coords = G.pos_to_coord(g["points"])
    assert np.array_equal(coords, g[f"{name}_coords"])
    assert np.array_equal(G.set_values(coords, g[f"{name}_vals"], return_was_on=True),
                          g[f"{name}_was"])
    v, f = G.get_values(g[f"{name}_q"], create=False)
    assert np.array_equal(v, g[f"{name}_qv"]) and np.array_equal(f, g[f"{name}_qf"])
    assert np.array_equal(G.set_cells_off(g[f"{name}_off"]), g[f"{name}_was_off"])
    assert np.array_equal(G.set_cells_on(g[f"{name}_on"], default=dt(7)), g[f"{name}_was_on2"])
    v, f = G.get_values(g[f"{name}_cq"], create=True)
    assert np.array_equal(v, g[f"{name}_cv"]) and np.array_equal(f, g[f"{name}_cf"])
    xyz, v = G.dump()
    assert np.array_equal(xyz, g[f"{name}_xyz"]) and np.array_equal(v, g[f"{name}_v"])
    assert G.active_cells_count() == int(g[f"{name}_active"])


def test_room_cloud_create_update_iterate(gpu, port):
    """VoxelGrid<float> at 0.02 m: create, update, iterate on 300k points."""
    pts = synth.room_cloud(300_000, seed=1000)
    v1 = synth.room_values(len(pts), 1001)
    v2 = synth.room_values(len(pts), 1002)
    G = gpu.VoxelGrid(0.02)
    O = port.grid(0.02)
    G.set_values_at_points(pts, v1)
    coords = O.pos_to_coord(pts.astype(np.float64))
    O.set_values(coords, v1)
    G.set_values_at_points(pts, v2)
    O.set_values(coords, v2)
    a, av = G.dump()
    b, bv = O.dump()
    assert np.array_equal(a, b) and np.array_equal(av.view(np.uint32), bv.view(np.uint32))
    assert G.active_cells_count() == O.active_cells()
    # canonical-order sum (the reference's forEachCell order is an unordered_map's)
    assert float(np.sum(av, dtype=np.float64)) == float(np.sum(bv, dtype=np.float64))


@pytest.mark.parametrize("ib,lb", [(1, 1), (3, 2), (2, 3), (4, 4), (2, 5)])
@pytest.mark.parametrize("dt,odt", [(np.float32, 0), (np.float64, 3), (np.int64, 4)])
def test_grid_ops_vs_oracle(gpu, port, ib, lb, dt, odt):
    rng = np.random.default_rng(ib * 7 + lb)
    coords = rng.integers(-200, 200, (30000, 3)).astype(np.int32)
    coords = np.concatenate([coords, coords[:8000], coords[5000:6000]])
    vals = (rng.random(len(coords)) * 100).astype(dt)
    G = gpu.VoxelGrid(0.1, ib, lb, dtype=dt)
    O = port.grid(0.1, ib, lb, odt)
    assert np.array_equal(G.set_values(coords, vals, return_was_on=True), O.set_values(coords, vals))
    q = np.concatenate([coords[::3], rng.integers(-250, 250, (5000, 3)).astype(np.int32)])
    gv, gf = G.get_values(q)
    ov, of = O.get_values(q)
    assert np.array_equal(gv, ov) and np.array_equal(gf, of)
    off = np.concatenate([coords[::5], coords[::10]])
    assert np.array_equal(G.set_cells_off(off), O.set_cells_off(off))
    on = np.concatenate([off[::2], q[-100:]])
    assert np.array_equal(G.set_cells_on(on, 3), O.set_cells_on(on, 3))
    cq = rng.integers(-260, 260, (4000, 3)).astype(np.int32)
    gv, gf = G.get_values(cq, create=True)
    ov, of = O.get_values(cq, create=True)
    assert np.array_equal(gv, ov) and np.array_equal(gf, of)
    assert np.array_equal(G.is_cell_on(q), O.is_cell_on(q))
    a, av = G.dump()
    b, bv = O.dump()
    assert np.array_equal(a, b) and np.array_equal(av, bv)
    G.release_unused_memory()
    O.release_unused()
    assert G.node_counts()[1] == O.leaf_count()
    assert G.node_counts()[0] == O.root_count()
    a, av = G.dump()
    assert np.array_equal(a, b) and np.array_equal(av, bv)
    # reuse of released leaves
    more = rng.integers(-200, 200, (5000, 3)).astype(np.int32)
    mv = (rng.random(len(more)) * 100).astype(dt)
    G.set_values(more, mv)
    O.set_values(more, mv)
    a, av = G.dump()
    b, bv = O.dump()
    assert np.array_equal(a, b) and np.array_equal(av, bv)
    G.clear(gpu.SET_ALL_CELLS_OFF)
    O.clear(1)
    assert G.active_cells_count() == 0
    G.clear(gpu.CLEAR_MEMORY)
    assert G.node_counts() == (0, 0)


def test_binary_grid(gpu, port):
    rng = np.random.default_rng(8)
    coords = rng.integers(-50, 50, (20000, 3)).astype(np.int32)
    G = gpu.VoxelGrid(0.1, dtype=None)
    O = port.grid(0.1, 2, 3, 1)
    assert np.array_equal(G.set_cells_on(coords), O.set_cells_on(coords, 0))
    off = coords[::3]
    assert np.array_equal(G.set_cells_off(off), O.set_cells_off(off))
    a, _ = G.dump()
    b, _ = O.dump()
    assert np.array_equal(a, b)


def test_tutorial_known_answers(gpu):
    """The reference's examples/tutorial.cpp: a 2x2x2 m cube at 0.1 m holds
    8000 cells; value at the origin can be set; create gives T{}."""
    G = gpu.VoxelGrid(0.1, dtype=np.int64)
    xs = []
    x = -1.0
    while x < 1.0:
        xs.append(x)
        x += 0.1
    P = np.array([(a, b, c) for a in xs for b in xs for c in xs], np.float64)
    coords = G.pos_to_coord(P)
    G.set_values(coords, np.arange(len(P), dtype=np.int64))
    assert G.active_cells_count() == 8000
    o = G.pos_to_coord([[0.0, 0.0, 0.0]])
    G.set_values(o, np.array([500], np.int64))
    v, f = G.get_values(o)
    assert f[0] == 1 and v[0] == 500
    far = G.pos_to_coord([[10.0, 10.0, 10.0]])
    v, f = G.get_values(far, create=True)
    assert f[0] == 1 and v[0] == 0


def test_test_serialization_overwrite_known_answer(gpu, port):
    """examples/test_serialization.cpp writes 1000 values on an accumulated
    0.1 m lattice that maps to only 729 distinct cells: last writer wins."""
    pts = []
    x = -0.5
    while x < 0.5:
        y = -0.5
        while y < 0.5:
            z = -0.5
            while z < 0.5:
                pts.append((x, y, z))
                z += 0.1
            y += 0.1
        x += 0.1
    P = np.array(pts, np.float64)
    G = gpu.VoxelGrid(0.1, dtype=np.int32)
    O = port.grid(0.1, 2, 3, 1)
    c = G.pos_to_coord(P)
    vals = np.arange(len(P), dtype=np.int32)
    G.set_values(c, vals)
    O.set_values(O.pos_to_coord(P), vals)
    assert len(P) == 1000 and G.active_cells_count() == O.active_cells() == 729
    a, av = G.dump()
    b, bv = O.dump()
    assert np.array_equal(a, b) and np.array_equal(av, bv)
