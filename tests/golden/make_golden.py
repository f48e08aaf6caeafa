"""Generates the golden fixtures in tests/golden/ from the reference's own code.

Run where the reference sources are mounted (it builds oracle/_ref with
oracle/build_ref.sh): ``python tests/golden/make_golden.py``. Each fixture
stores its inputs and the reference's outputs, so tests can replay them
anywhere without the reference.

Fixtures
  rays.npz          ComputeRay for every end cell in [-5,5]^3 around two
                    origins (probabilistic_map.hpp:13-19,162-203).
  pmap_lidar.npz    8 insertPointCloud scans of 2000 LiDAR points (0.1 m, max
                    range 12 m so that both hits and max-range misses occur),
                    sorted cells + packed CellT words after scans 3 and 8, the
                    ray-cell totals, and isOccupied/isUnknown/isFree answers.
  pmap_repeat.npz   the same 1500-point scan inserted 7 times (exercises the
                    update_id cycle 1->2->3->1 and the skip of cells already at
                    the current id).
  pmap_addpts.npz   addHitPoint/addMissPoint batches then updateFreeCells.
  grid_setvalue.npz VoxelGrid<float> and <int32> setValue with duplicates
                    (last writer wins), value(create), setCellOn/Off, was_on.
  serialized.npz    the reference's Serialize byte streams of a VoxelGrid<float>
                    and of a ProbabilisticMap's grid after 3 LiDAR scans.
  constants.npz     default Options (logods of 0.4, 0.7, 0.12, 0.97, 0.5).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from bonxai_gb300 import synth  # noqa: E402
from oracle import oracle as O  # noqa: E402


FIX_RANGE = 12.0


def sorted_dump(m):
    return m.dump()


def main():
    if O.build_ref() is None:
        raise SystemExit("reference sources not mounted; cannot make golden fixtures")
    R = O.ref()
    assert R is not None

    # ---- rays
    origins = np.array([[0, 0, 0], [3, -7, 11]], np.int32)
    ends, lens, cells = [], [], []
    r = np.arange(-5, 6)
    grid = np.stack(np.meshgrid(r, r, r, indexing="ij"), -1).reshape(-1, 3).astype(np.int32)
    for o in origins:
        for d in grid:
            e = o + d
            ray = R.compute_ray(o, e)
            ends.append(np.concatenate([o, e]))
            lens.append(len(ray))
            cells.append(ray)
    np.savez_compressed(HERE / "rays.npz", pairs=np.array(ends, np.int32),
                        lens=np.array(lens, np.int32),
                        cells=np.concatenate(cells).astype(np.int32))

    # ---- LiDAR scans
    scene = synth.LidarScene()
    scans = [scene.scan(k, n_points=2000) for k in range(8)]
    m = R.pmap(scene.resolution)
    vs = []
    snaps = {}
    for k, (pts, o) in enumerate(scans):
        vs.append(m.insert(pts, o, FIX_RANGE))
        if k in (2, 7):
            snaps[k] = sorted_dump(m)
    xyz, cells_ = snaps[7]
    rng = np.random.default_rng(5)
    q = rng.integers(xyz.min(0) - 3, xyz.max(0) + 4, (20000, 3)).astype(np.int32)
    q = np.concatenate([q, xyz[::7]])
    occ, unk, fre = m.query(q)
    np.savez_compressed(
        HERE / "pmap_lidar.npz", points=np.stack([s[0] for s in scans]),
        origins=np.stack([s[1] for s in scans]), max_range=FIX_RANGE,
        resolution=scene.resolution, v=np.array(vs, np.uint64), xyz3=snaps[2][0],
        cells3=snaps[2][1], xyz8=xyz, cells8=cells_, query=q, occ=occ, unk=unk, fre=fre,
        occupied=m.occupied(), free=m.free())

    # ---- the same scan, 7 times
    pts, o = scene.scan(3, n_points=1500)
    m = R.pmap(scene.resolution)
    vs = [m.insert(pts, o, 12.0) for _ in range(7)]
    xyz, cells_ = sorted_dump(m)
    np.savez_compressed(HERE / "pmap_repeat.npz", points=pts, origin=o, max_range=12.0,
                        resolution=scene.resolution, v=np.array(vs, np.uint64), xyz=xyz,
                        cells=cells_)

    # ---- addHitPoint / addMissPoint / updateFreeCells
    rng = np.random.default_rng(11)
    m = R.pmap(0.05)
    batches = []
    for k in range(3):
        hits = rng.normal(0, 0.6, (400, 3))
        misses = rng.normal(0, 1.2, (300, 3))
        dup = hits[:50] + 1e-4  # same cells, later index
        m.add_hit(hits)
        m.add_miss(np.concatenate([dup, misses]))
        origin = rng.normal(0, 0.1, 3)
        rc = m.update_free_cells(origin)
        batches.append((hits, np.concatenate([dup, misses]), origin, rc))
    xyz, cells_ = sorted_dump(m)
    np.savez_compressed(HERE / "pmap_addpts.npz", hits=np.stack([b[0] for b in batches]),
                        misses=np.stack([b[1] for b in batches]),
                        origins=np.stack([b[2] for b in batches]),
                        ray_cells=np.array([b[3] for b in batches], np.uint64), resolution=0.05,
                        xyz=xyz, cells=cells_)

    # ---- VoxelGrid setValue & co
    out = {}
    pts = synth.room_cloud(6000, seed=21).astype(np.float64)
    for name, dt, odt in (("f32", np.float32, O.ORC_F32), ("i32", np.int32, O.ORC_I32)):
        g = R.grid(0.05, 2, 3, odt)
        coords = g.pos_to_coord(pts)
        vals = (np.random.default_rng(3).random(len(pts)) * 1000).astype(dt)
        was = g.set_values(coords, vals)
        qv = np.concatenate([coords[::5], coords[::5] + 1000])
        gv, gf = g.get_values(qv, create=False)
        off = coords[::9]
        was_off = g.set_cells_off(off)
        on = np.concatenate([off[::2], coords[::11] + 2])
        was_on2 = g.set_cells_on(on, default=dt(7))
        cv, cf = g.get_values(coords[::13] - 3, create=True)
        xyz, v = g.dump()
        out.update({f"{name}_coords": coords, f"{name}_vals": vals, f"{name}_was": was,
                    f"{name}_q": qv, f"{name}_qv": gv, f"{name}_qf": gf, f"{name}_off": off,
                    f"{name}_was_off": was_off, f"{name}_on": on, f"{name}_was_on2": was_on2,
                    f"{name}_cq": coords[::13] - 3, f"{name}_cv": cv, f"{name}_cf": cf,
                    f"{name}_xyz": xyz, f"{name}_v": v,
                    f"{name}_active": g.active_cells()})
    out["points"] = pts
    np.savez_compressed(HERE / "grid_setvalue.npz", **out)

    # ---- Serialize (serialization.hpp:77-116) of a grid and of a map's grid
    gpts = np.load(HERE / "grid_setvalue.npz")["points"]
    g = R.grid(0.05, 2, 3, O.ORC_F32)
    gc = g.pos_to_coord(gpts)
    gv = (np.random.default_rng(3).random(len(gpts)) * 1000).astype(np.float32)
    g.set_values(gc, gv)
    m = R.pmap(scene.resolution)
    lid = np.load(HERE / "pmap_lidar.npz")
    for k in range(3):
        m.insert(lid["points"][k], lid["origins"][k], float(lid["max_range"]))
    np.savez_compressed(HERE / "serialized.npz",
                        grid_f32=np.frombuffer(g.serialize_reference(), np.uint8),
                        grid_coords=gc, grid_values=gv,
                        pmap=np.frombuffer(m.serialize_reference(), np.uint8))

    # ---- constants
    m = R.pmap(0.1)
    np.savez_compressed(HERE / "constants.npz", options=m.options)
    for f in sorted(HERE.glob("*.npz")):
        print(f.name, f.stat().st_size)


if __name__ == "__main__":
    main()
