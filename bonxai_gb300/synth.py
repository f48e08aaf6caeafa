"""Seeded synthetic inputs for the five workloads (they stand in for the
reference's missing PCD / KITTI data).

Every generator returns float32 world points (and float32 sensor origins), the
types the reference's insertPointCloud receives from a PCL cloud
(bonxai_ros/src/bonxai_server.cpp:167-182). Randomness comes from numpy's PCG64
with fixed seeds (seed = workload * 1000 + map index).

* room_cloud     -- VoxelGrid<float> create/update/iterate: 300k points on the
                    inner faces of a 6x4x3 m room plus 20 spheres, N(0, 5 mm) noise.
* LidarScene     -- ProbabilisticMap with a 64 x 2048 LiDAR (elevation -25..+15 deg)
                    in a 40x40x8 m scene of 200 boxes on a floor, 20 poses 0.5 m apart
                    along +x at 1.7 m height; misses are emitted at 2 x max_range.
* DepthRoom      -- ProbabilisticMap from a 640x480 pinhole depth camera
                    (fx=fy=525) in an 8x6x3 m room with 50 boxes, 6-DoF random walk
                    (0.05 m, 2 deg steps), depth kept in [0.3, 5] m.
* multi_map_workload -- 64 maps with log-uniform [10k, 500k] points per scan,
                    drawn from the room and LiDAR generators, resolutions cycling
                    0.02 / 0.05 / 0.1 m.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

# ----------------------------------------------------------------------------
# Room + spheres surface cloud (VoxelGrid create / update / iterate)
# ----------------------------------------------------------------------------
ROOM_LO = np.array([-3.0, -2.0, 0.0])
ROOM_HI = np.array([3.0, 2.0, 3.0])


def room_cloud(n_points: int = 300_000, seed: int = 1000, noise: float = 0.005,
               n_spheres: int = 20) -> np.ndarray:
    """Area-uniform samples on the six inner faces of a 6x4x3 m room and on the
    surfaces of ``n_spheres`` spheres (radius U(0.1, 0.5) m) inside it."""
    rng = np.random.default_rng(seed)
    size = ROOM_HI - ROOM_LO
    radii = rng.uniform(0.1, 0.5, n_spheres)
    centers = rng.uniform(ROOM_LO + 0.5, ROOM_HI - 0.5, (n_spheres, 3))
    faces = []  # (area, axis, value)
    for ax in range(3):
        other = [a for a in range(3) if a != ax]
        area = size[other[0]] * size[other[1]]
        faces.append((area, ax, ROOM_LO[ax]))
        faces.append((area, ax, ROOM_HI[ax]))
    areas = np.array([f[0] for f in faces] + list(4 * np.pi * radii ** 2))
    counts = rng.multinomial(n_points, areas / areas.sum())
    parts = []
    for k, c in enumerate(counts):
        if c == 0:
            continue
        if k < 6:
            _, ax, val = faces[k]
            p = rng.uniform(ROOM_LO, ROOM_HI, (c, 3))
            p[:, ax] = val
        else:
            s = k - 6
            d = rng.normal(size=(c, 3))
            d /= np.linalg.norm(d, axis=1, keepdims=True)
            p = centers[s] + radii[s] * d
        parts.append(p)
    pts = np.concatenate(parts)
    pts += rng.normal(0.0, noise, pts.shape)
    rng.shuffle(pts, axis=0)
    return pts.astype(np.float32)


def room_values(n: int, seed: int) -> np.ndarray:
    return np.random.default_rng(seed).random(n, dtype=np.float32)


# ----------------------------------------------------------------------------
# Ray casting against axis-aligned boxes (slab test), chunked
# ----------------------------------------------------------------------------
def _cast_boxes(origin: np.ndarray, dirs: np.ndarray, lo: np.ndarray, hi: np.ndarray,
                chunk: int = 8192) -> np.ndarray:
    """Smallest positive entry distance of each ray into any box; inf if none."""
    out = np.full(len(dirs), np.inf)
    if len(lo) == 0:
        return out
    # zero direction components become tiny ones so every slab bound is finite
    d_all = np.where(dirs == 0, 1e-30, dirs)
    inv_all = (1.0 / d_all).astype(np.float32)
    lo_rel = (lo - origin[None, :]).astype(np.float32)  # [B,3]
    hi_rel = (hi - origin[None, :]).astype(np.float32)
    for s in range(0, len(dirs), chunk):
        inv = inv_all[s:s + chunk]
        tmin = None
        tmax = None
        for ax in range(3):
            a = inv[:, ax:ax + 1] * lo_rel[None, :, ax]  # [c,B]
            b = inv[:, ax:ax + 1] * hi_rel[None, :, ax]
            lo_t = np.minimum(a, b)
            hi_t = np.maximum(a, b)
            tmin = lo_t if tmin is None else np.maximum(tmin, lo_t)
            tmax = hi_t if tmax is None else np.minimum(tmax, hi_t)
        hit = (tmax >= tmin) & (tmax > 1e-6)
        tent = np.where(tmin > 1e-6, tmin, tmax)  # origin inside a box: exit face
        tent = np.where(hit, tent, np.float32(np.inf))
        out[s:s + chunk] = tent.min(axis=1)
    return out


# ----------------------------------------------------------------------------
# LiDAR in a box scene (ProbabilisticMap, 20 sequential scans)
# ----------------------------------------------------------------------------
@dataclass
class LidarScene:
    seed: int = 2000
    n_boxes: int = 200
    extent: float = 20.0       # scene is [-20, 20]^2 x [0, 8] m
    height: float = 8.0
    sensor_z: float = 1.7
    step: float = 0.5
    start_x: float = -5.0
    n_el: int = 64
    n_az: int = 2048
    max_range: float = 30.0
    resolution: float = 0.1

    def __post_init__(self):
        rng = np.random.default_rng(self.seed)
        lo, hi = [], []
        while len(lo) < self.n_boxes:
            size = rng.uniform(0.5, 4.0, 3)
            cxy = rng.uniform(-self.extent + size[:2] / 2, self.extent - size[:2] / 2)
            b_lo = np.array([cxy[0] - size[0] / 2, cxy[1] - size[1] / 2, 0.0])
            b_hi = np.array([cxy[0] + size[0] / 2, cxy[1] + size[1] / 2,
                             min(size[2], self.height)])
            # keep the sensor corridor (|y| < 1.5 m) clear
            if b_lo[1] < 1.5 and b_hi[1] > -1.5:
                continue
            lo.append(b_lo)
            hi.append(b_hi)
        self.box_lo = np.array(lo)
        self.box_hi = np.array(hi)
        el = np.deg2rad(np.linspace(-25.0, 15.0, self.n_el))
        az = np.linspace(0.0, 2 * np.pi, self.n_az, endpoint=False)
        E, A = np.meshgrid(el, az, indexing="ij")
        self.dirs = np.stack([np.cos(E) * np.cos(A), np.cos(E) * np.sin(A), np.sin(E)],
                             axis=-1).reshape(-1, 3)

    def origin(self, scan: int) -> np.ndarray:
        return np.array([self.start_x + self.step * scan, 0.0, self.sensor_z])

    def scan(self, scan: int, n_points: int | None = None):
        """(points float32 [n,3], origin float32 [3]) for scan index ``scan``.
        ``n_points`` < 64*2048 keeps a regular subset of the azimuth columns."""
        o = self.origin(scan)
        dirs = self.dirs
        if n_points is not None and n_points < len(dirs):
            idx = np.linspace(0, len(dirs), n_points, endpoint=False).astype(np.int64)
            dirs = dirs[idx]
        t = _cast_boxes(o, dirs, self.box_lo, self.box_hi)
        with np.errstate(divide="ignore", invalid="ignore"):
            t_floor = np.where(dirs[:, 2] < 0, -o[2] / dirs[:, 2], np.inf)
        t = np.minimum(t, t_floor)
        t = np.where(np.isfinite(t), t, 2.0 * self.max_range)
        pts = o[None, :] + t[:, None] * dirs
        return pts.astype(np.float32), o.astype(np.float32)


# ----------------------------------------------------------------------------
# Depth camera in a room with boxes (ProbabilisticMap, 100 frames)
# ----------------------------------------------------------------------------
def _rot(yaw, pitch, roll):
    cy, sy, cp, sp, cr, sr = (math.cos(yaw), math.sin(yaw), math.cos(pitch), math.sin(pitch),
                              math.cos(roll), math.sin(roll))
    Rz = np.array([[cy, -sy, 0], [sy, cy, 0], [0, 0, 1]])
    Ry = np.array([[cp, 0, sp], [0, 1, 0], [-sp, 0, cp]])
    Rx = np.array([[1, 0, 0], [0, cr, -sr], [0, sr, cr]])
    return Rz @ Ry @ Rx


@dataclass
class DepthRoom:
    seed: int = 3000
    n_boxes: int = 50
    width: int = 640
    height: int = 480
    fx: float = 525.0
    fy: float = 525.0
    cx: float = 319.5
    cy: float = 239.5
    d_min: float = 0.3
    d_max: float = 5.0
    max_range: float = 5.0
    resolution: float = 0.02
    step_m: float = 0.05
    step_deg: float = 2.0

    def __post_init__(self):
        rng = np.random.default_rng(self.seed)
        self.lo = np.array([-4.0, -3.0, 0.0])
        self.hi = np.array([4.0, 3.0, 3.0])
        lo, hi = [], []
        while len(lo) < self.n_boxes:
            size = rng.uniform(0.2, 1.2, 3)
            c = rng.uniform(self.lo[:2] + size[:2] / 2, self.hi[:2] - size[:2] / 2)
            b_lo = np.array([c[0] - size[0] / 2, c[1] - size[1] / 2, 0.0])
            b_hi = np.array([c[0] + size[0] / 2, c[1] + size[1] / 2, size[2]])
            if b_lo[0] < 1.0 and b_hi[0] > -1.0 and b_lo[1] < 1.0 and b_hi[1] > -1.0:
                continue  # keep the camera's start area clear
            lo.append(b_lo)
            hi.append(b_hi)
        self.box_lo = np.array(lo)
        self.box_hi = np.array(hi)
        u, v = np.meshgrid(np.arange(self.width), np.arange(self.height))
        self.rays_cam = np.stack([(u.ravel() - self.cx) / self.fx,
                                  (v.ravel() - self.cy) / self.fy,
                                  np.ones(u.size)], axis=-1)  # z = 1 (depth units)
        self.poses = self._walk(rng, 100)

    def _walk(self, rng, n):
        pos = np.array([0.0, 0.0, 1.5])
        ang = np.zeros(3)
        poses = []
        for _ in range(n):
            poses.append((pos.copy(), ang.copy()))
            d = rng.normal(size=3)
            pos = np.clip(pos + self.step_m * d / np.linalg.norm(d), self.lo + 0.5,
                          self.hi - 0.5)
            ang = ang + np.deg2rad(rng.uniform(-self.step_deg, self.step_deg, 3))
            ang[1] = np.clip(ang[1], -0.6, 0.6)
            ang[2] = np.clip(ang[2], -0.3, 0.3)
        return poses

    def frame(self, k: int, subsample: int = 1):
        """(points float32 [n,3], origin float32 [3]) of frame k. The camera's
        optical axis (+z in the camera frame) is mapped to world +x."""
        pos, ang = self.poses[k]
        cam_to_body = np.array([[0, 0, 1], [-1, 0, 0], [0, -1, 0]], float)
        R = _rot(*ang) @ cam_to_body
        rays = self.rays_cam[::subsample] @ R.T  # world direction, depth-scaled
        # walls: the camera is inside the room, take the exit distance
        with np.errstate(divide="ignore", invalid="ignore"):
            t1 = (self.lo[None] - pos[None]) / rays
            t2 = (self.hi[None] - pos[None]) / rays
            t_wall = np.nanmin(np.where(np.maximum(t1, t2) > 0, np.maximum(t1, t2), np.inf),
                               axis=1)
        t_box = _cast_boxes(pos, rays, self.box_lo, self.box_hi)
        depth = np.minimum(t_wall, t_box)
        keep = (depth >= self.d_min) & (depth <= self.d_max)
        pts = pos[None] + depth[keep, None] * rays[keep]
        return pts.astype(np.float32), pos.astype(np.float32)


def lookup_coords(lo_cell: np.ndarray, hi_cell: np.ndarray, n: int, seed: int) -> np.ndarray:
    """n int32 coordinates uniform in the inclusive cell box [lo_cell, hi_cell]."""
    rng = np.random.default_rng(seed)
    return rng.integers(lo_cell, np.asarray(hi_cell) + 1, (n, 3)).astype(np.int32)


# ----------------------------------------------------------------------------
# 64 independent maps of uneven size
# ----------------------------------------------------------------------------
@dataclass
class MapSpec:
    index: int
    kind: str          # "room" or "lidar"
    resolution: float
    n_points: int
    seed: int


def multi_map_specs(n_maps: int = 64, lo: int = 10_000, hi: int = 500_000,
                    seed: int = 4000) -> list[MapSpec]:
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), n_maps)).astype(np.int64)
    res = [0.02, 0.05, 0.1]
    return [MapSpec(i, "room" if i % 2 == 0 else "lidar", res[i % 3], int(sizes[i]),
                    4000 + i) for i in range(n_maps)]


class MapStream:
    """Scans for one map of the multi-map workload, tick by tick."""

    def __init__(self, spec: MapSpec):
        self.spec = spec
        if spec.kind == "lidar":
            self.scene = LidarScene(seed=spec.seed)
        else:
            self.center = ((ROOM_LO + ROOM_HI) / 2).astype(np.float32)

    def scan(self, tick: int):
        s = self.spec
        if s.kind == "lidar":
            return self.scene.scan(tick % 20, n_points=s.n_points)
        pts = room_cloud(s.n_points, seed=s.seed * 100 + tick)
        return pts, self.center.copy()
