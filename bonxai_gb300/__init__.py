"""bonxai_gb300 -- GB300-native sparse voxel grid and probabilistic occupancy map.

Python front end of the C ABI in include/bonxai_gb300.h (the C++ drop-in
headers in include/bonxai/ and include/bonxai_map/ are the other front end).
The classes mirror the reference's interface (bonxai_core/include/bonxai/
bonxai.hpp: VoxelGrid; bonxai_map/include/bonxai_map/probabilistic_map.hpp:
ProbabilisticMap) as batch calls: arrays of coordinates or points in, arrays
out. Arrays may be numpy arrays (host) or CUDA torch tensors (device); the
library stages host arrays itself.

There is no CPU fallback: if the CUDA library is missing or no GPU is visible,
constructing a map raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

__all__ = ["VoxelGrid", "ProbabilisticMap", "Batch", "Server", "BonxaiError", "Config",
           "ServerConfig", "load_library",
           "compute_rays", "library_path", "CLEAR_MEMORY", "SET_ALL_CELLS_OFF"]

PKG = Path(__file__).resolve().parent
_LIB_PATH = PKG / "_build" / "libbonxai_gb300.so"

CLEAR_MEMORY = 0
SET_ALL_CELLS_OFF = 1

FLAG_KEEP_NONFINITE = 1
FLAG_TIMING = 2
FLAG_NO_GRAPH = 4
FLAG_RAYS_SINGLE_PASS = 8

STATUS = {0: "ok", 1: "invalid argument", 2: "node pool exhausted", 3: "root hash full",
          4: "device wait timed out", 5: "CUDA error", 6: "no CUDA device",
          7: "output buffer too small"}


class BonxaiError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Config(C.Structure):
    _fields_ = [("pool_budget_bytes", C.c_size_t), ("initial_leaves", C.c_uint32),
                ("initial_inners", C.c_uint32), ("hash_buckets", C.c_uint32),
                ("hash_load_factor", C.c_float), ("device", C.c_int),
                ("stream", C.c_void_p), ("rays_per_warp", C.c_uint32),
                ("block_size", C.c_uint32), ("flags", C.c_uint32),
                ("ray_unroll", C.c_uint32)]

    def __init__(self, **kw):
        super().__init__()
        self.device = -1
        for k, v in kw.items():
            setattr(self, k, v)


class Options(C.Structure):
    _fields_ = [("prob_miss_log", C.c_int32), ("prob_hit_log", C.c_int32),
                ("clamp_min_log", C.c_int32), ("clamp_max_log", C.c_int32),
                ("occupancy_threshold_log", C.c_int32)]


_vp, _sz, _int, _dbl, _u64p = C.c_void_p, C.c_size_t, C.c_int, C.c_double, C.POINTER(C.c_uint64)
_SIGS = {
    "bxg_config_default": (None, [_vp]),
    "bxg_status_string": (C.c_char_p, [_int]),
    "bxg_version": (_int, []),
    "bxg_last_error": (C.c_char_p, [_vp]),
    "bxg_grid_create": (_int, [_vp, _dbl, _int, _int, _sz, _vp]),
    "bxg_grid_destroy": (_int, [_vp]),
    "bxg_grid_pos_to_coord": (_int, [_vp, _vp, _sz, _vp]),
    "bxg_grid_set_values": (_int, [_vp, _vp, _vp, _sz, _vp]),
    "bxg_grid_set_values_noalloc": (_int, [_vp, _vp, _vp, _sz]),
    "bxg_grid_set_values_at_points_f32": (_int, [_vp, _vp, _sz, _sz, _vp]),
    "bxg_grid_set_values_at_points_f64": (_int, [_vp, _vp, _sz, _sz, _vp]),
    "bxg_grid_get_values": (_int, [_vp, _vp, _sz, _vp, _vp, _int]),
    "bxg_grid_set_cells_on": (_int, [_vp, _vp, _sz, _vp, _vp]),
    "bxg_grid_set_cells_off": (_int, [_vp, _vp, _sz, _vp]),
    "bxg_grid_is_cell_on": (_int, [_vp, _vp, _sz, _vp]),
    "bxg_grid_active_cells": (_int, [_vp, _vp]),
    "bxg_grid_node_counts": (_int, [_vp, _vp, _vp]),
    "bxg_grid_mem_usage": (_int, [_vp, _vp]),
    "bxg_grid_dump": (_int, [_vp, _vp, _vp, _sz, _vp]),
    "bxg_grid_clear": (_int, [_vp, _int]),
    "bxg_grid_release_unused": (_int, [_vp]),
    "bxg_grid_synchronize": (_int, [_vp]),
    "bxg_grid_serialize": (_int, [_vp, C.c_char_p, _vp, _sz, _vp]),
    "bxg_grid_deserialize": (_int, [_vp, _vp, _sz]),
    "bxg_pmap_create": (_int, [_vp, _dbl, _vp]),
    "bxg_pmap_destroy": (_int, [_vp]),
    "bxg_pmap_get_options": (_int, [_vp, _vp]),
    "bxg_pmap_set_options": (_int, [_vp, _vp]),
    "bxg_pmap_insert_point_cloud_f32": (_int, [_vp, _vp, _sz, _sz, _vp, _dbl, _vp]),
    "bxg_pmap_insert_point_cloud_f64": (_int, [_vp, _vp, _sz, _sz, _vp, _dbl, _vp]),
    "bxg_pmap_insert_point_cloud_f32_async": (_int, [_vp, _vp, _sz, _sz, _vp, _dbl]),
    "bxg_pmap_add_hit_points": (_int, [_vp, _vp, _sz]),
    "bxg_pmap_add_miss_points": (_int, [_vp, _vp, _sz]),
    "bxg_pmap_update_free_cells": (_int, [_vp, _vp, _vp]),
    "bxg_pmap_is_occupied": (_int, [_vp, _vp, _sz, _vp]),
    "bxg_pmap_is_unknown": (_int, [_vp, _vp, _sz, _vp]),
    "bxg_pmap_is_free": (_int, [_vp, _vp, _sz, _vp]),
    "bxg_pmap_get_occupied": (_int, [_vp, _vp, _sz, _vp]),
    "bxg_pmap_export_occupied_f32": (_int, [_vp, _vp, _sz, _vp, _dbl, _dbl]),
    "bxg_pmap_insert_sensor_cloud_f32": (_int, [_vp, _vp, _sz, _sz, _vp, _dbl, _vp]),
    "bxg_pmap_get_free": (_int, [_vp, _vp, _sz, _vp]),
    "bxg_pmap_dump": (_int, [_vp, _vp, _vp, _sz, _vp]),
    "bxg_pmap_active_cells": (_int, [_vp, _vp]),
    "bxg_pmap_node_counts": (_int, [_vp, _vp, _vp]),
    "bxg_pmap_mem_usage": (_int, [_vp, _vp]),
    "bxg_pmap_update_count": (_int, [_vp, _vp]),
    "bxg_pmap_clear": (_int, [_vp]),
    "bxg_pmap_synchronize": (_int, [_vp]),
    "bxg_pmap_last_stats": (_int, [_vp, _vp]),
    "bxg_pmap_kernel_times": (_int, [_vp, _vp]),
    "bxg_pmap_stream": (_vp, [_vp]),
    "bxg_pmap_grid": (_vp, [_vp]),
    "bxg_debug_hold_leaf": (_int, [_vp, _vp]),
    "bxg_pmap_last_query_ms": (_int, [_vp, _vp]),
    "bxg_pmap_add_points": (_int, [_vp, _vp, _vp, _sz]),
    "bxg_grid_store_if_on": (_int, [_vp, _vp, _vp, _sz]),
    "bxg_compute_rays": (_int, [_vp, _vp, _sz, _vp, _vp, _vp]),
    "bxg_batch_create": (_int, [_vp, _vp]),
    "bxg_batch_destroy": (_int, [_vp]),
    "bxg_batch_last_error": (C.c_char_p, [_vp]),
    "bxg_batch_insert_f32": (_int, [_vp, _vp, _sz, _vp, _vp, _vp, _vp, _vp]),
    "bxg_batch_stats": (_int, [_vp, _vp]),
    "bxg_batch_phase_ms": (_int, [_vp, _vp]),
    "bxg_server_config_default": (None, [_vp]),
    "bxg_server_create": (_int, [_vp, _vp, _sz, _vp]),
    "bxg_server_destroy": (_int, [_vp]),
    "bxg_server_last_error": (C.c_char_p, [_vp]),
    "bxg_server_insert": (_int, [_vp, C.c_uint32, _vp, _sz, _vp, _dbl, _int, _vp]),
    "bxg_server_query": (_int, [_vp, C.c_uint32, _vp, _sz, _int, _int, _vp]),
    "bxg_server_get_occupied": (_int, [_vp, C.c_uint32, _int, _vp]),
    "bxg_server_clear": (_int, [_vp, C.c_uint32, _int, _int, _vp]),
    "bxg_server_wait": (_int, [_vp, C.c_uint64, _dbl, _vp, _vp, _sz]),
    "bxg_server_drain": (_int, [_vp, _dbl]),
    "bxg_server_stats": (_int, [_vp, _vp]),
    "bxg_server_map": (_vp, [_vp, C.c_uint32]),
}

_lib = None


def library_path() -> Path:
    return Path(os.environ.get("BONXAI_GB300_LIB", str(_LIB_PATH)))


def load_library() -> C.CDLL:
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        path = library_path()
        if not path.exists():
            raise ImportError(f"{path} is missing: run `python -m bonxai_gb300.build` "
                              "(or __graft_entry__.build()) first; there is no CPU fallback")
        lib = C.CDLL(str(path))
        for name, (res, args) in _SIGS.items():
            f = getattr(lib, name)
            f.restype, f.argtypes = res, args
        _lib = lib
    return _lib


# ----------------------------------------------------------------------------
# array plumbing: numpy (host) or torch CUDA tensors (device)
# ----------------------------------------------------------------------------
def _is_torch(a) -> bool:
    return type(a).__module__.startswith("torch")


def _in(a, dtype, cols=None):
    """(pointer, keepalive, n_rows) for an input array."""
    if _is_torch(a):
        import torch
        tdt = {np.float32: torch.float32, np.float64: torch.float64, np.int32: torch.int32,
               np.uint8: torch.uint8, np.uint32: torch.int32, np.int64: torch.int64}[dtype]
        t = a.contiguous()
        if t.dtype != tdt:
            raise TypeError(f"expected {tdt}, got {t.dtype}")
        n = t.shape[0] if t.dim() else 1
        return C.c_void_p(t.data_ptr()), t, n
    arr = np.ascontiguousarray(a, dtype=dtype)
    if cols and (arr.ndim != 2 or arr.shape[1] != cols):
        arr = arr.reshape(-1, cols)
    # the address as a plain int: the c_void_p argtypes take it as is, and it
    # is cheaper than building a ctypes pointer object per call
    return arr.ctypes.data, arr, (arr.shape[0] if arr.ndim else 1)


def _ptr(arr):
    if arr is None:
        return None
    if _is_torch(arr):
        return arr.data_ptr()
    return arr.ctypes.data


class _Handle:
    _destroy = None

    def _check(self, st: int):
        if st != 0:
            msg = self.lib.bxg_last_error(self.h)
            raise BonxaiError(st, msg.decode() if msg else "")

    def close(self):
        if getattr(self, "_owner", None) is not None:  # a borrowed view
            self.h = None
            return
        if getattr(self, "h", None):
            getattr(self.lib, self._destroy)(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


_VALUE_BYTES = {np.dtype(np.float32): 4, np.dtype(np.int32): 4, np.dtype(np.uint32): 4,
                np.dtype(np.float64): 8, np.dtype(np.int64): 8, np.dtype(np.uint64): 8,
                np.dtype(np.int16): 2, np.dtype(np.uint16): 2, np.dtype(np.int8): 1,
                np.dtype(np.uint8): 1}


class VoxelGrid(_Handle):
    """VoxelGrid<T> (bonxai.hpp:114-333); dtype=None gives BinaryVoxelGrid."""
    _destroy = "bxg_grid_destroy"

    def __init__(self, voxel_size: float, inner_bits: int = 2, leaf_bits: int = 3,
                 dtype=np.float32, config: Config | None = None):
        self.lib = load_library()
        self.dtype = None if dtype is None else np.dtype(dtype)
        esz = 0 if dtype is None else _VALUE_BYTES[self.dtype]
        h = C.c_void_p()
        st = self.lib.bxg_grid_create(C.byref(h), float(voxel_size), int(inner_bits),
                                      int(leaf_bits), esz, C.byref(config) if config else None)
        if st:
            raise BonxaiError(st, (self.lib.bxg_last_error(None) or b"").decode())
        self.h = h
        self.voxel_size = float(voxel_size)

    def pos_to_coord(self, xyz):
        p, keep, n = _in(xyz, np.float64, 3)
        out = np.zeros((n, 3), np.int32)
        self._check(self.lib.bxg_grid_pos_to_coord(self.h, p, n, _ptr(out)))
        return out

    posToCoord = pos_to_coord

    def coord_to_pos(self, coords):
        """coordToPos (bonxai.hpp:412-417): the cell corner coord * voxel_size."""
        return np.asarray(coords, np.float64) * self.voxel_size

    def set_values(self, coords, values, return_was_on: bool = False):
        p, keep, n = _in(coords, np.int32, 3)
        v, keepv, _ = (None, None, 0) if self.dtype is None else _in(values, self.dtype)
        was = np.zeros(n, np.uint8) if return_was_on else None
        self._check(self.lib.bxg_grid_set_values(self.h, p, v, n, _ptr(was)))
        return was

    setValue = set_values

    def set_values_at_points(self, points, values):
        dt = np.float64 if (getattr(points, "dtype", None) == np.float64 or
                            str(getattr(points, "dtype", "")) == "torch.float64") else np.float32
        p, keep, n = _in(points, dt, 3)
        v, keepv, _ = (None, None, 0) if self.dtype is None else _in(values, self.dtype)
        f = (self.lib.bxg_grid_set_values_at_points_f64 if dt == np.float64 else
             self.lib.bxg_grid_set_values_at_points_f32)
        self._check(f(self.h, p, 0, n, v))

    def get_values(self, coords, create: bool = False):
        p, keep, n = _in(coords, np.int32, 3)
        vals = None if self.dtype is None else np.zeros(n, self.dtype)
        found = np.zeros(n, np.uint8)
        self._check(self.lib.bxg_grid_get_values(self.h, p, n, _ptr(vals), _ptr(found),
                                                 int(create)))
        return vals, found

    value = get_values

    def set_cells_on(self, coords, default=0):
        p, keep, n = _in(coords, np.int32, 3)
        d = None if self.dtype is None else np.array([default], self.dtype)
        was = np.zeros(n, np.uint8)
        self._check(self.lib.bxg_grid_set_cells_on(self.h, p, n, _ptr(d), _ptr(was)))
        return was

    def set_cells_off(self, coords):
        p, keep, n = _in(coords, np.int32, 3)
        was = np.zeros(n, np.uint8)
        self._check(self.lib.bxg_grid_set_cells_off(self.h, p, n, _ptr(was)))
        return was

    def store_if_on(self, coords, values):
        p, keep, n = _in(coords, np.int32, 3)
        v, keepv, _ = _in(values, self.dtype)
        self._check(self.lib.bxg_grid_store_if_on(self.h, p, v, n))

    def is_cell_on(self, coords):
        p, keep, n = _in(coords, np.int32, 3)
        out = np.zeros(n, np.uint8)
        self._check(self.lib.bxg_grid_is_cell_on(self.h, p, n, _ptr(out)))
        return out

    def active_cells_count(self) -> int:
        out = C.c_size_t()
        self._check(self.lib.bxg_grid_active_cells(self.h, C.byref(out)))
        return out.value

    activeCellsCount = active_cells_count

    def node_counts(self):
        r, l = C.c_size_t(), C.c_size_t()
        self._check(self.lib.bxg_grid_node_counts(self.h, C.byref(r), C.byref(l)))
        return r.value, l.value

    def mem_usage(self) -> int:
        out = C.c_size_t()
        self._check(self.lib.bxg_grid_mem_usage(self.h, C.byref(out)))
        return out.value

    def dump(self, sort: bool = True):
        """forEachCell as arrays: (coords int32 [n,3], values [n]) sorted by xyz."""
        n = self.active_cells_count()
        xyz = np.zeros((max(n, 1), 3), np.int32)
        vals = None if self.dtype is None else np.zeros(max(n, 1), self.dtype)
        got = C.c_size_t()
        self._check(self.lib.bxg_grid_dump(self.h, _ptr(xyz), _ptr(vals), n, C.byref(got)))
        xyz = xyz[:got.value]
        vals = None if vals is None else vals[:got.value]
        if sort:
            o = np.lexsort((xyz[:, 2], xyz[:, 1], xyz[:, 0]))
            xyz = xyz[o]
            vals = None if vals is None else vals[o]
        return xyz, vals

    def for_each_cell(self, func):
        xyz, vals = self.dump(sort=False)
        for k in range(len(xyz)):
            func(None if vals is None else vals[k], tuple(int(c) for c in xyz[k]))

    forEachCell = for_each_cell

    def clear(self, option: int = CLEAR_MEMORY):
        self._check(self.lib.bxg_grid_clear(self.h, int(option)))

    def release_unused_memory(self):
        self._check(self.lib.bxg_grid_release_unused(self.h))

    _TYPE_NAMES = {np.dtype(np.float32): "float", np.dtype(np.float64): "double",
                   np.dtype(np.int32): "int", np.dtype(np.uint32): "unsigned int",
                   np.dtype(np.int64): "long", np.dtype(np.uint64): "unsigned long",
                   np.dtype(np.int16): "short", np.dtype(np.uint16): "unsigned short",
                   np.dtype(np.int8): "signed char", np.dtype(np.uint8): "unsigned char"}

    def serialize(self, type_name: str | None = None) -> bytes:
        """Serialize in the reference's byte format (serialization.hpp:77-116)."""
        if type_name is None:
            type_name = "Bonxai::EmptyVoxel" if self.dtype is None else self._TYPE_NAMES[self.dtype]
        n = C.c_size_t()
        st = self.lib.bxg_grid_serialize(self.h, type_name.encode(), None, 0, C.byref(n))
        if st not in (0, 7):
            self._check(st)
        buf = C.create_string_buffer(n.value)
        self._check(self.lib.bxg_grid_serialize(self.h, type_name.encode(), buf, n.value,
                                                C.byref(n)))
        return buf.raw[:n.value]

    def deserialize(self, data: bytes):
        self._check(self.lib.bxg_grid_deserialize(self.h, data, len(data)))

    releaseUnusedMemory = release_unused_memory


class ProbabilisticMap(_Handle):
    """ProbabilisticMap (probabilistic_map.hpp:27-137) on one GPU."""
    _destroy = "bxg_pmap_destroy"

    def __init__(self, resolution: float, config: Config | None = None):
        self.lib = load_library()
        h = C.c_void_p()
        st = self.lib.bxg_pmap_create(C.byref(h), float(resolution),
                                      C.byref(config) if config else None)
        if st:
            raise BonxaiError(st, (self.lib.bxg_last_error(None) or b"").decode())
        self.h = h
        self.resolution = float(resolution)

    @property
    def options(self) -> np.ndarray:
        o = Options()
        self._check(self.lib.bxg_pmap_get_options(self.h, C.byref(o)))
        return np.array([o.prob_miss_log, o.prob_hit_log, o.clamp_min_log, o.clamp_max_log,
                         o.occupancy_threshold_log], np.int32)

    @options.setter
    def options(self, v):
        v = [int(x) for x in v]
        o = Options(*v)
        self._check(self.lib.bxg_pmap_set_options(self.h, C.byref(o)))

    @property
    def update_count(self) -> int:
        out = C.c_int()
        self._check(self.lib.bxg_pmap_update_count(self.h, C.byref(out)))
        return out.value

    @property
    def stream(self) -> int:
        return self.lib.bxg_pmap_stream(self.h) or 0

    def insert_point_cloud(self, points, origin, max_range: float, stride: int = 0) -> int:
        """insertPointCloud; returns V = points + cast ray cells."""
        if isinstance(points, np.ndarray):
            is64 = points.dtype == np.float64
        else:
            is64 = str(getattr(points, "dtype", "")) == "torch.float64"
        dt = np.float64 if is64 else np.float32
        p, keep, n = _in(points, dt, None if stride else 3)
        o = np.ascontiguousarray(np.asarray(origin, dt).reshape(3))
        v = C.c_uint64()
        f = (self.lib.bxg_pmap_insert_point_cloud_f64 if is64 else
             self.lib.bxg_pmap_insert_point_cloud_f32)
        if stride:
            n = n  # caller passes rows already
        self._check(f(self.h, p, int(stride), n, _ptr(o), float(max_range), C.byref(v)))
        return v.value

    insertPointCloud = insert_point_cloud

    def insert_sensor_cloud(self, points, sensor_to_world, max_range: float) -> int:
        """The ROS node's ingest fused into one scan (bonxai_server.cpp:140-182):
        sensor-frame float points, a 3x4 or 4x4 sensor-to-world transform;
        non-finite points are dropped, the origin is the translation, and a
        negative max_range means no limit. Returns V."""
        p, keep, n = _in(points, np.float32, 3)
        m = np.ascontiguousarray(np.asarray(sensor_to_world, np.float32)[:3, :4].reshape(12))
        v = C.c_uint64()
        self._check(self.lib.bxg_pmap_insert_sensor_cloud_f32(self.h, p, 0, n, _ptr(m),
                                                              float(max_range), C.byref(v)))
        return v.value

    def insert_point_cloud_async(self, points, origin, max_range: float):
        p, keep, n = _in(points, np.float32, 3)
        o = np.ascontiguousarray(np.asarray(origin, np.float32).reshape(3))
        self._check(self.lib.bxg_pmap_insert_point_cloud_f32_async(self.h, p, 0, n, _ptr(o),
                                                                   float(max_range)))
        self._keep = (keep, o)

    def add_hit_points(self, points):
        p, keep, n = _in(points, np.float64, 3)
        self._check(self.lib.bxg_pmap_add_hit_points(self.h, p, n))

    def add_miss_points(self, points):
        p, keep, n = _in(points, np.float64, 3)
        self._check(self.lib.bxg_pmap_add_miss_points(self.h, p, n))

    def add_points(self, points, kinds):
        """Ordered mix of addHitPoint (kind 0) and addMissPoint (kind 1) calls."""
        p, keep, n = _in(points, np.float64, 3)
        k, keepk, _ = _in(kinds, np.uint8)
        self._check(self.lib.bxg_pmap_add_points(self.h, p, k, n))

    addHitPoint = add_hit_points
    addMissPoint = add_miss_points

    def update_free_cells(self, origin) -> int:
        o = np.ascontiguousarray(np.asarray(origin, np.float64).reshape(3))
        v = C.c_uint64()
        self._check(self.lib.bxg_pmap_update_free_cells(self.h, _ptr(o), C.byref(v)))
        return v.value

    updateFreeCells = update_free_cells

    def _query(self, fn, coords, out=None):
        p, keep, n = _in(coords, np.int32, 3)
        if out is None:
            out = np.zeros(n, np.uint8)
        self._check(fn(self.h, p, n, _ptr(out)))
        return out

    def is_occupied(self, coords, out=None):
        return self._query(self.lib.bxg_pmap_is_occupied, coords, out)

    def is_unknown(self, coords, out=None):
        return self._query(self.lib.bxg_pmap_is_unknown, coords, out)

    def is_free(self, coords, out=None):
        return self._query(self.lib.bxg_pmap_is_free, coords, out)

    isOccupied, isUnknown, isFree = is_occupied, is_unknown, is_free

    def last_query_ms(self) -> float:
        """Device time of the last lookup kernel (maps created with FLAG_TIMING)."""
        out = C.c_float()
        self._check(self.lib.bxg_pmap_last_query_ms(self.h, C.byref(out)))
        return out.value

    def active_cells_count(self) -> int:
        out = C.c_size_t()
        self._check(self.lib.bxg_pmap_active_cells(self.h, C.byref(out)))
        return out.value

    def node_counts(self):
        r, l = C.c_size_t(), C.c_size_t()
        self._check(self.lib.bxg_pmap_node_counts(self.h, C.byref(r), C.byref(l)))
        return r.value, l.value

    def mem_usage(self) -> int:
        out = C.c_size_t()
        self._check(self.lib.bxg_pmap_mem_usage(self.h, C.byref(out)))
        return out.value

    def _coords(self, fn, sort=True):
        got = C.c_size_t()
        st = fn(self.h, None, 0, C.byref(got))
        if st not in (0, 7):
            self._check(st)
        n = got.value
        out = np.zeros((max(n, 1), 3), np.int32)
        self._check(fn(self.h, _ptr(out), n, C.byref(got)))
        out = out[:got.value]
        if sort:
            out = out[np.lexsort((out[:, 2], out[:, 1], out[:, 0]))]
        return out

    def get_occupied_voxels(self, sort: bool = True):
        return self._coords(self.lib.bxg_pmap_get_occupied, sort)

    def get_free_voxels(self, sort: bool = True):
        return self._coords(self.lib.bxg_pmap_get_free, sort)

    getOccupiedVoxels, getFreeVoxels = get_occupied_voxels, get_free_voxels

    def export_occupied(self, min_z=-np.inf, max_z=np.inf, out=None, sort: bool = True):
        """Occupied corner positions (float xyz) with min_z <= z <= max_z, as
        the ROS node publishes them. With out = a CUDA float32 tensor [cap, 3]
        the positions stay on the GPU and the count is returned instead."""
        got = C.c_size_t()
        if out is not None:
            st = self.lib.bxg_pmap_export_occupied_f32(self.h, _ptr(out), out.shape[0],
                                                       C.byref(got), float(min_z), float(max_z))
            if st not in (0, 7):
                self._check(st)
            return got.value
        st = self.lib.bxg_pmap_export_occupied_f32(self.h, None, 0, C.byref(got),
                                                   float(min_z), float(max_z))
        if st not in (0, 7):
            self._check(st)
        n = got.value
        pts = np.zeros((max(n, 1), 3), np.float32)
        self._check(self.lib.bxg_pmap_export_occupied_f32(self.h, _ptr(pts), n, C.byref(got),
                                                          float(min_z), float(max_z)))
        pts = pts[:got.value]
        if sort:
            pts = pts[np.lexsort((pts[:, 2], pts[:, 1], pts[:, 0]))]
        return pts

    def dump(self, sort: bool = True):
        """Every cell as (coords [n,3] int32, packed CellT words [n] int32)."""
        n = self.active_cells_count()
        xyz = np.zeros((max(n, 1), 3), np.int32)
        cells = np.zeros(max(n, 1), np.int32)
        got = C.c_size_t()
        self._check(self.lib.bxg_pmap_dump(self.h, _ptr(xyz), _ptr(cells), n, C.byref(got)))
        xyz, cells = xyz[:got.value], cells[:got.value]
        if sort:
            o = np.lexsort((xyz[:, 2], xyz[:, 1], xyz[:, 0]))
            xyz, cells = xyz[o], cells[o]
        return xyz, cells

    def clear(self):
        self._check(self.lib.bxg_pmap_clear(self.h))

    def grid(self) -> VoxelGrid:
        """grid() (probabilistic_map.hpp:70-72): the map's own VoxelGrid<CellT>,
        its values the packed int32 CellT word. A borrowed view: valid while
        this map lives; closing it leaves the map alone."""
        g = VoxelGrid.__new__(VoxelGrid)
        g.lib = self.lib
        g.dtype = np.dtype(np.int32)
        g.voxel_size = self.resolution
        g._owner = self
        g.h = self.lib.bxg_pmap_grid(self.h)
        return g

    def synchronize(self):
        self._check(self.lib.bxg_pmap_synchronize(self.h))

    def last_stats(self) -> dict:
        out = (C.c_uint64 * 8)()
        self._check(self.lib.bxg_pmap_last_stats(self.h, out))
        keys = ["points", "cast_rays", "ray_cells_visited", "ray_cells_updated", "leaves",
                "launches"]
        return {k: int(out[i]) for i, k in enumerate(keys)}

    def kernel_times(self) -> list[float]:
        out = (C.c_float * 4)()
        self._check(self.lib.bxg_pmap_kernel_times(self.h, out))
        return [float(x) for x in out]


class Batch(_Handle):
    """One insertPointCloud per map for many maps per call, in one persistent
    graph-replayed launch (bxg_batch_insert_f32)."""
    _destroy = "bxg_batch_destroy"

    def __init__(self, config: Config | None = None):
        self.lib = load_library()
        h = C.c_void_p()
        st = self.lib.bxg_batch_create(C.byref(h), C.byref(config) if config else None)
        if st:
            raise BonxaiError(st, "bxg_batch_create")
        self.h = h

    def _check(self, st: int):
        if st != 0:
            msg = self.lib.bxg_batch_last_error(self.h)
            raise BonxaiError(st, msg.decode() if msg else "")

    def insert(self, maps, points, offsets, origins, max_ranges):
        """points: packed float32 [N,3] (numpy or CUDA tensor) holding every
        scan back to back; offsets: N_scans+1 int64; returns ray cells per scan."""
        n = len(maps)
        handles = (C.c_void_p * n)(*[m.h.value for m in maps])
        p, keep, _ = _in(points, np.float32, 3)
        off = np.ascontiguousarray(offsets, np.uint64)
        org = np.ascontiguousarray(np.asarray(origins, np.float32).reshape(n, 3))
        mr = np.ascontiguousarray(np.broadcast_to(np.asarray(max_ranges, np.float64), (n,)))
        out = np.zeros(n, np.uint64)
        self._check(self.lib.bxg_batch_insert_f32(self.h, handles, n, p, _ptr(off), _ptr(org),
                                                  _ptr(mr), _ptr(out)))
        return out

    def stats(self) -> dict:
        out = (C.c_double * 8)()
        self._check(self.lib.bxg_batch_stats(self.h, out))
        ph = (C.c_double * 6)()
        self._check(self.lib.bxg_batch_phase_ms(self.h, ph))
        return {"device_ms": out[0], "graph": bool(out[1]), "retried_maps": int(out[2]),
                "ticks": int(out[3]), "grid": int(out[4]), "launches": int(out[5]),
                "phase_ms": {"clear": ph[0], "endpoints": ph[1], "winners": ph[2],
                             "prefix": ph[3], "rays": ph[4], "rays_mark": ph[5]}}


class ServerConfig(C.Structure):
    _fields_ = [("pool_budget_bytes", C.c_size_t), ("max_scans_per_tick", C.c_uint32),
                ("max_points_per_tick", C.c_uint64), ("max_lookups_per_tick", C.c_uint64),
                ("device", C.c_int), ("rays_per_warp", C.c_uint32), ("ray_unroll", C.c_uint32),
                ("flags", C.c_uint32), ("initial_leaves", C.c_uint32),
                ("admission_timeout_s", C.c_double)]

    def __init__(self, **kw):
        super().__init__()
        self.device = -1
        for k, v in kw.items():
            setattr(self, k, v)


class ServerResult(C.Structure):
    _fields_ = [("status", C.c_int), ("kind", C.c_int), ("map", C.c_uint32),
                ("ray_cells", C.c_uint64), ("n_out", C.c_size_t), ("latency_ms", C.c_double),
                ("queue_ms", C.c_double), ("tick", C.c_uint64)]


class Server(_Handle):
    """Continuous-batching server over one persistent map per client
    (bxg_server_*). Requests on one map run in submission order."""
    _destroy = "bxg_server_destroy"

    def __init__(self, resolutions, config: ServerConfig | None = None):
        self.lib = load_library()
        res = np.ascontiguousarray(resolutions, np.float64)
        h = C.c_void_p()
        st = self.lib.bxg_server_create(C.byref(h), _ptr(res), len(res),
                                        C.byref(config) if config else None)
        if st:
            raise BonxaiError(st, "bxg_server_create")
        self.h = h
        self.n_maps = len(res)

    def _check(self, st: int):
        if st != 0:
            msg = self.lib.bxg_server_last_error(self.h)
            raise BonxaiError(st, msg.decode() if msg else "")

    def insert(self, map_id, points, origin, max_range, discard=False) -> int:
        p, keep, n = _in(points, np.float32, 3)
        o = np.ascontiguousarray(np.asarray(origin, np.float32).reshape(3))
        t = C.c_uint64()
        self._check(self.lib.bxg_server_insert(self.h, int(map_id), p, n, _ptr(o),
                                               float(max_range), int(discard), C.byref(t)))
        return t.value

    def query(self, map_id, coords, mode=0, discard=False) -> int:
        p, keep, n = _in(coords, np.int32, 3)
        t = C.c_uint64()
        self._check(self.lib.bxg_server_query(self.h, int(map_id), p, n, int(mode), int(discard),
                                              C.byref(t)))
        return t.value

    def get_occupied(self, map_id, discard=False) -> int:
        t = C.c_uint64()
        self._check(self.lib.bxg_server_get_occupied(self.h, int(map_id), int(discard),
                                                     C.byref(t)))
        return t.value

    def clear(self, map_id, release_memory=True, discard=False) -> int:
        """clear(CLEAR_MEMORY) of one client's map, in its request order; with
        release_memory its pools shrink back, freeing budget for waiting inserts."""
        t = C.c_uint64()
        self._check(self.lib.bxg_server_clear(self.h, int(map_id), int(release_memory),
                                              int(discard), C.byref(t)))
        return t.value

    def wait_query(self, ticket, n, timeout=120.0):
        res = ServerResult()
        out = np.zeros(max(n, 1), np.uint8)
        self._check(self.lib.bxg_server_wait(self.h, int(ticket), float(timeout), C.byref(res),
                                             _ptr(out), n))
        return self._res(res), out[:res.n_out]

    def wait_insert(self, ticket, timeout=120.0):
        res = ServerResult()
        self._check(self.lib.bxg_server_wait(self.h, int(ticket), float(timeout), C.byref(res),
                                             None, 0))
        return self._res(res)

    def wait_occupied(self, ticket, timeout=120.0):
        res = ServerResult()
        self._check(self.lib.bxg_server_wait(self.h, int(ticket), float(timeout), C.byref(res),
                                             None, 0))
        n = res.n_out
        out = np.zeros((max(n, 1), 3), np.int32)
        self._check(self.lib.bxg_server_wait(self.h, int(ticket), float(timeout), C.byref(res),
                                             _ptr(out), n))
        o = out[:n]
        return self._res(res), o[np.lexsort((o[:, 2], o[:, 1], o[:, 0]))]

    @staticmethod
    def _res(r):
        return {"status": r.status, "kind": r.kind, "map": r.map, "ray_cells": int(r.ray_cells),
                "n_out": int(r.n_out), "latency_ms": r.latency_ms, "queue_ms": r.queue_ms,
                "tick": int(r.tick)}

    def drain(self, timeout=600.0):
        self._check(self.lib.bxg_server_drain(self.h, float(timeout)))

    def stats(self) -> dict:
        out = (C.c_double * 20)()
        self._check(self.lib.bxg_server_stats(self.h, out))
        keys = ["completed", "inserts", "lookups", "occupied", "ticks", "p50_ms", "p99_ms",
                "insert_p50_ms", "insert_p99_ms", "lookup_p50_ms", "lookup_p99_ms", "ray_cells",
                "lookup_coords", "rejected", "busy_s", "span_s", "occupied_p50_ms",
                "occupied_p99_ms", "pool_bytes", "deferred"]
        return {k: out[i] for i, k in enumerate(keys)}

    def map_dump(self, map_id):
        """Cells of one client's map (after drain), sorted."""
        h = self.lib.bxg_server_map(self.h, int(map_id))
        m = ProbabilisticMap.__new__(ProbabilisticMap)
        m.lib, m.h = self.lib, C.c_void_p(h)
        try:
            return m.dump()
        finally:
            m.h = None  # borrowed: the server owns it


def compute_rays(origins, ends):
    """ComputeRay for each (origin, end) pair on the GPU: list of [len,3] arrays."""
    lib = load_library()
    o, ko, n = _in(origins, np.int32, 3)
    e, ke, _ = _in(ends, np.int32, 3)
    lens = np.zeros(n, np.uint32)
    st = lib.bxg_compute_rays(o, e, n, _ptr(lens), None, None)
    if st:
        raise BonxaiError(st, "compute_rays")
    off = np.zeros(n, np.uint64)
    off[1:] = np.cumsum(lens[:-1].astype(np.uint64))
    total = int(lens.astype(np.uint64).sum())
    cells = np.zeros((max(total, 1), 3), np.int32)
    st = lib.bxg_compute_rays(o, e, n, _ptr(lens), _ptr(off), _ptr(cells))
    if st:
        raise BonxaiError(st, "compute_rays")
    return [cells[int(off[i]):int(off[i]) + int(lens[i])] for i in range(n)]
