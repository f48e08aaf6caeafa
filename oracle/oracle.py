"""ctypes front end of the CPU oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline legs import
this module; the shipped library never does.

Two libraries implement the C API of ``oracle/oracle_api.h``:

* ``port()`` -- this project's restatement of the reference algorithm
  (``oracle/bonxai_oracle.cpp``), built by :func:`build_port` wherever g++ exists.
* ``ref()`` -- the reference's own code compiled unmodified
  (``oracle/build_ref.sh``); present only where the reference sources are
  mounted, else ``None``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_SO = HERE / "_build" / "liboracle_port.so"
REF_SO = HERE / "_ref" / "liboracle_ref.so"

ORC_F32, ORC_I32, ORC_U32, ORC_F64, ORC_I64 = range(5)
_NP_OF = {ORC_F32: np.float32, ORC_I32: np.int32, ORC_U32: np.uint32,
          ORC_F64: np.float64, ORC_I64: np.int64}

_vp, _sz, _u64, _dbl, _int = C.c_void_p, C.c_size_t, C.c_uint64, C.c_double, C.c_int


def build_port(force: bool = False) -> Path:
    """Compile the restatement with the flags the reference needs for fp64 parity
    (-O3 -ffp-contract=off, so no multiply-add is fused)."""
    src = HERE / "bonxai_oracle.cpp"
    if (not force and PORT_SO.exists()
            and PORT_SO.stat().st_mtime >= max(src.stat().st_mtime,
                                                (HERE / "oracle_api.h").stat().st_mtime)):
        return PORT_SO
    PORT_SO.parent.mkdir(parents=True, exist_ok=True)
    tmp = PORT_SO.with_suffix(".so.tmp%d" % os.getpid())
    subprocess.check_call(["g++", "-std=c++17", "-O3", "-ffp-contract=off", "-fPIC",
                           "-shared", "-I", str(HERE), str(src), "-o", str(tmp)])
    os.replace(tmp, PORT_SO)
    return PORT_SO


def build_ref(ref_root: str | None = None) -> Path | None:
    """Build oracle/_ref with the recipe oracle/build_ref.sh. The reference root
    is the argument, else $BONXAI_REFERENCE, else the recipe's own default; the
    recipe skips the build (exit 0) where the sources are not mounted."""
    script = HERE / "build_ref.sh"
    cmd = ["bash", str(script)]
    root = ref_root or os.environ.get("BONXAI_REFERENCE")
    if root:
        cmd.append(root)
    subprocess.check_call(cmd)
    return REF_SO if REF_SO.exists() else None


def _ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(_vp)


class OracleLib:
    def __init__(self, path: Path):
        self.path = Path(path)
        L = self.lib = C.CDLL(str(path))
        sig = {
            "orc_pmap_create": (_vp, [_dbl]),
            "orc_pmap_destroy": (None, [_vp]),
            "orc_pmap_get_options": (None, [_vp, _vp]),
            "orc_pmap_set_options": (None, [_vp, _vp]),
            "orc_pmap_update_count": (_int, [_vp]),
            "orc_pmap_insert_f32": (_u64, [_vp, _vp, _sz, _vp, _dbl]),
            "orc_pmap_insert_f64": (_u64, [_vp, _vp, _sz, _vp, _dbl]),
            "orc_pmap_add_hit": (None, [_vp, _vp, _sz]),
            "orc_pmap_add_miss": (None, [_vp, _vp, _sz]),
            "orc_pmap_update_free_cells": (_u64, [_vp, _vp]),
            "orc_pmap_cell_count": (_sz, [_vp]),
            "orc_pmap_dump": (_sz, [_vp, _vp, _vp, _sz]),
            "orc_pmap_query": (None, [_vp, _vp, _sz, _vp, _vp, _vp]),
            "orc_pmap_get_occupied": (_sz, [_vp, _vp, _sz]),
            "orc_pmap_get_free": (_sz, [_vp, _vp, _sz]),
            "orc_grid_create": (_vp, [_dbl, _int, _int, _int]),
            "orc_grid_destroy": (None, [_vp]),
            "orc_grid_pos_to_coord": (None, [_vp, _vp, _sz, _vp]),
            "orc_grid_set_values": (None, [_vp, _vp, _vp, _sz, _vp]),
            "orc_grid_get_values": (None, [_vp, _vp, _sz, _vp, _vp, _int]),
            "orc_grid_set_cells_on": (None, [_vp, _vp, _sz, _vp, _vp]),
            "orc_grid_set_cells_off": (None, [_vp, _vp, _sz, _vp]),
            "orc_grid_is_cell_on": (None, [_vp, _vp, _sz, _vp]),
            "orc_grid_active_cells": (_sz, [_vp]),
            "orc_grid_leaf_count": (_sz, [_vp]),
            "orc_grid_root_count": (_sz, [_vp]),
            "orc_grid_dump": (_sz, [_vp, _vp, _vp, _sz]),
            "orc_grid_clear": (None, [_vp, _int]),
            "orc_grid_release_unused": (None, [_vp]),
            "orc_compute_ray": (_sz, [_vp, _vp, _vp, _sz]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype, f.argtypes = res, args
        if hasattr(L, "orc_pmap_export_occupied_f32"):
            f = L.orc_pmap_export_occupied_f32
            f.restype, f.argtypes = _sz, [_vp, _dbl, _dbl, _vp, _sz]
        if hasattr(L, "orc_sensor_to_world_f32"):
            f = L.orc_sensor_to_world_f32
            f.restype, f.argtypes = _sz, [_vp, _vp, _sz, _vp]
        if hasattr(L, "orc_ref_insert_point_cloud_f32"):
            f = L.orc_ref_insert_point_cloud_f32
            f.restype, f.argtypes = None, [_vp, _vp, _sz, _vp, _dbl]
        for name in ("orc_ref_grid_serialize", "orc_ref_pmap_serialize"):
            if hasattr(L, name):
                f = getattr(L, name)
                f.restype, f.argtypes = _sz, [_vp, _vp, _sz]

    # ------------------------------------------------------------------ rays
    def compute_ray(self, o, e) -> np.ndarray:
        o = np.ascontiguousarray(o, np.int32)
        e = np.ascontiguousarray(e, np.int32)
        n = self.lib.orc_compute_ray(_ptr(o), _ptr(e), None, 0)
        out = np.zeros((n, 3), np.int32)
        self.lib.orc_compute_ray(_ptr(o), _ptr(e), _ptr(out), n)
        return out

    def sensor_to_world(self, m12, xyz) -> np.ndarray:
        """The ROS node's ingest restated: finite points, transformed in float."""
        m = np.ascontiguousarray(m12, np.float32).reshape(12)
        p = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
        out = np.zeros_like(p)
        k = self.lib.orc_sensor_to_world_f32(_ptr(m), _ptr(p), len(p), _ptr(out))
        return out[:k]

    def pmap(self, resolution: float) -> "OraclePMap":
        return OraclePMap(self, resolution)

    def grid(self, voxel_size: float, inner_bits=2, leaf_bits=3, dtype=ORC_F32):
        return OracleGrid(self, voxel_size, inner_bits, leaf_bits, dtype)


class OraclePMap:
    def __init__(self, L: OracleLib, resolution: float):
        self.L, self.lib = L, L.lib
        self.h = self.lib.orc_pmap_create(float(resolution))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_pmap_destroy(self.h)
            self.h = None

    @property
    def options(self) -> np.ndarray:
        o = np.zeros(5, np.int32)
        self.lib.orc_pmap_get_options(self.h, _ptr(o))
        return o

    @options.setter
    def options(self, o):
        o = np.ascontiguousarray(o, np.int32)
        self.lib.orc_pmap_set_options(self.h, _ptr(o))

    @property
    def update_count(self) -> int:
        return self.lib.orc_pmap_update_count(self.h)

    def insert(self, pts: np.ndarray, origin, max_range: float) -> int:
        if pts.dtype == np.float64:
            pts = np.ascontiguousarray(pts, np.float64)
            o = np.ascontiguousarray(origin, np.float64)
            return self.lib.orc_pmap_insert_f64(self.h, _ptr(pts), len(pts), _ptr(o),
                                                float(max_range))
        pts = np.ascontiguousarray(pts, np.float32)
        o = np.ascontiguousarray(origin, np.float32)
        return self.lib.orc_pmap_insert_f32(self.h, _ptr(pts), len(pts), _ptr(o),
                                            float(max_range))

    def insert_reference_path(self, pts: np.ndarray, origin, max_range: float) -> None:
        """The reference's own insertPointCloud (reference library only)."""
        pts = np.ascontiguousarray(pts, np.float32)
        o = np.ascontiguousarray(origin, np.float32)
        self.lib.orc_ref_insert_point_cloud_f32(self.h, _ptr(pts), len(pts), _ptr(o),
                                                float(max_range))

    def add_hit(self, pts):
        pts = np.ascontiguousarray(pts, np.float64).reshape(-1, 3)
        self.lib.orc_pmap_add_hit(self.h, _ptr(pts), len(pts))

    def add_miss(self, pts):
        pts = np.ascontiguousarray(pts, np.float64).reshape(-1, 3)
        self.lib.orc_pmap_add_miss(self.h, _ptr(pts), len(pts))

    def update_free_cells(self, origin) -> int:
        o = np.ascontiguousarray(origin, np.float64)
        return self.lib.orc_pmap_update_free_cells(self.h, _ptr(o))

    def cell_count(self) -> int:
        return self.lib.orc_pmap_cell_count(self.h)

    def dump(self):
        """All active cells as (xyz int32 [n,3], packed cell int32 [n]), sorted by xyz."""
        n = self.lib.orc_pmap_dump(self.h, None, None, 0)
        xyz = np.zeros((n, 3), np.int32)
        cells = np.zeros(n, np.int32)
        self.lib.orc_pmap_dump(self.h, _ptr(xyz), _ptr(cells), n)
        order = np.lexsort((xyz[:, 2], xyz[:, 1], xyz[:, 0]))
        return xyz[order], cells[order]

    def query(self, coords):
        c = np.ascontiguousarray(coords, np.int32).reshape(-1, 3)
        occ = np.zeros(len(c), np.uint8)
        unk = np.zeros(len(c), np.uint8)
        fre = np.zeros(len(c), np.uint8)
        self.lib.orc_pmap_query(self.h, _ptr(c), len(c), _ptr(occ), _ptr(unk), _ptr(fre))
        return occ, unk, fre

    def _coords(self, fn):
        n = fn(self.h, None, 0)
        out = np.zeros((n, 3), np.int32)
        fn(self.h, _ptr(out), n)
        order = np.lexsort((out[:, 2], out[:, 1], out[:, 0]))
        return out[order]

    def occupied(self):
        return self._coords(self.lib.orc_pmap_get_occupied)

    def export_occupied(self, min_z=-np.inf, max_z=np.inf) -> np.ndarray:
        """Occupied corner positions as float xyz in the z band, sorted."""
        fn = self.lib.orc_pmap_export_occupied_f32
        n = fn(self.h, float(min_z), float(max_z), None, 0)
        out = np.zeros((n, 3), np.float32)
        fn(self.h, float(min_z), float(max_z), _ptr(out), n)
        return out[np.lexsort((out[:, 2], out[:, 1], out[:, 0]))]

    def serialize_reference(self) -> bytes:
        """Bonxai::Serialize of the map's grid (reference library only)."""
        n = self.lib.orc_ref_pmap_serialize(self.h, None, 0)
        buf = C.create_string_buffer(n)
        self.lib.orc_ref_pmap_serialize(self.h, buf, n)
        return buf.raw[:n]

    def free(self):
        return self._coords(self.lib.orc_pmap_get_free)


class OracleGrid:
    def __init__(self, L: OracleLib, voxel_size, inner_bits, leaf_bits, dtype):
        self.L, self.lib, self.dtype = L, L.lib, dtype
        self.np_dtype = _NP_OF[dtype]
        self.h = self.lib.orc_grid_create(float(voxel_size), int(inner_bits), int(leaf_bits),
                                          int(dtype))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_grid_destroy(self.h)
            self.h = None

    def pos_to_coord(self, xyz):
        p = np.ascontiguousarray(xyz, np.float64).reshape(-1, 3)
        out = np.zeros((len(p), 3), np.int32)
        self.lib.orc_grid_pos_to_coord(self.h, _ptr(p), len(p), _ptr(out))
        return out

    def set_values(self, coords, values):
        c = np.ascontiguousarray(coords, np.int32).reshape(-1, 3)
        v = np.ascontiguousarray(values, self.np_dtype)
        was = np.zeros(len(c), np.uint8)
        self.lib.orc_grid_set_values(self.h, _ptr(c), _ptr(v), len(c), _ptr(was))
        return was

    def get_values(self, coords, create=False):
        c = np.ascontiguousarray(coords, np.int32).reshape(-1, 3)
        v = np.zeros(len(c), self.np_dtype)
        f = np.zeros(len(c), np.uint8)
        self.lib.orc_grid_get_values(self.h, _ptr(c), len(c), _ptr(v), _ptr(f), int(create))
        return v, f

    def set_cells_on(self, coords, default=0):
        c = np.ascontiguousarray(coords, np.int32).reshape(-1, 3)
        d = np.array([default], self.np_dtype)
        was = np.zeros(len(c), np.uint8)
        self.lib.orc_grid_set_cells_on(self.h, _ptr(c), len(c), _ptr(d), _ptr(was))
        return was

    def set_cells_off(self, coords):
        c = np.ascontiguousarray(coords, np.int32).reshape(-1, 3)
        was = np.zeros(len(c), np.uint8)
        self.lib.orc_grid_set_cells_off(self.h, _ptr(c), len(c), _ptr(was))
        return was

    def is_cell_on(self, coords):
        c = np.ascontiguousarray(coords, np.int32).reshape(-1, 3)
        out = np.zeros(len(c), np.uint8)
        self.lib.orc_grid_is_cell_on(self.h, _ptr(c), len(c), _ptr(out))
        return out

    def active_cells(self):
        return self.lib.orc_grid_active_cells(self.h)

    def leaf_count(self):
        return self.lib.orc_grid_leaf_count(self.h)

    def root_count(self):
        return self.lib.orc_grid_root_count(self.h)

    def dump(self):
        n = self.lib.orc_grid_dump(self.h, None, None, 0)
        xyz = np.zeros((n, 3), np.int32)
        v = np.zeros(n, self.np_dtype)
        self.lib.orc_grid_dump(self.h, _ptr(xyz), _ptr(v), n)
        order = np.lexsort((xyz[:, 2], xyz[:, 1], xyz[:, 0]))
        return xyz[order], v[order]

    def clear(self, option: int):
        self.lib.orc_grid_clear(self.h, int(option))

    def release_unused(self):
        self.lib.orc_grid_release_unused(self.h)

    def serialize_reference(self) -> bytes:
        """Bonxai::Serialize of this grid (reference library only)."""
        n = self.lib.orc_ref_grid_serialize(self.h, None, 0)
        buf = C.create_string_buffer(n)
        self.lib.orc_ref_grid_serialize(self.h, buf, n)
        return buf.raw[:n]


_port = None
_ref = None


def port() -> OracleLib:
    global _port
    if _port is None:
        _port = OracleLib(build_port())
    return _port


def ref() -> OracleLib | None:
    """The reference compiled unmodified, or None where it was not built."""
    global _ref
    if _ref is None and REF_SO.exists():
        try:
            _ref = OracleLib(REF_SO)
        except OSError:  # e.g. an x86 build carried to an Arm host
            _ref = None
    return _ref
