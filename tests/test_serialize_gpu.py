"""Serialization of the device pools in the reference's byte format
(serialization.hpp:77-199): the GPU's stream holds the reference's content
(roots may come in another order, which the format allows), and the
reference's stream deserializes into the same GPU grid."""
import numpy as np
import pytest

import serial_format as sf
from conftest import golden

pytestmark = pytest.mark.gpu


def test_grid_stream_matches_reference(gpu):
    g = golden("serialized.npz")
    ref_bytes = g["grid_f32"].tobytes()
    G = gpu.VoxelGrid(0.05)
    G.set_values(g["grid_coords"], g["grid_values"])
    mine = G.serialize()
    h1, x1, v1 = sf.parse(mine, 4)
    h0, x0, v0 = sf.parse(ref_bytes, 4)
    assert mine.split(b"\n", 1)[0] == ref_bytes.split(b"\n", 1)[0]
    assert len(mine) == len(ref_bytes)
    assert np.array_equal(x1, x0) and np.array_equal(v1, v0)
    # the reference's stream, read back into a fresh GPU grid
    H = gpu.VoxelGrid(0.05)
    H.deserialize(ref_bytes)
    a, av = H.dump()
    b, bv = G.dump()
    assert np.array_equal(a, b) and np.array_equal(av.view(np.uint32), bv.view(np.uint32))
    # and the GPU's own stream round-trips
    K = gpu.VoxelGrid(0.05)
    K.deserialize(mine)
    c, cv = K.dump()
    assert np.array_equal(c, b) and np.array_equal(cv.view(np.uint32), bv.view(np.uint32))


def test_pmap_stream_matches_reference(gpu):
    import ctypes as C
    g = golden("serialized.npz")
    lid = golden("pmap_lidar.npz")
    m = gpu.ProbabilisticMap(0.1)
    for k in range(3):
        m.insert_point_cloud(lid["points"][k], lid["origins"][k], float(lid["max_range"]))
    lib = gpu.load_library()
    view = lib.bxg_pmap_grid(m.h)
    name = b"Bonxai::ProbabilisticMap::CellT"
    n = C.c_size_t()
    lib.bxg_grid_serialize(view, name, None, 0, C.byref(n))
    buf = C.create_string_buffer(n.value)
    assert lib.bxg_grid_serialize(view, name, buf, n.value, C.byref(n)) == 0
    mine = buf.raw[:n.value]
    ref_bytes = g["pmap"].tobytes()
    h1, x1, v1 = sf.parse(mine, 4)
    h0, x0, v0 = sf.parse(ref_bytes, 4)
    assert h1 == h0 and len(mine) == len(ref_bytes)
    assert np.array_equal(x1, x0) and np.array_equal(v1, v0)
    # a checkpoint restored into a fresh map continues bit-exactly
    m2 = gpu.ProbabilisticMap(0.1)
    assert lib.bxg_grid_deserialize(lib.bxg_pmap_grid(m2.h), ref_bytes, len(ref_bytes)) == 0
    a, ac = m2.dump()
    b, bc = m.dump()
    assert np.array_equal(a, b) and np.array_equal(ac, bc)


def test_empty_and_binary_grids(gpu):
    E = gpu.VoxelGrid(0.1)
    s = E.serialize()
    assert s == b"Bonxai::VoxelGrid<float,2,3>(0.100000)\n" + b"\x00" * 4
    B = gpu.VoxelGrid(0.1, dtype=None)
    coords = np.random.default_rng(0).integers(-30, 30, (500, 3)).astype(np.int32)
    B.set_cells_on(coords)
    s = B.serialize()
    h, x, _ = sf.parse(s, 0)
    assert np.array_equal(x, B.dump()[0])
    B2 = gpu.VoxelGrid(0.1, dtype=None)
    B2.deserialize(s)
    assert np.array_equal(B2.dump()[0], x)
