"""The setValue batch that allocates no GPU memory.

Some callers of this library must not allocate device memory while they run:
a real-time mapping or control thread, where cudaMalloc can block for
milliseconds and cudaFree synchronises the whole device, or a process that
reserves its device memory up front. bxg_grid_set_values_noalloc serves them
with a fixed scratch array instead of the growable scratch of
bxg_grid_set_values. These tests call both through the C ABI on the same
device-resident inputs, twice in a row (so the second call runs on a scratch
array that still holds the first call's contents), and require identical grids.

This file is collected last so that a run stopping at the first failure has
already run every other test; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _noalloc(lib, grid, d_xyz, d_vals):
    return lib.bxg_grid_set_values_noalloc(grid.h, C.c_void_p(d_xyz.data_ptr()),
                                           C.c_void_p(d_vals.data_ptr()), d_xyz.shape[0])


def _batch(rng, n):
    coords = rng.integers(-120, 120, (n, 3)).astype(np.int32)
    coords[::7] = coords[1::7][: len(coords[::7])]  # repeated cells: last writer wins
    vals = rng.random(n).astype(np.float32)
    return coords, vals


def test_noalloc_matches_set_values_on_two_calls(gpu, port):
    lib = gpu.load_library()
    rng = np.random.default_rng(2024)
    cfg = gpu.Config(initial_leaves=1 << 15, initial_inners=1 << 10)
    ref = gpu.VoxelGrid(0.05, dtype=np.float32, config=cfg)
    cand = gpu.VoxelGrid(0.05, dtype=np.float32, config=cfg)
    og = port.grid(0.05)  # the CPU oracle, setValue in input order
    for _ in range(2):
        coords, vals = _batch(rng, 100_000)
        d_xyz = torch.from_numpy(coords).cuda()
        d_vals = torch.from_numpy(vals).cuda()
        assert lib.bxg_grid_set_values(ref.h, C.c_void_p(d_xyz.data_ptr()),
                                       C.c_void_p(d_vals.data_ptr()), len(coords), None) == 0
        st = _noalloc(lib, cand, d_xyz, d_vals)
        assert st == 0, lib.bxg_last_error(cand.h)
        og.set_values(coords, vals)
        a, av = ref.dump()
        b, bv = cand.dump()
        o, ov = og.dump()
        # bit-exact, the tolerance of every parity test here
        assert np.array_equal(a, b) and np.array_equal(b, o)
        assert np.array_equal(av.view(np.uint32), bv.view(np.uint32))
        assert np.array_equal(bv.view(np.uint32), ov.view(np.uint32))


def test_noalloc_full_pool_reports_and_keeps_capacity(gpu, port):
    """A batch needing more leaves than the pool holds: OUT_OF_POOL, no pool
    growth, and the same batch through bxg_grid_set_values then gives the
    oracle's grid (a failed call may have written part of the batch)."""
    lib = gpu.load_library()
    rng = np.random.default_rng(7)
    g = gpu.VoxelGrid(0.05, dtype=np.float32,
                      config=gpu.Config(initial_leaves=64, initial_inners=256, hash_buckets=4096))
    # 64 roots (fit the inner pool and the hash), ~3400 leaves (do not fit 64 slots)
    coords = rng.integers(-60, 60, (20_000, 3)).astype(np.int32)
    vals = rng.random(len(coords)).astype(np.float32)
    d_xyz = torch.from_numpy(coords).cuda()
    d_vals = torch.from_numpy(vals).cuda()
    mem0 = g.mem_usage()
    st = _noalloc(lib, g, d_xyz, d_vals)
    assert st == 2, (st, lib.bxg_last_error(g.h))  # BXG_ERR_OUT_OF_POOL
    assert g.mem_usage() == mem0
    assert lib.bxg_grid_set_values(g.h, C.c_void_p(d_xyz.data_ptr()),
                                   C.c_void_p(d_vals.data_ptr()), len(coords), None) == 0
    og = port.grid(0.05)
    og.set_values(coords, vals)
    a, av = g.dump()
    o, ov = og.dump()
    assert np.array_equal(a, o) and np.array_equal(av.view(np.uint32), ov.view(np.uint32))


def test_noalloc_rejects_other_gpu_memory(gpu):
    if torch.cuda.device_count() < 2:
        pytest.skip("needs a second GPU")
    lib = gpu.load_library()
    g = gpu.VoxelGrid(0.05, dtype=np.float32)
    x = torch.zeros((10, 3), dtype=torch.int32, device="cuda:1")
    v = torch.zeros(10, dtype=torch.float32, device="cuda:1")
    assert _noalloc(lib, g, x, v) == 1
    assert b"grid's device" in lib.bxg_last_error(g.h)
    assert g.active_cells_count() == 0


def test_noalloc_rejects_oversized_and_host_inputs(gpu):
    lib = gpu.load_library()
    g = gpu.VoxelGrid(0.05, dtype=np.float32)
    big = torch.zeros((131073, 3), dtype=torch.int32, device="cuda")
    bigv = torch.zeros(131073, dtype=torch.float32, device="cuda")
    assert _noalloc(lib, g, big, bigv) == 1
    assert b"131072" in lib.bxg_last_error(g.h)
    host_xyz = np.zeros((10, 3), np.int32)
    host_val = np.zeros(10, np.float32)
    st = lib.bxg_grid_set_values_noalloc(g.h, host_xyz.ctypes.data_as(C.c_void_p),
                                         host_val.ctypes.data_as(C.c_void_p), 10)
    assert st == 1 and b"device" in lib.bxg_last_error(g.h)
    assert g.active_cells_count() == 0
