"""Failure detection without a GPU fault: every device-side wait is bounded.
A leaf marked as being created by a creator that never publishes (a flag
nothing sets, planted by the bxg_debug_hold_leaf test hook) makes the scan's
waits run out; the call returns BXG_ERR_WAIT_TIMEOUT within seconds, and the
map stays usable after clear()."""
import time

import numpy as np
import pytest

from bonxai_gb300 import synth

pytestmark = pytest.mark.gpu


def test_wait_on_a_leaf_that_never_appears_times_out(gpu, port):
    scene = synth.LidarScene()
    pts, org = scene.scan(0, n_points=4096)
    m = gpu.ProbabilisticMap(0.1)
    lib = gpu.load_library()
    # every ray starts in the origin cell, so every ray needs this leaf
    oc = np.ascontiguousarray(np.floor(org.astype(np.float64) / 0.1).astype(np.int32))
    assert lib.bxg_debug_hold_leaf(lib.bxg_pmap_grid(m.h), oc.ctypes.data) == 0
    t0 = time.time()
    with pytest.raises(gpu.BonxaiError) as ei:
        m.insert_point_cloud(pts, org, 30.0)
    assert ei.value.status == 4  # BXG_ERR_WAIT_TIMEOUT
    assert time.time() - t0 < 60
    # the context and the handle stay usable; clear() releases the mark
    m.clear()
    o = port.pmap(0.1)
    while o.update_count != m.update_count:
        o.update_free_cells(np.zeros(3))
    assert m.insert_point_cloud(pts, org, 30.0) == o.insert(pts, org, 30.0)
    gx, gc = m.dump()
    ox, occ = o.dump()
    assert np.array_equal(gx, ox) and np.array_equal(gc, occ)


def test_hold_on_an_existing_leaf_is_refused(gpu):
    m = gpu.ProbabilisticMap(0.1)
    pts, org = synth.LidarScene().scan(0, n_points=2048)
    m.insert_point_cloud(pts, org, 30.0)
    lib = gpu.load_library()
    oc = np.ascontiguousarray(np.floor(org.astype(np.float64) / 0.1).astype(np.int32))
    assert lib.bxg_debug_hold_leaf(lib.bxg_pmap_grid(m.h), oc.ctypes.data) == 1
