import numpy as np

from bonxai_gb300 import synth


def test_room_cloud_shape_and_seed():
    a = synth.room_cloud(5000, seed=1)
    b = synth.room_cloud(5000, seed=1)
    assert a.shape == (5000, 3) and a.dtype == np.float32
    assert np.array_equal(a, b)
    assert (a.min(0) > synth.ROOM_LO - 0.05).all() and (a.max(0) < synth.ROOM_HI + 0.05).all()


def test_lidar_scan_properties():
    s = synth.LidarScene()
    pts, o = s.scan(0, n_points=4096)
    assert pts.shape == (4096, 3) and pts.dtype == np.float32 and o.dtype == np.float32
    d = np.linalg.norm(pts - o, axis=1)
    assert (d >= s.max_range).any() and (d < s.max_range).any()
    assert np.allclose(s.origin(3), [-3.5, 0.0, 1.7])


def test_depth_frame_properties():
    r = synth.DepthRoom()
    pts, o = r.frame(5, subsample=8)
    assert len(pts) > 1000
    d = np.linalg.norm(pts - o, axis=1)
    assert d.max() < 5.0 * 1.6  # depth <= 5 m, off-axis rays are longer


def test_multi_map_specs():
    specs = synth.multi_map_specs()
    assert len(specs) == 64
    assert min(s.n_points for s in specs) >= 10_000 and max(s.n_points for s in specs) <= 500_000
    assert {s.resolution for s in specs} == {0.02, 0.05, 0.1}
