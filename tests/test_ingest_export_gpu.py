"""The ROS node's two host loops moved onto the GPU, bit-exact with the
oracle: the cloud ingest (non-finite filter + sensor-to-world transform,
bonxai_server.cpp:147-182) fused into the scan's endpoint kernel, and the
occupied-voxel export (bonxai_server.cpp:217-243) as a device compaction."""
import numpy as np
import pytest
import torch

from conftest import golden
from bonxai_gb300 import synth

pytestmark = pytest.mark.gpu


def _pose(k):
    yaw = 0.15 * k - 0.4
    c, s = np.cos(yaw), np.sin(yaw)
    return np.array([[c, -s, 0.0, 0.5 * k - 3.0],
                     [s, c, 0.0, 0.25 * k + 1.0],
                     [0.0, 0.0, 1.0, 1.7]], np.float32)


def _sensor_points(world, m):
    """World points expressed in the sensor frame of pose m (float32)."""
    r = m[:, :3].astype(np.float64)
    t = m[:, 3].astype(np.float64)
    return ((world.astype(np.float64) - t) @ r).astype(np.float32)


def _same(gmap, omap):
    gx, gc = gmap.dump()
    ox, oc = omap.dump()
    assert np.array_equal(gx, ox) and np.array_equal(gc, oc)


@pytest.mark.parametrize("max_range", [30.0, 8.0, -1.0])
def test_sensor_ingest_matches_oracle(gpu, port, max_range):
    scene = synth.LidarScene()
    g = gpu.ProbabilisticMap(0.1)
    o = port.pmap(0.1)
    rng = np.random.default_rng(5)
    for k in range(4):
        world, _ = scene.scan(k, n_points=40000)
        m = _pose(k)
        sp = _sensor_points(world, m)
        bad = rng.choice(len(sp), 300, replace=False)
        sp[bad[:100], 0] = np.nan
        sp[bad[100:200], 1] = np.inf
        sp[bad[200:], 2] = -np.inf
        v = g.insert_sensor_cloud(sp, m, max_range)
        w = port.sensor_to_world(m, sp)
        assert len(w) == len(sp) - 300
        vo = o.insert(w, m[:, 3].copy(), np.inf if max_range < 0 else max_range)
        assert v == vo
    _same(g, o)


def test_sensor_ingest_identity_equals_plain_insert(gpu):
    """With the identity pose the fused ingest is insertPointCloud itself."""
    scene = synth.LidarScene()
    world, origin = scene.scan(0, n_points=30000)
    m = np.hstack([np.eye(3, dtype=np.float32), origin.reshape(3, 1).astype(np.float32)])
    a, b = gpu.ProbabilisticMap(0.1), gpu.ProbabilisticMap(0.1)
    va = a.insert_sensor_cloud(world - origin, m, 30.0)
    vb = b.insert_point_cloud((world - origin) + origin, origin, 30.0)
    assert va == vb
    xa, ca = a.dump()
    xb, cb = b.dump()
    assert np.array_equal(xa, xb) and np.array_equal(ca, cb)


@pytest.mark.parametrize("zband", [(-np.inf, np.inf), (0.0, 2.0), (-1.0, 0.05)])
def test_export_occupied_matches_oracle(gpu, port, zband):
    scene = synth.LidarScene()
    g = gpu.ProbabilisticMap(0.1)
    o = port.pmap(0.1)
    for k in range(3):
        pts, org = scene.scan(k, n_points=50000)
        g.insert_point_cloud(pts, org, 30.0)
        o.insert(pts, org, 30.0)
    eg = g.export_occupied(*zband)
    eo = o.export_occupied(*zband)
    assert len(eg) == len(eo) > 0
    assert np.array_equal(eg.view(np.uint32), eo.view(np.uint32))
    # the headless form: positions stay in a device buffer
    buf = torch.zeros((len(eo) + 7, 3), dtype=torch.float32, device="cuda")
    n = g.export_occupied(*zband, out=buf)
    assert n == len(eo)
    d = buf[:n].cpu().numpy()
    d = d[np.lexsort((d[:, 2], d[:, 1], d[:, 0]))]
    assert np.array_equal(d.view(np.uint32), eo.view(np.uint32))
    # too small a buffer: the count is still reported, nothing past cap written
    small = torch.full((3, 3), -7.0, dtype=torch.float32, device="cuda")
    assert g.export_occupied(*zband, out=small[:2]) == len(eo)
    assert torch.all(small[2] == -7.0)


def test_export_occupied_golden(gpu):
    """Against the reference's own occupied set of the 8-scan LiDAR fixture:
    coordToPos = double(c) * res, narrowed to float."""
    gd = golden("pmap_lidar.npz")
    res = float(gd["resolution"])
    m = gpu.ProbabilisticMap(res)
    for k in range(len(gd["points"])):
        m.insert_point_cloud(gd["points"][k], gd["origins"][k], float(gd["max_range"]))
    pos = gd["occupied"].astype(np.float64) * res

    def narrowed(p):
        f = p.astype(np.float32)
        return f[np.lexsort((f[:, 2], f[:, 1], f[:, 0]))]

    got = m.export_occupied()
    assert np.array_equal(got.view(np.uint32), narrowed(pos).view(np.uint32))
    # the z band applies to the double position, before narrowing
    sel = pos[(pos[:, 2] >= 0.3) & (pos[:, 2] <= 1.0)]
    got = m.export_occupied(0.3, 1.0)
    assert len(sel) > 0
    assert np.array_equal(got.view(np.uint32), narrowed(sel).view(np.uint32))


def test_export_empty_map(gpu):
    m = gpu.ProbabilisticMap(0.05)
    assert len(m.export_occupied()) == 0
