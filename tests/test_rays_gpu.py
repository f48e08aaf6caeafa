import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def test_compute_rays_golden(gpu):
    g = golden("rays.npz")
    rays = gpu.compute_rays(g["pairs"][:, :3], g["pairs"][:, 3:])
    off = 0
    for r, n in zip(rays, g["lens"]):
        assert np.array_equal(r, g["cells"][off:off + n])
        off += n


def test_compute_rays_random_long(gpu, port):
    rng = np.random.default_rng(0)
    o = rng.integers(-1000, 1000, (3000, 3)).astype(np.int32)
    e = o + rng.integers(-700, 700, (3000, 3)).astype(np.int32)
    rays = gpu.compute_rays(o, e)
    for k in range(0, 3000, 7):
        assert np.array_equal(rays[k], port.compute_ray(o[k], e[k]))
