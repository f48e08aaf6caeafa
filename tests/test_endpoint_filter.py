"""The float filter of the endpoint math (bxg_scan.cuh: make_ep_fast,
endpoint_fast), restated in numpy float32, against the double computation of
insertPointCloud (probabilistic_map.hpp:144-156): wherever the filter accepts a
point, its hit/miss decision and cell equal the double result. numpy float32
and float64 operations round to nearest without contraction, as the kernels'
__f*_rn / __d*_rn intrinsics do."""
import numpy as np
import pytest

U = np.float32(2.0 ** -24)


def make_fast(origin, max_range, res):
    inv_res = 1.0 / res
    mr2 = max_range * max_range
    hi = np.float32(mr2 * (1.0 + 2.0 ** -19))
    lo = np.float32(mr2 * (1.0 - 2.0 ** -19))
    return dict(o=origin.astype(np.float32), inv_res=np.float32(inv_res),
                mr=np.float32(max_range), sq_hi=np.nextafter(hi, np.float32(np.inf)),
                sq_lo=np.nextafter(lo, np.float32(0)))


def double_path(p, origin, max_range, res):
    t = p.astype(np.float64)
    f = origin.astype(np.float64)
    v = t - f
    sq = (v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2]
    miss = sq >= max_range * max_range
    s = np.sqrt(sq)
    with np.errstate(divide="ignore", invalid="ignore"):
        e_m = f + (v / s[:, None]) * max_range
    e = np.where(miss[:, None], e_m, t)
    return np.floor(e * (1.0 / res)).astype(np.int64), miss


def fast_path(p, F):
    o = F["o"]
    v = (p - o).astype(np.float32)
    sq = (v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2]
    hit = sq < F["sq_lo"]
    miss = sq > F["sq_hi"]
    ok = (hit | miss) & (sq < np.float32(1e30))
    s = np.sqrt(sq)
    with np.errstate(divide="ignore", invalid="ignore"):
        e_m = o + (v / s[:, None]) * F["mr"]
    e = np.where(miss[:, None], e_m, p).astype(np.float32)
    y = (e * F["inv_res"]).astype(np.float32)
    ay, ae = np.abs(y), np.abs(e)
    tol_hit = ay * np.float32(4.76837158e-7)
    tol_miss = ((np.float32(8) * F["mr"] + ae) * F["inv_res"] + np.float32(2) * ay) * \
        np.float32(2.38418579e-7)
    tol = np.where(miss[:, None], tol_miss, tol_hit).astype(np.float32)
    fl = np.floor(y)
    good = (np.abs(y) < np.float32(8388608)) & ((y - fl) > tol) & (((fl + 1) - y) > tol)
    zero = hit[:, None] & (e == 0)
    cell = np.where(zero, 0, fl).astype(np.int64)
    ok &= np.all(good | zero, axis=1)
    return cell, miss, ok


CASES = [
    (0.1, (0.0, 0.0, 0.0), 30.0),
    (0.1, (1.25, -3.5, 1.7), 30.0),
    (0.05, (0.3, 0.1, 0.0), 12.5),
    (0.02, (-2.0, 4.0, 1.0), 5.0),
    (0.3, (100.0, -50.0, 3.0), 60.0),
    (0.07, (12.345, 6.789, -0.5), 1e6),
]


@pytest.mark.parametrize("res,origin,max_range", CASES)
def test_filter_agrees_with_double(res, origin, max_range):
    origin = np.array(origin, np.float32)
    rng = np.random.default_rng(int(res * 1e4))
    n = 400_000
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rand = (origin + d * rng.uniform(0.0, 2.5 * min(max_range, 80.0), (n, 1))).astype(np.float32)
    k = rng.integers(-500, 500, (n, 3))
    grid = (k * res).astype(np.float32)
    near = np.nextafter(grid, np.where(rng.random((n, 3)) < 0.5, -np.inf, np.inf).astype(np.float32))
    scale = max_range * (1.0 + rng.integers(-16, 17, (n, 1)) * 2.0 ** -24)
    ring = (origin.astype(np.float64) + d * scale).astype(np.float32)
    tgt = rng.integers(-300, 300, (n, 3)) * res - origin.astype(np.float64)
    tgt /= np.linalg.norm(tgt, axis=1, keepdims=True)
    far = (origin + tgt * (max_range * rng.uniform(1.0, 2.0, (n, 1)))).astype(np.float32)
    F = make_fast(origin, max_range, res)
    for name, p in [("random", rand), ("grid", grid), ("near-grid", near), ("ring", ring),
                    ("far", far)]:
        want, wmiss = double_path(p, origin, max_range, res)
        got, gmiss, ok = fast_path(p, F)
        assert np.array_equal(got[ok], want[ok]), name
        assert np.array_equal(gmiss[ok], wmiss[ok]), name
        if name == "random":
            assert ok.mean() > 0.99, ok.mean()
