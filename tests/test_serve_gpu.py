"""Serving loop: a client's requests give the same results alone and mixed
with other clients' traffic (continuous batching), and match the oracle."""
import threading

import numpy as np
import pytest

from bonxai_gb300 import synth

pytestmark = pytest.mark.gpu


def _client_sequence(seed):
    scene = synth.LidarScene(seed=seed)
    rng = np.random.default_rng(seed)
    q1 = rng.integers([-60, -60, -5], [60, 60, 40], (20000, 3)).astype(np.int32)
    q2 = rng.integers([-60, -60, -5], [60, 60, 40], (5000, 3)).astype(np.int32)
    seq = []
    for k in range(3):
        pts, o = scene.scan(k, n_points=6000 + 2000 * k)
        seq.append(("insert", pts, o))
        seq.append(("query", q1 if k != 1 else q2, k % 3))
        if k == 1:
            seq.append(("occupied",))
    return seq


def _submit(srv, map_id, req):
    if req[0] == "insert":
        return srv.insert(map_id, req[1], req[2], 30.0)
    if req[0] == "query":
        return srv.query(map_id, req[1], mode=req[2])
    return srv.get_occupied(map_id)


def _collect(srv, req, t):
    if req[0] == "insert":
        r = srv.wait_insert(t)
        return ("insert", r["status"], r["ray_cells"])
    if req[0] == "query":
        r, out = srv.wait_query(t, len(req[1]))
        return ("query", r["status"], out.tobytes())
    r, out = srv.wait_occupied(t)
    return ("occupied", r["status"], out.tobytes())


def test_same_alone_and_in_the_mix(gpu, port):
    seq = _client_sequence(9100)
    # alone
    alone_srv = gpu.Server([0.1])
    tickets = [_submit(alone_srv, 0, r) for r in seq]
    alone = [_collect(alone_srv, r, t) for r, t in zip(seq, tickets)]
    alone_dump = alone_srv.map_dump(0)
    alone_srv.close()

    # in the mix: 6 clients, client 0's map is map 3, the others send load
    res = [0.05, 0.1, 0.02, 0.1, 0.05, 0.1]
    srv = gpu.Server(res)
    stop = threading.Event()

    noise_ids = (0, 1, 2, 4, 5)
    started = threading.Barrier(len(noise_ids) + 1)

    def noise(cid):
        # the load is generated up front, so that it is in flight while
        # client 0's requests run
        rng = np.random.default_rng(cid)
        sc = synth.LidarScene(seed=9200 + cid)
        work = []
        for k in range(6):
            if rng.random() < 0.6:
                work.append(("i",) + sc.scan(k, n_points=int(rng.integers(2000, 8000))))
            else:
                n = int(rng.integers(100, 50000))
                work.append(("q", rng.integers(-100, 100, (n, 3)).astype(np.int32),
                             int(rng.integers(0, 3))))
        first = True
        k = 0
        while (first or not stop.is_set()) and k < 200:
            w = work[k % len(work)]
            if w[0] == "i":
                srv.insert(cid, w[1], w[2], 30.0, discard=True)
            else:
                srv.query(cid, w[1], mode=w[2], discard=True)
            k += 1
            if first:
                started.wait(timeout=120)
                first = False

    threads = [threading.Thread(target=noise, args=(c,)) for c in noise_ids]
    for th in threads:
        th.start()
    started.wait(timeout=120)
    tickets = [_submit(srv, 3, r) for r in seq]
    mixed = [_collect(srv, r, t) for r, t in zip(seq, tickets)]
    stop.set()
    for th in threads:
        th.join()
    srv.drain()
    st = srv.stats()
    assert st["ticks"] > 1 and st["completed"] > len(seq)
    mixed_dump = srv.map_dump(3)
    srv.close()

    assert [m[:2] for m in mixed] == [a[:2] for a in alone]
    assert mixed == alone
    assert np.array_equal(mixed_dump[0], alone_dump[0])
    assert np.array_equal(mixed_dump[1], alone_dump[1])

    # and the oracle agrees
    om = port.pmap(0.1)
    for req, got in zip(seq, alone):
        if req[0] == "insert":
            assert got[2] == om.insert(req[1], req[2], 30.0)
        elif req[0] == "query":
            ans = om.query(req[1])[req[2]]
            assert got[2] == ans.tobytes()
        else:
            assert got[2] == om.occupied().tobytes()
    ox, oc = om.dump()
    assert np.array_equal(alone_dump[0], ox) and np.array_equal(alone_dump[1], oc)


def test_budget_admission_rejects_and_continues(gpu):
    cfg = gpu.ServerConfig(pool_budget_bytes=64 << 20, initial_leaves=1024)
    srv = gpu.Server([0.1, 0.1], cfg)
    scene = synth.LidarScene()
    t_big = srv.insert(0, *scene.scan(0), 30.0)          # 131k points: over the budget
    t_q = srv.query(1, np.zeros((10, 3), np.int32))
    r = srv.wait_insert(t_big)
    assert r["status"] == 2  # BXG_ERR_OUT_OF_POOL
    rq, out = srv.wait_query(t_q, 10)
    assert rq["status"] == 0 and len(out) == 10
    assert srv.stats()["rejected"] == 1


def test_insert_waits_for_budget_until_another_map_is_cleared(gpu, port):
    """An insert that does not fit the HBM budget waits at the head of its
    map's queue; clearing another client's map (releasing its pools) lets it
    in, and its result is the same as inserting alone."""
    scene = synth.LidarScene()
    pts_a, o_a = scene.scan(0)
    pts_b, o_b = scene.scan(3)
    srv = gpu.Server([0.1, 0.1], gpu.ServerConfig(pool_budget_bytes=120 << 20,
                                                  initial_leaves=4096))
    try:
        ra = srv.wait_insert(srv.insert(0, pts_a, o_a, 30.0))
        assert ra["status"] == 0
        tb = srv.insert(1, pts_b, o_b, 30.0)
        with pytest.raises(gpu.BonxaiError) as ei:  # still waiting for budget
            srv.wait_insert(tb, timeout=0.5)
        assert ei.value.status == 4
        assert srv.stats()["deferred"] >= 1
        srv.wait_insert(srv.clear(0))
        rb = srv.wait_insert(tb, timeout=60.0)
        assert rb["status"] == 0 and srv.stats()["rejected"] == 0
        o = port.pmap(0.1)
        assert rb["ray_cells"] == o.insert(pts_b, o_b, 30.0)
        srv.drain()
        xb, cb = srv.map_dump(1)
        ox, oc = o.dump()
        assert np.array_equal(xb, ox) and np.array_equal(cb, oc)
        xa, _ = srv.map_dump(0)
        assert len(xa) == 0  # cleared
    finally:
        srv.close()


def test_insert_that_never_fits_fails_at_its_deadline(gpu):
    scene = synth.LidarScene()
    pts, o = scene.scan(0)
    srv = gpu.Server([0.1], gpu.ServerConfig(pool_budget_bytes=24 << 20, initial_leaves=4096,
                                             admission_timeout_s=0.3))
    try:
        r = srv.wait_insert(srv.insert(0, pts, o, 30.0), timeout=30.0)
        assert r["status"] == 2  # BXG_ERR_OUT_OF_POOL
        assert r["latency_ms"] >= 250.0
        assert srv.stats()["rejected"] == 1
    finally:
        srv.close()
