"""Host-side multi-GPU logic on CPU: maps partition across ranks with no
collective on the data path; throughput aggregates over ranks (gloo, 2 ranks)."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from bonxai_gb300 import sharding, synth


def test_assignment_is_a_balanced_partition():
    sizes = [s.n_points for s in synth.multi_map_specs(64)]
    for ws in (1, 2, 3, 4, 8):
        rank_of = sharding.assign_maps(sizes, ws)
        assert sorted(sum((sharding.my_maps(sizes, ws, r) for r in range(ws)), [])) == list(range(64))
        loads = [sum(sizes[i] for i in range(64) if rank_of[i] == r) for r in range(ws)]
        assert max(loads) - min(loads) <= max(sizes)
    assert sharding.assign_maps(sizes, 4) == sharding.assign_maps(sizes, 4)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, ws, port, sizes, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    mine = sharding.my_maps(sizes, ws, rank)
    units = float(sum(sizes[i] for i in mine))
    seconds = 1.0 + rank  # rank 1 is the slow one
    tot_units, max_t = sharding.aggregate(units, seconds)
    q.put((rank, mine, tot_units, max_t))
    dist.destroy_process_group()


def test_two_rank_gloo_aggregation():
    sizes = [s.n_points for s in synth.multi_map_specs(64)]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, sizes, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, m0, u0, t0), (r1, m1, u1, t1) = res
    assert set(m0).isdisjoint(m1) and sorted(m0 + m1) == list(range(64))
    assert u0 == u1 == float(sum(sizes))
    assert t0 == t1 == 2.0
