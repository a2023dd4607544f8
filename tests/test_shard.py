"""Instance sharding (braingrid_gb300/shard.py): the split of batched networks and served jobs
over GPUs is a deterministic, complete and balanced partition that every rank computes alone;
whole-job figures and per-job results cross ranks only at the end.  The multi-rank parts run as
world_size-2 gloo groups on the CPU."""
import multiprocessing
import os
import socket

import numpy as np
import pytest

from braingrid_gb300 import shard


def test_partition_complete_disjoint_balanced_deterministic():
    rs = np.random.RandomState(0)
    for parts in (1, 2, 3, 8):
        for n in (0, 1, 5, 36, 512):
            w = rs.exponential(1.0, n)
            p = shard.partition(w, parts)
            assert len(p) == parts
            assert sorted(i for q in p for i in q) == list(range(n))
            if n:
                loads = [float(w[q].sum()) for q in p]
                assert max(loads) - min(loads) <= float(w.max()) + 1e-9
            assert p == shard.partition(list(w), parts)


def test_partition_rejects_bad_input():
    for bad in ([1.0, -1.0], [np.nan], [[1.0]]):
        with pytest.raises(ValueError):
            shard.partition(bad, 2)
    with pytest.raises(ValueError):
        shard.partition([1.0], 0)
    with pytest.raises(ValueError):
        shard.share([1], [1.0], 2, 2)


def test_single_process_reporting_is_local():
    assert shard.reduce_timing(10, 2.5) == (10.0, 2.5)
    assert shard.gather({"a": 1}) == [{"a": 1}]
    p = shard.latency_percentiles([1.0, 2.0, 3.0, 4.0])
    assert p["p50"] == 2.5 and p["p99"] == pytest.approx(3.97)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from braingrid_gb300 import serve, workloads
        members = workloads.sweep36_members()
        weights = [m["width"] * m["height"] * m["max_syn"] for m in members]
        mine = shard.share(list(range(len(members))), weights, rank, world)
        units, t = shard.reduce_timing(float(sum(weights[i] for i in mine)), 1.0 + rank)
        nets = shard.gather(mine)
        part = serve.sharded_trace(workloads.served_trace(12), rank, world)
        jobs = shard.gather([(a, job.name, int(job.desc.noise_seed)) for a, job in part])
        shard.barrier()
        q.put((rank, mine, units, t, nets, jobs))
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo_sharding_and_reporting():
    world = 2
    ctx = multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    got = {}
    try:
        for _ in range(world):
            r = q.get(timeout=240)
            got[r[0]] = r
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert all(p.exitcode == 0 for p in procs)
    from braingrid_gb300 import workloads
    members = workloads.sweep36_members()
    weights = [m["width"] * m["height"] * m["max_syn"] for m in members]
    r0, r1 = got[0], got[1]
    # the networks: each rank's share, disjoint and complete, as rank 0 gathered them
    assert sorted(r0[1] + r1[1]) == list(range(len(members)))
    assert r0[4] == [r0[1], r1[1]] and r1[4] is None
    # whole-job figures: units summed, time of the slowest rank, on every rank
    assert r0[2] == r1[2] == float(sum(weights))
    assert r0[3] == r1[3] == 2.0
    # the served trace: every job on exactly one rank, arrival times kept
    trace = workloads.served_trace(12)
    every = sorted(x for part in r0[5] for x in part)
    assert every == sorted((a, j.name, int(j.desc.noise_seed)) for a, j in trace)
    assert all(len(part) > 0 for part in r0[5])


def _rank_dies(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import datetime
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world,
                            timeout=datetime.timedelta(seconds=20))
    if rank == 1:
        os._exit(3)  # a rank lost before the end-of-run reporting
    try:
        shard.gather(["rank 0 results"])
        q.put("no error")
    except Exception as e:  # the loss surfaces as an error, not a hang
        q.put("error: " + type(e).__name__)


def test_a_lost_rank_is_reported_at_the_gather_not_hung():
    world = 2
    ctx = multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_dies, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    try:
        msg = q.get(timeout=120)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert msg.startswith("error"), msg
    assert procs[1].exitcode == 3
