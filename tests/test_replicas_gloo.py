"""Multi-rank bookkeeping (fastqsl_gb300.replicas) with two gloo ranks on the
CPU: the timing reduction takes the slowest rank, plane shards tile the cube,
and the whole-job rate counts every rank's units."""
import os
import socket

import pytest
import torch
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from fastqsl_gb300 import replicas
        r, w = replicas.world()
        replicas.barrier()
        ms = replicas.max_over_ranks(10.0 + 5.0 * rank)
        start, count = replicas.plane_shard(128, r, w)
        q.put((r, w, ms, start, count))
    finally:
        torch.distributed.destroy_process_group()


def test_two_gloo_ranks():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(world))
    assert [g[0] for g in got] == [0, 1] and all(g[1] == 2 for g in got)
    assert all(g[2] == 15.0 for g in got)  # the slowest rank's time on every rank
    assert got[0][3:] == (0, 64) and got[1][3:] == (64, 64)


def test_shards_and_rate():
    from fastqsl_gb300 import replicas
    for n, w in ((128, 3), (7, 4), (5, 5)):
        spans = [replicas.plane_shard(n, r, w) for r in range(w)]
        assert spans[0][0] == 0 and sum(c for _, c in spans) == n
        assert all(spans[i][0] + spans[i][1] == spans[i + 1][0] for i in range(w - 1))
    assert replicas.whole_job_rate(8_388_608, 70.0, 2) == pytest.approx(2 * 8_388_608 / 0.07)
    assert replicas.max_over_ranks(3.5) == 3.5
    with pytest.raises(ValueError):
        replicas.plane_shard(10, 3, 3)
