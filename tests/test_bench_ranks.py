"""Replicas on several ranks (host logic, CPU, gloo, world size 2): the
timed region's clock is the slowest rank's, the whole-job rate counts every
rank's trajectories, and the reference arm runs on rank 0 alone."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist

    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(10.0 + 5.0 * rank, world, "cpu")
        rate = bench.whole_job_rate(world, 24, 40, t)

        class Args:
            workload = "ccsd_o10_v14"
            method = "CCSD"
            nb = 24
            steps = 1
        if rank != 0:
            bench.run_reference(Args, rank, world)  # rank != 0: returns at once, no oracle run
        q.put((rank, t, rate))
    finally:
        dist.destroy_process_group()


def test_two_ranks_share_the_slowest_clock():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [15.0, 15.0]
    # 2 ranks x 24 trajectories x 40 steps in 15 ms
    assert out[0][2] == pytest.approx(2 * 24 * 40 / 0.015)


def test_single_rank_is_the_identity():
    import bench
    assert bench.max_over_ranks(3.5, 1, "cpu") == 3.5
    assert bench.whole_job_rate(1, 1, 10, 100.0) == pytest.approx(100.0)
