"""The N > 1 host logic of bench.py on CPU with gloo, world size 2: every
rank times its own replica, rank 0 reports the whole-job rate from the
slowest rank, and the reference arm runs on rank 0 only."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, q):
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    try:
        # rank r's replica took 10 + 5 r ms for 100 steps and 20 - r ms end to end
        local = [10.0 + 5.0 * rank, 20.0 - rank]
        dist.barrier()
        total_ms, e2e_ms = bench.max_over_ranks(torch, local, world, "cpu")
        value = bench.whole_job_rate(world, 100, total_ms)

        class A:
            steps, warmup, gpus = 3, 1, world
        # the reference arm: rank 0 alone does work; other ranks return at once
        if rank != 0:
            assert bench.run_reference(A, rank, world) is None
        q.put((rank, total_ms, e2e_ms, value))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_ranks_report_slowest():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs), [p.exitcode for p in procs]
    res = sorted(q.get(timeout=5) for _ in range(world))
    for rank, total_ms, e2e_ms, value in res:
        assert total_ms == 15.0 and e2e_ms == 20.0
        assert abs(value - 2 * 100 / 0.015) < 1e-6
