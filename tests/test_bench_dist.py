"""bench.py's multi-rank logic on CPU with the gloo backend (two ranks): the
timed region's max over ranks, the whole-job value of independent replicas,
and the reference arm's non-zero ranks exiting without work."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, world, port, out):
    import torch
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = 10.0 + 5.0 * rank  # rank 1 is the slow one
        total = bench.max_over_ranks(local_ms, world, torch)
        value = bench.job_value(1000, 4, world, total)
        dist.barrier()

        class Args:
            workload = "qspcfw_216_nb32"
            steps = 1
            warmup = 0

        ref = bench.run_reference(Args, rank, world) if rank != 0 else 0  # non-zero ranks: no work
        out.put((rank, total, value, ref))
    finally:
        dist.destroy_process_group()


def test_two_rank_aggregation():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in procs)
    for rank, total, value, ref in res:
        assert total == 15.0  # the slowest rank's time on every rank
        assert value == pytest.approx(2 * 4 * 1000 / 15e-3)
        assert ref == 0
