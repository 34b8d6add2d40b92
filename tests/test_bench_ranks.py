"""CPU tests of the multi-rank logic of bench.py (replicas only): two gloo
ranks on 127.0.0.1.  The timed value of a run over N GPUs takes the slowest
replica's time (the maximum over ranks), and the reference arm runs on rank 0
alone, the other ranks leaving without work."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        got = bench.max_over_ranks(torch, 10.0 + 3.0 * rank, "cpu", world)
        args = type("A", (), {"steps": 1, "warmup": 1, "gpus": world})()
        skipped = bench.run_reference(args) == 0 if rank != 0 else True
        q.put((rank, got, skipped))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_reference_rank_split():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert sorted(r for r, _, _ in out) == [0, 1]
    assert all(got == 13.0 for _, got, _ in out)
    assert all(skipped for _, _, skipped in out)


def test_max_over_ranks_single_rank_is_identity():
    import torch

    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks(torch, 1.25, "cpu", 1) == 1.25
