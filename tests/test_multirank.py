"""The benchmark's multi-process path on the CPU: two gloo ranks (the GPU
path runs one process per GPU over NCCL with the same logic). Each rank
scans its own shard (replicas, no data-path collective); the reported time
is the slowest rank's, and only rank 0 prints."""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, results):
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import numpy as np

    import bench
    import oracle
    try:
        # Every rank scans its own seeded shard with the oracle's threaded
        # CPU scan and "times" it; the job reports the slowest rank.
        rng = np.random.default_rng(100 + rank)
        x = rng.integers(0, 256, size=1 << 16, dtype=np.uint32)
        y = oracle.scan_mt(x, threads=2)
        assert oracle.validate(x, y, False) == 0
        slowest = bench.max_over_ranks(1.5 + rank, dist, device="cpu")
        # The reference arm works and prints on rank 0 only: the other ranks
        # return before looking at their arguments.
        buf = io.StringIO()
        if rank != 0:
            with redirect_stdout(buf):
                bench.run_reference(None, world, rank)
        results[rank] = (slowest, buf.getvalue())
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_report_the_slowest_rank():
    world = 2
    port = _free_port()
    manager = mp.get_context("spawn").Manager()
    results = manager.dict()
    mp.start_processes(_worker, args=(world, port, results), nprocs=world, join=True, start_method="spawn")
    assert results[0][0] == pytest.approx(2.5) and results[1][0] == pytest.approx(2.5)
    assert results[1][1] == ""  # non-zero ranks of the reference arm print nothing


def test_single_process_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25) == 3.25
