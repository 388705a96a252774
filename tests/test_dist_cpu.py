"""The N > 1 path of bench.py on CPU (gloo, world size 2): replicas only, the
job's time is the slowest rank's and its work the sum of every rank's; the
reference arm runs on rank 0 alone."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms, nsub = bench.reduce_over_ranks(10.0 + rank, 100 * (rank + 1))
        assert bench.dist_env() == (world, rank, rank)
        # the reference arm: every rank but 0 leaves without work
        ref = bench.run_reference(None, world, rank) if rank else "rank0"
        out.put((rank, ms, nsub, ref))
    finally:
        dist.destroy_process_group()


def test_two_ranks_reduce_time_and_work():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # max of 10, 11 ms; 100 + 200 substeps; the same on both ranks
    assert [(ms, n) for _, ms, n, _ in res] == [(11.0, 300.0), (11.0, 300.0)]
    assert res[1][3] is None
    assert bench.job_value(300.0, 1000, 11.0) == pytest.approx(300.0 * 1000 / 0.011)


def test_single_process_needs_no_group():
    assert bench.reduce_over_ranks(5.0, 7) == (5.0, 7.0)
