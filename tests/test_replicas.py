"""The multi-GPU path is replicas only: every rank runs its own system, with no
collective on the data path; the job's time is the slowest rank's and its
throughput counts every rank's particles.  These run as two gloo ranks on the
CPU (the reduction and the workload split), and check that the reference arm's
non-zero ranks leave without work."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    import torch.distributed as dist

    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")
        # each rank draws its own system: the replicas are independent
        class A:
            dist, n, so, sizes = "uniform", 1000, 0, None
        pos, _ = bench.workload(A, 0 + rank)
        out[rank] = (t, float(pos[0, 0]))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_independent_replicas():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    ps = [ctx.Process(target=_rank, args=(r, world, port, out)) for r in range(world)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
        assert p.exitcode == 0
    assert out[0][0] == out[1][0] == 15.0  # the slowest rank's time, on every rank
    assert out[0][1] != out[1][1]  # different systems per rank


def test_job_throughput_counts_every_rank():
    import bench

    assert bench.job_throughput(1_000_000, 10, 4, 1000.0) == pytest.approx(4e7)
    assert bench.max_over_ranks(3.0) == 3.0  # one process: no reduction


def test_reference_arm_other_ranks_do_nothing():
    import bench

    class A:
        pass

    assert bench.run_reference(A, 1, 2) is None  # returns before touching the workload
