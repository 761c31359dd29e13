"""The benchmark's N-rank logic on CPU (gloo, world size 2): each rank runs
its own beam (weak scaling, no data-path collective) and the job's time is
the slowest rank's; the whole-job value counts every rank's points."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    import bench
    from pydfcsr_gb300.synthetic import workload
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert bench.dist_env() == (rank, world, rank)
        step_ms = 2.0 + rank                       # rank 1 is the slow one
        slowest = bench.max_over_ranks(step_ms, world, "cpu")
        value = bench.job_value(4096, world, slowest)
        wl = workload("chicane_c2", n_particles=1000)
        beam = wl.beam(seed=2 + bench.beam_seed(rank))
        out[rank] = (slowest, value, float(beam[4].sum()))
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_ranks_gloo():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 3.0            # max over ranks on every rank
    assert res[0][1] == res[1][1] == pytest.approx(2 * 4096 * 1000.0 / 3.0)
    assert res[0][2] != res[1][2]                   # independent beams per rank


def test_single_rank_needs_no_collective():
    import bench
    assert bench.max_over_ranks(1.25, 1, "cpu") == 1.25
    assert bench.job_value(4096, 1, 2.0) == pytest.approx(2048000.0)
