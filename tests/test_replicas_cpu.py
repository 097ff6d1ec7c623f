"""The multi-rank host logic of bench.py (opensph_gb300/replicas.py) on two CPU processes over gloo: the barrier
before the timed region, the whole-job time as the maximum over the ranks, and the whole-job rate counting every
rank's particles. The GPU ranks run the same functions over NCCL."""
import os
import socket

import pytest
import torch
import torch.multiprocessing as mp

from opensph_gb300 import replicas


def free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def worker(rank, world, port, out):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank)})
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = replicas.world_info()
        replicas.barrier()
        # each rank's own timed region: rank k took 10 * (k + 1) ms for its 1,000 particles x 5 steps
        ms = replicas.max_over_ranks(10.0 * (rank + 1))
        out[rank] = (r, w, local, ms, replicas.job_rate(1000, 5, w, ms))
    finally:
        torch.distributed.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_gloo_ranks_take_the_slowest_time_and_count_every_rank():
    world = 2
    ctx = mp.get_context("spawn")
    with ctx.Manager() as manager:
        out = manager.dict()
        mp.start_processes(worker, args=(world, free_port(), out), nprocs=world, start_method="spawn", join=True)
        res = dict(out)
    assert sorted(res) == [0, 1]
    for rank, (r, w, local, ms, rate) in res.items():
        assert (r, w, local) == (rank, world, rank)
        assert ms == 20.0
        assert rate == pytest.approx(1000 * 5 * world / 0.020)


def test_single_process_needs_no_collective():
    assert not replicas.distributed()
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.job_rate(100, 2, 1, 10.0) == pytest.approx(20000.0)
