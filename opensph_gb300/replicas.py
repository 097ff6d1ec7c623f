"""Independent replicas on several GPUs of one node: one process per GPU, launched by torchrun.

The hot path does not shard (each rank steps its own copy of the workload; there is no data-path exchange), so
the only collective work is the timing: every rank is held at a barrier before its timed region, the whole-job
time is the maximum over the ranks, and the whole-job rate counts every rank's particles. NCCL carries these
scalars between GPU ranks, gloo between CPU processes (tests)."""
import os

import torch


def world_info():
    """(rank, world size, local rank) from the torchrun environment; (0, 1, 0) without it."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def distributed():
    return torch.distributed.is_available() and torch.distributed.is_initialized() and \
        torch.distributed.get_world_size() > 1


def barrier():
    if distributed():
        torch.distributed.barrier()


def max_over_ranks(value, device="cpu"):
    """The maximum of a per-rank float over all ranks (the value itself on one rank). device: where the
    collective's tensor lives (a CUDA device for NCCL, "cpu" for gloo)."""
    if not distributed():
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, steps, world, ms_max):
    """Whole-job throughput (units per second): every rank processed units_per_rank per step for the given steps
    within the slowest rank's time ms_max."""
    return units_per_rank * steps * world / (ms_max * 1e-3)
