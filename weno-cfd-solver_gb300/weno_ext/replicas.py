"""Independent replicas across GPUs (one process per GPU, torchrun layout).

The 2D step does not shard here: `bench.py --gpus N` runs N independent
replicas of the same workload, one per rank, and reports the whole-job rate
(all ranks' cell-updates over the slowest rank's time).  These helpers hold the
rank bookkeeping, the barrier around the timed region and the max-over-ranks
reduction; they work with NCCL on GPUs and with gloo on CPU (tests).
"""

from __future__ import annotations

import os


def world():
    """(world_size, rank, local_rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend):
    import torch.distributed as dist
    if world()[0] > 1 and not dist.is_initialized():
        dist.init_process_group(backend)


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def max_over_ranks(value, device="cpu"):
    """The largest `value` over all ranks (the timed region's wall: the slowest rank)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank, ms_max, world_size):
    """Whole-job rate: every rank processed `units_per_rank` in at most `ms_max`."""
    return units_per_rank * world_size / (ms_max / 1e3)


def finish():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.destroy_process_group()
