"""Replica runs on several GPUs: every rank runs its own independent job on
its own GPU (the path has no cross-GPU exchange), and only the timing and
throughput figures are combined across ranks -- the slowest rank's time, the
sum of the ranks' throughputs.  Works with any torch.distributed backend
(NCCL on GPUs, gloo on CPU)."""
import os

import torch
import torch.distributed as dist


def world():
    """(world size, rank, local rank) from the launcher's environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def _device():
    return "cuda" if dist.get_backend() == "nccl" else "cpu"


def barrier():
    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def max_over_ranks(x):
    """The largest x over all ranks (x itself when not distributed)."""
    if not (dist.is_available() and dist.is_initialized()):
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x):
    """The sum of x over all ranks (x itself when not distributed)."""
    if not (dist.is_available() and dist.is_initialized()):
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t)
    return float(t.item())


def replica_throughput(units_per_rank, seconds):
    """Whole-job throughput of a replica run: units all ranks processed over
    the slowest rank's time."""
    return sum_over_ranks(units_per_rank) / max_over_ranks(seconds)
