"""Replica bookkeeping for multi-GPU benchmark runs.

The step has no inter-GPU exchange on one GPU (the whole grid is resident),
so N GPUs run N independent replicas of the same problem ("replicas only").
These helpers do the only cross-rank work: agree on the slowest rank's time
and form the whole-job throughput.  They use torch.distributed with any
backend (NCCL on GPUs, gloo in the CPU tests).
"""
import os

import torch
import torch.distributed as dist


def rank_info():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def init(backend):
    """Join the process group described by the torchrun environment (no-op
    for a single process)."""
    rank, world, _ = rank_info()
    if world > 1 and not dist.is_initialized():
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend, rank=rank, world_size=world)
    return rank, world


def _device():
    if dist.is_initialized() and dist.get_backend() == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def max_over_ranks(x: float) -> float:
    if not dist.is_initialized():
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x: float) -> float:
    if not dist.is_initialized():
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=_device())
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier():
    if dist.is_initialized():
        dist.barrier()


def job_throughput(units_this_rank: float, seconds_this_rank: float) -> float:
    """Units of all ranks divided by the slowest rank's time."""
    return sum_over_ranks(units_this_rank) / max_over_ranks(seconds_this_rank)
