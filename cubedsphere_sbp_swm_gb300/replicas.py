"""Replica runs: one process per GPU, each stepping its own independent
instance.  The path does not shard (all six panels of an instance live on one
GPU and the cube-edge pairing is an in-device step), so several GPUs run
replicas with no data-path collective.  The whole-job rate is the units all
replicas processed over the slowest replica's time; the only collective is
that one maximum, taken after the timed region."""
from __future__ import annotations


def world() -> tuple[int, int]:
    """(world size, rank) of the initialised default process group, else (1, 0)."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        return dist.get_world_size(), dist.get_rank()
    return 1, 0


def max_over_ranks(value: float, device=None) -> float:
    """The maximum of `value` over the ranks of the default process group
    (value itself in a single process).  device: where the reduction tensor
    lives (a CUDA device for NCCL, None for gloo)."""
    import torch
    import torch.distributed as dist
    if world()[0] == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: float, seconds: float, device=None) -> tuple[float, float]:
    """(whole-job units per second, slowest rank's seconds) for replicas that
    each processed units_per_rank units in `seconds`."""
    if seconds <= 0:
        raise ValueError("seconds must be positive")
    ws = world()[0]
    slow = max_over_ranks(seconds, device)
    return ws * units_per_rank / slow, slow
