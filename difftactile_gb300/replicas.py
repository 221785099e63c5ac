"""Runs on several GPUs of one node: one process per GPU, each stepping a World of its own.

Environments never exchange data (the reference has no communication on this path), so there is
no collective on the data path: a rank either replicates the whole workload (weak scaling: the
per-GPU work stays fixed as ranks are added) or takes a contiguous share of the environments.  Ranks
meet only to time a step (the slowest rank's time) and to add up what they processed.  Every
function here works on any torch.distributed backend (NCCL between GPUs, gloo on the host).
"""
from __future__ import annotations

import os

import torch
import torch.distributed as dist


def rank_info() -> tuple[int, int, int]:
    """(rank, world size, local rank) from the launcher's environment (1 process when unset)."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard(n: int, rank: int, world_size: int) -> range:
    """Contiguous share of n environments for `rank`: sizes differ by at most one, every
    environment belongs to exactly one rank."""
    q, r = divmod(n, world_size)
    lo = rank * q + min(rank, r)
    return range(lo, lo + q + (1 if rank < r else 0))


def _reduce(x: float, op, device) -> float:
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=op)
    return float(t.item())


def slowest(x: float, device="cpu") -> float:
    """Maximum of x over the ranks (a step lasts as long as its slowest rank)."""
    return _reduce(x, dist.ReduceOp.MAX, device)


def total(x: float, device="cpu") -> float:
    """Sum of x over the ranks (units processed by the whole job)."""
    return _reduce(x, dist.ReduceOp.SUM, device)


def barrier():
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()
