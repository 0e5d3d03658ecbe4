"""Replica bookkeeping for runs on N GPUs of one node (one process per GPU,
launched by torchrun). The path shards by frames, views and pixels with
read-only scene copies and has no exchange step, so ranks only meet to
start the timed region together and to take the slowest rank's time: the
whole-job rate is the units all ranks processed over that maximum.
"""
from __future__ import annotations

import os
from dataclasses import dataclass


@dataclass
class Ranks:
    world: int
    rank: int
    local: int
    dist: object | None    # torch.distributed when world > 1
    device: str            # tensor device for collectives ("cuda" for nccl, "cpu" for gloo)


def init(backend: str = "nccl") -> Ranks:
    """Reads RANK / LOCAL_RANK / WORLD_SIZE (torchrun) and joins the process
    group when there is more than one rank."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend)
    return Ranks(world, rank, local, dist, "cuda" if backend == "nccl" else "cpu")


def barrier(r: Ranks) -> None:
    if r.dist is not None:
        r.dist.barrier()


def max_over_ranks(r: Ranks, x: float) -> float:
    """The largest x over all ranks (every rank gets it)."""
    if r.dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=r.device)
    r.dist.all_reduce(t, op=r.dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, r: Ranks, seconds_this_rank: float) -> float:
    """Units of all ranks per second of the slowest rank (weak scaling: every
    rank does the same work)."""
    return units_per_rank * r.world / max_over_ranks(r, seconds_this_rank)


def finish(r: Ranks) -> None:
    if r.dist is not None:
        r.dist.destroy_process_group()
