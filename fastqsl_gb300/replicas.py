"""Multi-GPU bookkeeping of the Q pipeline.

Seeds are independent, so the path shards with no exchange on the data path:
each rank traces its own planes (or, for weak scaling, its own copy of the
workload) on its own GPU.  The only collective is the timing reduction of a
benchmark (the slowest rank's time), done here over whatever process group
is initialised (NCCL on GPUs, gloo in the CPU tests).
"""
from __future__ import annotations

import torch


def world():
    d = torch.distributed
    if d.is_available() and d.is_initialized():
        return d.get_rank(), d.get_world_size()
    return 0, 1


def max_over_ranks(x: float, device="cpu") -> float:
    """The largest `x` over all ranks (x itself without a process group)."""
    r, w = world()
    if w == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def barrier():
    r, w = world()
    if w > 1:
        torch.distributed.barrier()


def plane_shard(nplanes: int, rank: int, nranks: int):
    """Contiguous z-plane range [start, start + count) of `rank` when
    `nplanes` planes are split over `nranks` ranks (sizes differ by at most
    one plane)."""
    if nranks < 1 or not (0 <= rank < nranks):
        raise ValueError("rank out of range")
    base, extra = divmod(int(nplanes), int(nranks))
    start = rank * base + min(rank, extra)
    return start, base + (1 if rank < extra else 0)


def whole_job_rate(units_per_rank: float, ms_max: float, nranks: int) -> float:
    """Units per second of the whole job: every rank processed
    units_per_rank units within the slowest rank's ms_max milliseconds."""
    return float(units_per_rank) * int(nranks) / (float(ms_max) / 1e3)
