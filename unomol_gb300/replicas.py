"""Multi-GPU measurement of the Fock build: replicas.  Every rank (one process per GPU, launched by
torchrun) runs the whole workload; the timed region is bracketed by barriers and the job's time is the
maximum over ranks, so the whole-job rate is world_size * steps / that time ("weak" scaling: the work
per GPU is fixed).  The reference shards shell quartets over MPI ranks and reduces G
(TwoElectronIntsMPI.cpp:350-354, RHF_MPI.hpp:105-108); one GB300 runs a 32-water build in a few milliseconds, so
replicas (no data-path collective) are the measured multi-GPU form here.

The helpers are backend-agnostic: the tensors live on `device` (CPU for gloo, the rank's GPU for NCCL).
"""
from __future__ import annotations


def env():
    """(world_size, rank, local_rank) from the torchrun environment (1, 0, 0 without it)."""
    import os
    return int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0"))


def barrier(ws: int):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, ws: int, device="cpu") -> float:
    """The largest x over the ranks (x itself on one rank)."""
    if ws <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_rate(steps: int, seconds: float, ws: int, device="cpu") -> float:
    """Whole-job rate: every rank ran `steps` steps; the job took the slowest rank's time."""
    return ws * steps / max_over_ranks(seconds, ws, device)
