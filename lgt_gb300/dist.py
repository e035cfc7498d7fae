"""Replica-parallel helpers (one process per GPU, no data-path collective).

Coupling points and lattices are independent units: each rank solves its own
share on its own GPU.  The only cross-rank operations are host-side timing
reductions (a barrier and the max of the elapsed time), done over whatever
process group torch.distributed provides (gloo on CPU, NCCL on GPUs).  The
reference distributes the same way, as independent SLURM array tasks
(run_finite_ed.sh:20, run_gs_benchmark_largeD.sh:23).
"""
from __future__ import annotations

import os


def world():
    """(rank, world_size, local_rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard(items, rank: int, world_size: int):
    """Contiguous block of `items` owned by `rank`; blocks differ in length
    by at most one and their concatenation over ranks is `items`."""
    n = len(items)
    base, extra = divmod(n, world_size)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return items[lo:hi]


def max_over_ranks(value: float) -> float:
    """Max of a host scalar over all ranks (identity without a process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64)
    if dist.get_backend() == "nccl":
        t = t.cuda()
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized():
        dist.barrier()
