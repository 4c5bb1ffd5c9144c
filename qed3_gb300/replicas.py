"""Multi-GPU = independent replicas (one process per GPU, no data-path collective).

The fermion hot path shards at job level -- right-hand sides, pseudofermions,
Zolotarev poles, lattices, seeds -- so N GPUs run N independent workloads.
These helpers split a job list across ranks and reduce timings for reporting;
the only collectives are the timing barrier and a max/sum of scalars.
"""
from __future__ import annotations


def shard(n_items: int, rank: int, world: int) -> range:
    """Contiguous block of items owned by `rank` (sizes differ by at most one)."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad rank/world")
    base, extra = divmod(n_items, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def _reduce(value: float, op: str) -> float:
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    backend = dist.get_backend()
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def max_over_ranks(value: float) -> float:
    return _reduce(value, "max")


def sum_over_ranks(value: float) -> float:
    return _reduce(value, "sum")


def barrier():
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized():
        dist.barrier()
