"""Sharding of ray workloads over ranks.

Rays are independent, so a multi-GPU trace partitions them: each rank traces
a contiguous shard with no communication.  The one exchange step is the sum
of the per-rank sensor images (:func:`reduce_image`), which works for CUDA
tensors over NCCL and for CPU tensors over gloo.
"""

from __future__ import annotations


def shard(n: int, rank: int, world: int) -> slice:
    """Contiguous shard of ``range(n)`` for ``rank`` of ``world`` (sizes
    differ by at most one; the union over ranks is ``range(n)``)."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("rank must be in [0, world)")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    stop = start + base + (1 if rank < extra else 0)
    return slice(start, stop)


def reduce_image(counts, flux, group=None):
    """Sum count and flux images over all ranks, in place."""
    import torch.distributed as dist

    dist.all_reduce(counts, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(flux, op=dist.ReduceOp.SUM, group=group)
    return counts, flux
