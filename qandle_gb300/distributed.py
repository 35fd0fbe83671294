"""Data-parallel training and inference over several GPUs.

Samples of a batch are independent, so the forward shards by batch with no
exchange: rank r evaluates rows ``shard_range(batch, r, world)`` of its
inputs on its own GPU.  The adjoint backward needs exactly one exchange, a
sum of the parameter gradients (a few hundred floats for the benchmark
circuits), done once per step by :func:`allreduce_gradients` on the default
``torch.distributed`` process group.  Per-sample gradients (named inputs,
input states) stay on the rank that owns the sample.

A loss that is a mean over the whole batch needs each rank's gradient
weighted by its share of the batch before the sum; ``weight`` does that.
"""
from __future__ import annotations

import typing

import torch
import torch.distributed as dist


def shard_range(batch: int, rank: int, world: int) -> typing.Tuple[int, int]:
    """Contiguous, balanced slice [start, stop) of `batch` samples for `rank`
    (the first batch % world ranks take one extra sample)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    if batch < 0:
        raise ValueError("batch must be >= 0")
    base, extra = divmod(batch, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def shard(x: torch.Tensor, rank: int, world: int, dim: int = 0) -> torch.Tensor:
    """The rank's slice of `x` along the batch dimension `dim`."""
    start, stop = shard_range(x.shape[dim], rank, world)
    return x.narrow(dim, start, stop - start)


def allreduce_gradients(params: typing.Iterable[torch.Tensor], weight: float = 1.0, group=None) -> None:
    """Sum ``weight * p.grad`` over the ranks of `group` into every ``p.grad``.

    All gradients travel as one flat buffer (one collective per step).
    Parameters without a gradient contribute zeros, so every rank passes the
    same list.  The buffer has the widest dtype of the parameters (at least
    float32).  Pass ``weight = local_batch / global_batch`` when the loss is
    a mean over the global batch."""
    params = [p for p in params]
    if not params:
        return
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    grads = []
    for p in params:
        g = p.grad if p.grad is not None else torch.zeros_like(p)
        grads.append(g.reshape(-1))
    # one buffer in the widest dtype of the list (float32 at least), so
    # float64 parameters keep their precision through the sum
    dtype = torch.float32
    for p in params:
        dtype = torch.promote_types(dtype, p.dtype)
    flat = torch.cat([g.to(dtype) for g in grads]) * weight
    if world > 1:
        dist.all_reduce(flat, op=dist.ReduceOp.SUM, group=group)
    off = 0
    for p in params:
        k = p.numel()
        g = flat[off:off + k].view_as(p).to(p.dtype)
        if p.grad is None:
            p.grad = g.clone()
        else:
            p.grad.copy_(g)
        off += k
