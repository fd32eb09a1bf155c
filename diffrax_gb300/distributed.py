"""Data-parallel batches of trajectories across ranks (one process per GPU).

Trajectories are independent, so a batched solve shards its batch across
ranks with no communication in the forward.  A gradient of a loss summed (or
averaged with the global batch size) over the whole batch is the sum of the
per-rank gradients: the one exchange on the path is a sum of the parameter
gradients dL/dtheta (and of shared args) after the backward -- one all-reduce
of one flat buffer.  Gradients with respect to per-trajectory inputs (y0,
per-trajectory args) stay on the rank that owns the trajectory.

In the reference a vmapped diffeqsolve under jax.grad leaves this to JAX's
sharding; here torch.distributed carries it (NCCL between GPUs, gloo on CPU).
"""
from __future__ import annotations

from typing import Iterable, Optional, Sequence

import torch


def shard_bounds(batch: int, rank: int, world: int) -> tuple[int, int]:
    """[start, stop) of the trajectories rank `rank` of `world` owns: the batch
    split into contiguous shards whose sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} is not in a world of {world}")
    if batch < 0:
        raise ValueError("negative batch")
    base, extra = divmod(batch, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def shard(x: torch.Tensor, rank: int, world: int, dim: int = 0) -> torch.Tensor:
    """This rank's contiguous shard of a batched tensor along `dim`."""
    a, b = shard_bounds(int(x.shape[dim]), rank, world)
    return x.narrow(dim, a, b - a)


def all_reduce_gradients(grads: Sequence[Optional[torch.Tensor]], group=None,
                         average: bool = False) -> None:
    """Sum (or average over ranks) `grads` across the ranks of `group` in place:
    one flat buffer, one all-reduce.  None entries are skipped; every rank
    must pass tensors of the same shapes in the same order."""
    import torch.distributed as dist
    live = [g for g in grads if g is not None]
    if not live or not dist.is_available() or not dist.is_initialized():
        return
    world = dist.get_world_size(group)
    if world == 1:
        return
    dtype = live[0].dtype
    if any(g.dtype != dtype for g in live):
        raise TypeError("all gradients must have one dtype")
    flat = torch.cat([g.reshape(-1) for g in live])
    dist.all_reduce(flat, op=dist.ReduceOp.SUM, group=group)
    if average:
        flat /= world
    off = 0
    for g in live:
        n = g.numel()
        g.copy_(flat[off:off + n].view_as(g))
        off += n


def all_reduce_parameter_grads(params: Iterable[torch.Tensor], group=None,
                               average: bool = False) -> None:
    """all_reduce_gradients over the .grad of `params` (e.g. an MLPField's
    weights and biases after loss.backward())."""
    all_reduce_gradients([p.grad for p in params], group=group, average=average)
