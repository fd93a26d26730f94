"""Data-parallel replicas of the conv path.

Convolution forward, backward_input and pooling are independent per batch
sample: a replica computes its shard of the batch and nothing is exchanged.
backward_kernel is a sum over the batch, so each replica produces a partial
dW for its shard and the partials are summed across replicas.  The sum is
taken in rank order after an all-gather (not by a reduction tree whose
order depends on the transport), so every replica holds bit-identical dW
and the result does not change from run to run.

One process drives one GPU; on a machine with one GPU per box the replicas
are independent boxes and this exchange is exercised on CPU ranks (gloo).
"""

from __future__ import annotations


def shard(n: int, world: int, rank: int) -> tuple[int, int]:
    """[start, stop) of rank's share of n samples: contiguous, sizes differ
    by at most one, lower ranks take the remainder."""
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def allreduce_fixed_order(t, group=None):
    """Sum of `t` over all ranks, added in rank order 0, 1, ..., world-1."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    parts = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(parts, t.contiguous(), group=group)
    out = parts[0].clone()
    for p in parts[1:]:
        out += p
    return out


def conv2d_backward_kernel_dp(nn, x, w, stride, dy, group=None):
    """dW of conv2d over the whole batch from this rank's shard: `x` and
    `dy` are the full batch as seen by every rank (each rank reads only its
    rows); returns the summed dW, identical on every rank."""
    import numpy as np
    import torch
    import torch.distributed as dist

    rank, world = dist.get_rank(group), dist.get_world_size(group)
    a, b = shard(x.shape[0], world, rank)
    if b > a:
        part = nn.conv2d_backward_kernel(x[a:b], w, stride, dy[a:b])
    else:
        part = np.zeros_like(w) if isinstance(w, np.ndarray) else torch.zeros_like(w)
    is_np = isinstance(part, np.ndarray)
    t = torch.from_numpy(part) if is_np else part
    s = allreduce_fixed_order(t, group)
    return s.numpy() if is_np else s
