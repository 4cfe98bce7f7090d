"""View sharding of the batched form across ranks (one process per GPU).

Every rank holds all Gaussians and renders a contiguous share of the views,
balanced by pixel count; its backward yields per-Gaussian gradients for its
views only, and one all-reduce (sum) over the ranks gives the gradients of the
whole batch. The forward needs no exchange at all. A single view is not
sharded: its sort is global over the frame's keys, so more GPUs run replicas.
"""
from __future__ import annotations


def view_shard(pixels_per_view: list[int], rank: int, world: int) -> range:
    """Contiguous views of `rank`: the cut points split the cumulative pixel
    count into `world` nearly equal parts (every view goes to exactly one rank;
    a rank may get none when there are fewer views than ranks)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    total = sum(pixels_per_view)
    cuts = [0]
    acc, v = 0, 0
    for r in range(1, world):
        target = total * r / world
        while v < len(pixels_per_view) and acc + pixels_per_view[v] / 2 <= target:
            acc += pixels_per_view[v]
            v += 1
        cuts.append(v)
    cuts.append(len(pixels_per_view))
    return range(cuts[rank], cuts[rank + 1])


def shard_cameras(cams: list, rank: int, world: int) -> list:
    """The cameras rank `rank` renders."""
    r = view_shard([c.width * c.height for c in cams], rank, world)
    return [cams[i] for i in r]


def allreduce_gradients(grads, group=None) -> None:
    """Sums per-Gaussian gradient tensors over the ranks of `group`, in place."""
    import torch.distributed as dist

    for g in grads:
        dist.all_reduce(g, op=dist.ReduceOp.SUM, group=group)
