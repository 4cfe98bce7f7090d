"""View sharding of the batched form across ranks (one process per GPU).

Every rank holds all Gaussians and renders a contiguous share of the views,
balanced by pixel count; its backward yields per-Gaussian gradients for its
views only, and one all-reduce (sum) over the ranks gives the gradients of the
whole batch. The forward needs no exchange at all. A single view is not
sharded: its sort is global over the frame's keys, so more GPUs run replicas.

ShardedStep drives it through the engine: the parameters are broadcast once
from rank 0 when the step is built, each step runs the rank's views through
GaussianEngine.step_async, and the five gradient tensors go through one
all-reduce as one flat bucket (staged through host memory when the process
group's backend is gloo).
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


def allreduce_gradients(tensors, group=None) -> None:
    """Sums per-Gaussian gradient tensors over the ranks of `group`, in place,
    with one all-reduce of their concatenation (one bucket; staged through
    host memory when the backend is gloo and the tensors are on a GPU)."""
    import torch
    import torch.distributed as dist

    flat = torch.cat([t.reshape(-1) for t in tensors])
    host = dist.get_backend(group) == "gloo" and flat.is_cuda
    buf = flat.cpu() if host else flat
    dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
    if host:
        flat.copy_(buf)
    off = 0
    for t in tensors:
        n = t.numel()
        t.copy_(flat[off:off + n].view_as(t))
        off += n


class ShardedStep:
    """One rank's part of a batched training step on the views of `cams`.

    params: the raw parameters (means, log-scales, quaternions, opacity
    logits, SH) as CUDA tensors of this rank's device; rank 0's values are
    broadcast to every rank once, here. settings: GaussianEngine settings.
    step(dL_dimage) takes the whole batch's upstream image gradient (all views
    packed in order, on any device) and returns the whole batch's parameter
    gradients, identical on every rank."""

    def __init__(self, cams: list, params: list, group=None, **settings):
        import torch
        import torch.distributed as dist

        from .engine import GaussianEngine

        self.group = group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)
        self.params = [p.contiguous() for p in params]
        flat = torch.cat([p.reshape(-1) for p in self.params])
        host = dist.get_backend(group) == "gloo"
        buf = flat.cpu() if host else flat
        dist.broadcast(buf, src=0, group=group)  # the Gaussians, once at upload
        if host:
            flat.copy_(buf)
        off = 0
        for p in self.params:
            p.copy_(flat[off:off + p.numel()].view_as(p))
            off += p.numel()
        views = view_shard([c.width * c.height for c in cams], self.rank, self.world)
        self.cams = cams
        self.mine = [cams[v] for v in views]
        px = [c.width * c.height * 3 for c in cams]
        self.slice = slice(sum(px[:views.start]), sum(px[:views.stop]))
        self.grads = [torch.zeros_like(p) for p in self.params]
        self.engine = None
        if self.mine:
            self.engine = GaussianEngine(device=self.params[0].device.index or 0, **settings)
            self.engine.compile_params(*self.params)
            if len(self.mine) == 1:
                self.engine.set_camera(self.mine[0])
            else:
                self.engine.set_views(self.mine)
            self.engine.raster_frame()

    def step(self, dL_dimage):
        """Forward + backward of this rank's views, then one all-reduce."""
        import torch

        if self.engine is not None:
            d = dL_dimage[self.slice].to(self.params[0].device).contiguous()
            self.engine.step_async(d, self.grads, 1)
            self.engine.sync()
        else:
            for g in self.grads:
                g.zero_()
        torch.cuda.synchronize(self.params[0].device)
        allreduce_gradients(self.grads, self.group)
        return self.grads

    def close(self) -> None:
        if self.engine is not None:
            self.engine.close()
            self.engine = None
