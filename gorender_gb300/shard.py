"""Sharding a batch of views across GPUs: one process per GPU, no collective.

The reference parallelises one frame inside one process: one projection task
per object and one raster task per screen tile (renderer.go:451-473).  Here a
single frame stays on one GPU (it takes 0.13 ms; splitting it would need an
exchange of binned triangles between GPUs), so N GPUs render N independent
replicas of it; a batch of views is what shards: every view is independent,
so each rank renders its own subset of the views as one CUDA-graph batch on
its own GPU.  Nothing crosses between ranks but a barrier and the maximum of
the timed durations (the caller's process group).

Partition: views are dealt to ranks by estimated cost, largest first, each to
the rank with the least cost so far (ties: lowest rank), which keeps the
ranks within one view's cost of each other.  The cost of a view is estimated
as its submitted faces plus PIXEL_COST times its pixels (a pixel's clear,
depth resolve and shading against a face's transform, clip, set-up and
binning).
"""
from __future__ import annotations

import os
from typing import List, Sequence, Tuple

import numpy as np

from . import renderer as R
from .scenes import SceneData

PIXEL_COST = 0.25  # cost of a framebuffer pixel relative to a submitted face


def dist_env() -> Tuple[int, int, int]:
    """(world size, rank, local rank) from the launcher's environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", os.environ.get("RANK", "0"))))


def view_cost(scene: SceneData) -> float:
    return float(scene.num_triangles) + PIXEL_COST * scene.width * scene.height


def partition_views(costs: Sequence[float], world_size: int) -> List[List[int]]:
    """Indices of the views each rank renders (each list in view order).  Every
    view goes to exactly one rank; deterministic for given costs."""
    if world_size < 1:
        raise ValueError("world_size must be at least 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    load = [0.0] * world_size
    parts: List[List[int]] = [[] for _ in range(world_size)]
    for i in order:
        r = min(range(world_size), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += float(costs[i])
    return [sorted(p) for p in parts]


def shard_of(scenes: Sequence[SceneData], rank: int, world_size: int) -> List[int]:
    return partition_views([view_cost(s) for s in scenes], world_size)[rank]


class ShardedBatch:
    """The views of ``scenes`` listed in ``indices`` (this rank's share),
    rendered as one autotuned CUDA-graph batch on ``ctx``'s GPU into device
    buffers owned through the library."""

    def __init__(self, ctx: R.Context, scenes: Sequence[SceneData], indices: Sequence[int], autotune: bool = True):
        self.ctx = ctx
        self.indices = list(indices)
        self.scenes = [scenes[i] for i in self.indices]
        self.uploads, self.outputs = [], []
        views, entries = [], []
        for v, sc in enumerate(self.scenes):
            up = R.UploadedScene(ctx, sc)
            rgba = ctx.device_buffer(sc.width * sc.height * 4)
            z = ctx.device_buffer(sc.width * sc.height * 4)
            self.uploads.append(up)
            self.outputs.append((rgba, z))
            views.append((up.params, rgba.ptr, z.ptr))
            entries += [(h, mvp, w, v) for h, (mvp, w) in zip(up.mesh_handles, up.matrices)]
        self.batch = R.Batch(ctx, views, entries, autotune=autotune) if views else None

    @property
    def faces(self) -> int:
        return sum(s.num_triangles for s in self.scenes)

    def run(self):
        if self.batch:
            self.batch.run()

    def sync(self):
        if self.batch:
            self.batch.sync()

    def view_tpf(self) -> List[int]:
        return self.batch.view_tpf() if self.batch else []

    def frame(self, k: int) -> Tuple[np.ndarray, np.ndarray]:
        """RGBA8 and z-buffer of this rank's k-th view (host copies)."""
        sc = self.scenes[k]
        rgba, z = self.outputs[k]
        return rgba.download((sc.height, sc.width, 4), np.uint8), z.download((sc.height, sc.width), np.float32)

    def close(self):
        if self.batch:
            self.batch.close()
            self.batch = None
        for rgba, z in self.outputs:
            rgba.free()
            z.free()
        self.outputs = []


def allreduce_host(dist):
    """A sum over ranks of host arrays, in place, through a torch.distributed
    process group (gloo or any backend that takes CPU tensors)."""
    import torch

    def reduce(arrays):
        for a in arrays:
            t = torch.from_numpy(a)
            dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return reduce


class ShardedDiff:
    """The differentiable forward and backward of one mesh over many views,
    the views dealt across ranks (one process per GPU).

    The loss is a sum over views and pixels, so it and every gradient (vertex
    positions and colours, texels, the light) are sums of the ranks' shares:
    each rank differentiates its own views and one sum over ranks of its
    loss and gradients gives the whole step's -- the only data that crosses
    between GPUs (16 + 12 bytes a vertex, 16 a texel, 32 for the light and
    the loss).  ``views`` is the full list of ``renderer.diff_views``;
    ``indices`` this rank's share (``partition_views`` of equal costs).
    Parameters and targets are device buffers of the rank's context; the
    target holds the pixels of this rank's views only, in their order."""

    def __init__(self, ctx: R.Context, mesh: int, world, views, indices: Sequence[int],
                 tex_size: Tuple[int, int] = (0, 0)):
        self.ctx = ctx
        self.indices = list(indices)
        self.views = [views[i] for i in self.indices]
        self.pixels = sum(w * h for w, h, _, _, _ in self.views)
        self.diff = R.Diff(ctx, mesh, world, self.views, tex_size=tex_size) if self.views else None

    def forward(self, pos, vcol, tex, light, target, image=None) -> float:
        """This rank's share of the loss (device pointers as in Diff.forward)."""
        return self.diff.forward(pos, vcol, tex, light, target, image) if self.diff else 0.0

    def step(self, pos, vcol, tex, light, target, grads, shapes, allreduce):
        """Forward + backward of this rank's views, then the sum over ranks:
        returns (loss, light gradient, [position, colour, texel gradients])
        of the whole step as host arrays; ``grads`` are this rank's device
        gradient buffers and ``shapes`` their (shape, dtype)."""
        loss = np.array([self.forward(pos, vcol, tex, light, target)], np.float64)
        if self.diff:
            g_light = np.asarray(self.diff.backward(*(int(g) for g in grads)), np.float64).reshape(3)
            host = [R.DeviceBuffer.download_from(self.ctx, g, shape, dtype) for g, (shape, dtype) in zip(grads, shapes)]
        else:
            g_light = np.zeros(3, np.float64)
            host = [np.zeros(shape, dtype) for shape, dtype in shapes]
        allreduce([loss, g_light] + host)
        return float(loss[0]), g_light, host

    def close(self):
        if self.diff:
            self.diff.close()
            self.diff = None
