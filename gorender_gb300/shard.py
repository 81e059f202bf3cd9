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
