"""Renders a named workload for a fixed number of iterations, for profilers.

    python profile_frames.py --scene heightfield --frames 10 [--autotune]

Scenes: uvsphere (960 tris, 640x360), heightfield (199,712 tris, 1280x720),
icospheres (64 level-5/6 icospheres, 1920x1080), batch (the 256-view
multi-view batch, one CUDA-graph replay per iteration) and diff (forward +
backward of the differentiable icosphere workload, --views views at
512x512).  Frames are issued with gr_draw_async on the context stream; the
process exits non-zero on any error.  Every device buffer comes from the
library (gr_device_alloc), as a host without a CUDA allocator would get it.
"""
from __future__ import annotations

import argparse
import ctypes as C
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from gorender_gb300 import _native as N  # noqa: E402
from gorender_gb300 import renderer as R  # noqa: E402
from gorender_gb300 import scenes  # noqa: E402

SCENES = {
    "uvsphere": scenes.scene_uvsphere_640x360,
    "heightfield": scenes.scene_heightfield_1280x720,
    "icospheres": scenes.scene_icospheres_1920x1080,
}


def run_frames(args):
    sc = SCENES[args.scene]()
    ctx = R.Context(args.device)
    up = R.UploadedScene(ctx, sc)
    if args.autotune:
        N.check(N.lib().gr_context_autotune(ctx.handle, up.items, len(sc.objects), C.byref(up.params)))
    if args.tile or args.slice:
        ctx.set_tuning(args.tile, 0)
        N.check(N.lib().gr_context_set_raster(ctx.handle, args.slice, 0))
    up.draw()  # sizes the buffers (and re-runs on overflow)
    t0 = time.perf_counter()
    for _ in range(args.frames):
        R.draw_async(ctx, up.items, len(sc.objects), up.params)
    ctx.sync()
    dt = time.perf_counter() - t0
    print(f"{sc.name}: {args.frames} frames, {dt * 1e3 / args.frames:.4f} ms/frame (host wall clock), "
          f"{sc.num_triangles * args.frames / dt / 1e6:.1f} Mtris/s, tuning {ctx.tuning()} {ctx.raster()}")
    ctx.close()


def run_batch(args):
    vs = scenes.multiview_batch(256, seed=0)
    ctx = R.Context(args.device)
    if args.tile or args.slice:  # the autotuner's choice for this batch, without running it
        ctx.set_tuning(args.tile, args.bins)
        N.check(N.lib().gr_context_set_raster(ctx.handle, args.slice, 0))
    views, entries, bufs = [], [], []
    for v, sc in enumerate(vs):
        up = R.UploadedScene(ctx, sc)
        rgba = ctx.device_buffer(sc.width * sc.height * 4)
        z = ctx.device_buffer(sc.width * sc.height * 4)
        bufs += [rgba, z]
        views.append((up.params, rgba.ptr, z.ptr))
        entries += [(h, mvp, w, v) for h, (mvp, w) in zip(up.mesh_handles, up.matrices)]
    b = R.Batch(ctx, views, entries, autotune=args.autotune)
    t0 = time.perf_counter()
    for _ in range(args.frames):
        b.run()
    b.sync()
    dt = time.perf_counter() - t0
    print(f"batch of {len(vs)} views: {args.frames} replays, {dt * 1e3 / args.frames:.4f} ms/replay, "
          f"tuning {b.tuning()}")
    b.close()
    for x in bufs:
        x.free()
    ctx.close()


def run_diff(args):
    sc = scenes.diff_scene(views=args.views, size=512, level=6, tex_size=256, seed=0)
    ctx = R.Context(args.device)

    def dev(a):
        a = np.ascontiguousarray(a, np.float32)
        return ctx.device_buffer(a.nbytes).upload(a)

    mesh = ctx.mesh(sc.mesh)
    world, views = R.diff_views(sc)
    d = R.Diff(ctx, mesh, world, views, tex_size=sc.tex.shape[:2])
    npx = sum(w * h for w, h, _, _, _ in views)
    p = [dev(sc.mesh.pos), dev(sc.vcol), dev(sc.tex)]
    target = dev(np.zeros((npx, 4), np.float32))
    g = [ctx.device_buffer(sc.mesh.nv * 16), ctx.device_buffer(sc.mesh.nv * 12), ctx.device_buffer(sc.tex.nbytes)]
    t0 = time.perf_counter()
    loss = 0.0
    for _ in range(args.frames):
        loss = d.forward(p[0].ptr, p[1].ptr, p[2].ptr, sc.light, target.ptr)
        d.backward(*(x.ptr for x in g))
    dt = time.perf_counter() - t0
    print(f"diff {args.views} views: {args.frames} forward+backward, {dt * 1e3 / args.frames:.4f} ms each, "
          f"loss {loss:.6e}")
    d.close()
    for x in p + g + [target]:
        x.free()
    ctx.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scene", default="heightfield", choices=sorted(SCENES) + ["batch", "diff"])
    ap.add_argument("--frames", type=int, default=10)
    ap.add_argument("--views", type=int, default=64, help="views of the diff workload")
    ap.add_argument("--autotune", action="store_true", help="run the library autotuner first")
    ap.add_argument("--tile", type=int, default=0, help="raster tile size (16 or 32; 0 keeps the default)")
    ap.add_argument("--slice", type=int, default=0, help="raster cost per slice (0 keeps the default)")
    ap.add_argument("--bins", type=int, default=0, help="tile bin capacity (0 keeps the default)")
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args()
    from gorender_gb300 import build
    build.build()
    if args.scene == "batch":
        run_batch(args)
    elif args.scene == "diff":
        run_diff(args)
    else:
        run_frames(args)


if __name__ == "__main__":
    main()
