"""Renders a named scene for a fixed number of frames (for profilers).

    python -m gorender_gb300.profile --scene heightfield --frames 10

Scenes: uvsphere (960 tris, 640x360), heightfield (199,712 tris, 1280x720),
icospheres (64 level-5/6 icospheres, 1920x1080).  Frames are issued with
gr_draw_async on the context stream; the process exits non-zero on any error.
"""
from __future__ import annotations

import argparse
import time

from . import renderer as R
from . import scenes

SCENES = {
    "uvsphere": scenes.scene_uvsphere_640x360,
    "heightfield": scenes.scene_heightfield_1280x720,
    "icospheres": scenes.scene_icospheres_1920x1080,
}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scene", default="heightfield", choices=sorted(SCENES))
    ap.add_argument("--frames", type=int, default=10)
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args()
    sc = SCENES[args.scene]()
    ctx = R.Context(args.device)
    up = R.UploadedScene(ctx, sc)
    up.draw()  # sizes the buffers (and re-runs on overflow)
    t0 = time.perf_counter()
    for _ in range(args.frames):
        R.draw_async(ctx, up.items, len(sc.objects), up.params)
    ctx.sync()
    dt = time.perf_counter() - t0
    print(f"{sc.name}: {args.frames} frames, {dt * 1e3 / args.frames:.4f} ms/frame (host wall clock), "
          f"{sc.num_triangles * args.frames / dt / 1e6:.1f} Mtris/s")
    ctx.close()


if __name__ == "__main__":
    main()
