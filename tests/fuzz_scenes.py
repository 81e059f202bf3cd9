"""Seeded triangle soups for the fuzz parity tests.

Each soup mixes the inputs the frame path treats specially: small and
screen-sized triangles, triangles crossing the near plane (W near 0, so
screen coordinates of +-Inf or NaN reach the bin test), triangles beyond
the far plane, triangles whose screen coordinates leave +-2^14 (the int64
edge path), degenerate triangles (collinear or repeated corners), exact
duplicates (depth ties decided by draw order) and both windings; corner UVs
are negative as well as positive (the wrap and clamp rules of
Texture.Sample).  Everything is generated with the splitmix64 stream of
gorender_gb300.scenes, so x86 and Arm hosts build the same float32 meshes.
"""
from __future__ import annotations

import numpy as np

from gorender_gb300 import scenes
from gorender_gb300.scenes import SplitMix64


def soup(seed: int, n: int = 1500, huge: float = 1000.0, vcolor: bool = False) -> scenes.MeshData:
    """n triangles of mixed kinds; the camera is expected at the origin
    looking along -z (the view volume spans z in [-50, 0])."""
    rng = SplitMix64(seed)
    kind = rng.integers(n, 0, 100)
    tri = np.zeros((n, 3, 3), np.float32)
    for t in range(n):
        k = int(kind[t])
        if k < 40:    # small, in view
            c = rng.uniform(3, -1.0, 1.0) * np.array([2.0, 1.5, 4.0], np.float32) - np.array([0, 0, 5.0], np.float32)
            tri[t] = c + rng.uniform(9, -0.25, 0.25).reshape(3, 3)
        elif k < 58:  # large, across the view
            tri[t] = rng.uniform(9, -1.0, 1.0).reshape(3, 3) * np.array([6.0, 4.0, 5.0], np.float32) \
                - np.array([0, 0, 5.5], np.float32)
        elif k < 72:  # across the near plane, some corners behind the camera
            tri[t] = rng.uniform(9, -1.0, 1.0).reshape(3, 3) * np.array([2.0, 2.0, 2.0], np.float32)
        elif k < 80:  # around the far plane
            tri[t] = rng.uniform(9, -1.0, 1.0).reshape(3, 3) * np.array([20.0, 20.0, 8.0], np.float32) \
                - np.array([0, 0, 50.0], np.float32)
        elif k < 86:  # screen coordinates far beyond 2^14
            tri[t] = rng.uniform(9, -1.0, 1.0).reshape(3, 3) * np.array([huge, huge, 1.0], np.float32) \
                - np.array([0, 0, 2.0], np.float32)
        elif k < 92:  # degenerate: two equal corners, or three collinear ones
            a = rng.uniform(3, -1.5, 1.5) - np.array([0, 0, 4.0], np.float32)
            b = rng.uniform(3, -1.5, 1.5) - np.array([0, 0, 4.0], np.float32)
            tri[t] = np.stack([a, b, b if k % 2 else (a + b) * np.float32(0.5)])
        elif t > 0:   # an exact copy of an earlier triangle: a depth tie
            tri[t] = tri[int(rng.integers(1, 0, t)[0])]
        else:
            tri[t] = rng.uniform(9, -1.0, 1.0).reshape(3, 3) - np.array([0, 0, 4.0], np.float32)
    flip = rng.integers(n, 0, 2).astype(bool)  # both windings
    tri[flip] = tri[flip][:, ::-1]
    pos = np.ones((3 * n, 4), np.float32)
    pos[:, :3] = tri.reshape(-1, 3)
    vidx = np.arange(3 * n, dtype=np.int32).reshape(n, 3)
    nrm = rng.uniform(9 * n, -1.0, 1.0).reshape(3 * n, 3)
    vn = np.ones((3 * n, 4), np.float32)
    vn[:, :3] = nrm
    m = scenes.MeshData(pos=pos, vidx=vidx, vnrm=vn, nidx=vidx.copy(), name=f"soup{seed}")
    m.uv = rng.uniform(6 * n, -2.0, 2.0).reshape(n, 6)
    m.tex = (rng.integers(n, 0, 3) - 1).astype(np.int32)  # -1 nil, 0 image, 1 second texture
    if vcolor:
        m.vcolor = rng.uniform(9 * n, 0.0, 1.0).reshape(3 * n, 3)
    return m


def soup_scene(seed: int, width: int, height: int, flags: int, objects: int = 2, n: int = 1200,
               huge: float = 1000.0, vcolor: bool = False) -> scenes.SceneData:
    """A scene of `objects` soups with seeded transforms, the camera at the
    origin looking along -z, a power-of-two and a non-power-of-two texture."""
    rng = SplitMix64(seed * 7919 + 1)
    objs = []
    for k in range(objects):
        m = soup(seed * 31 + k, n, huge=huge, vcolor=vcolor)
        r = rng.uniform(3, -0.4, 0.4)
        tr = rng.uniform(3, -0.5, 0.5)
        s = float(rng.uniform(1, 0.7, 1.3)[0])
        objs.append(scenes.ObjectData(m, scale=(s, s, s), rotation=tuple(float(x) for x in r),
                                      translation=(float(tr[0]), float(tr[1]), float(tr[2]))))
    tex = [scenes.random_texture(16, 16, seed=seed + 3, scale=2.0),
           scenes.random_texture(13, 7, seed=seed + 4, scale=1.5)]
    cam = scenes.CameraData((0.0, 0.0, 0.0), (0.0, 0.0, -1.0), (0.0, 1.0, 0.0))
    return scenes.SceneData(f"soup{seed}-{width}x{height}", width, height, objs, cam, tex, flags)
