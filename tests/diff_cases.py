"""Shared set-up of the differentiable-shading tests: small seeded cases of
the 64-view icosphere workload, visibility from the oracle, and the
comparison metric.

Relative error of a gradient vector g against the FP64 adjoint g64 is
max|g - g64| / max|g64| (the infinity norm of the error over that of the
gradient)."""
import dataclasses

import numpy as np

from gorender_gb300 import scenes
from oracle import oracle

NO_FACE = 0xFFFFFFFF


def small_case(views=3, size=96, level=3, tex_size=32, seed=1):
    return scenes.diff_scene(views=views, size=size, level=level, tex_size=tex_size, seed=seed)


def oracle_views(sc):
    """[(width, height, screen16, mvp16)] and the world matrix, from the oracle's matrix code."""
    fov = oracle.fov_radians(sc.fov_deg)
    obj = scenes.ObjectData(sc.mesh)
    out, world = [], None
    for cam in sc.cameras:
        mvp, world = oracle.object_matrices(obj, cam, sc.width, sc.height, fov)
        out.append((sc.width, sc.height, oracle.screen_matrix(sc.width, sc.height), mvp))
    return out, world


def oracle_ids(sc, pos=None):
    """Per-pixel visible face over all views (view v's faces are v * nf + f), from the
    oracle's raster with the diff views' visibility flags."""
    mesh = sc.mesh if pos is None else dataclasses.replace(sc.mesh, pos=np.asarray(pos, np.float32))
    nf = mesh.nf
    chunks = []
    for v, cam in enumerate(sc.cameras):
        s = scenes.SceneData("diffview", sc.width, sc.height, [scenes.ObjectData(mesh)], cam, [], sc.flags,
                             sc.fov_deg)
        _, _, _, st, ids = oracle.draw_scene(s, face_ids=True)
        assert st == 0
        ids = ids.reshape(-1).astype(np.uint64)
        ids = np.where(ids == NO_FACE, NO_FACE, ids + v * nf).astype(np.uint32)
        chunks.append(ids)
    return np.concatenate(chunks)


def params_of(sc, world, target=False):
    src = sc.target_params if target else {"pos": sc.mesh.pos, "vcol": sc.vcol, "tex": sc.tex,
                                            "light": sc.light}
    return {"pos": src["pos"], "vcol": src["vcol"], "tex": src["tex"], "light": src["light"], "world": world}


def rel_err(g, g64):
    g = np.asarray(g, np.float64).reshape(-1)
    g64 = np.asarray(g64, np.float64).reshape(-1)
    scale = np.abs(g64).max()
    return float(np.abs(g - g64).max() / scale) if scale > 0 else float(np.abs(g).max())
