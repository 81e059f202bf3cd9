"""Frames of the reference's own sample models (models/cube.obj with its
cube.mtl and textures-16.png atlas, models/suzanne.obj), vendored unchanged
under tests/golden/reference_models/, drawn the way the reference's viewer
draws them (main.go:186-241): an 800x600 framebuffer, NewRenderer's defaults
(renderer.go:114-145: 45 degree vertical field of view, faces, backface
culling, lighting, clipping and textures on, Gouraud), one NewObject per mesh
(mesh.go:81-89: unit scale, no rotation, no translation), the camera at
(0, 0, 5) looking along -z, and the demo mode's turn of Rotation.Y += 0.01
per frame (main.go:236-240) accumulated in float32."""
import dataclasses
import os

import numpy as np

from gorender_gb300 import loaders, scenes

MODELS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_models")
VIEW_W, VIEW_H = 800, 600  # main.go:17-18 (downscaleFactor 1)


def demo_rotation(frame: int) -> float:
    """Rotation.Y after `frame` demo-mode steps of `+= 0.01` in float32."""
    y = np.float32(0.0)
    step = np.float32(0.01)
    for _ in range(frame):
        y = np.float32(y + step)
    return float(y)


def model_scene(name: str, frame: int = 0, flags: int = scenes.DEFAULT_FLAGS, width: int = VIEW_W,
                height: int = VIEW_H) -> scenes.SceneData:
    meshes, texs = loaders.load_obj(os.path.join(MODELS, name + ".obj"))
    rot = (0.0, demo_rotation(frame), 0.0)
    objs = [scenes.ObjectData(m, rotation=rot) for m in meshes]
    cam = scenes.CameraData((0.0, 0.0, 5.0), (0.0, 0.0, -1.0), (0.0, 1.0, 0.0))
    return scenes.SceneData(f"{name}-{width}x{height}-frame{frame}", width, height, objs, cam, texs, flags,
                            fov_deg=45.0)


def with_flags(sc: scenes.SceneData, flags: int) -> scenes.SceneData:
    return dataclasses.replace(sc, flags=flags)


REFERENCE_MODEL_SCENES = {
    "ref-cube-800x600-frame0": lambda: model_scene("cube", 0),
    "ref-cube-800x600-frame60": lambda: model_scene("cube", 60),
    "ref-cube-800x600-frame60-flat": lambda: model_scene("cube", 60, scenes.DEFAULT_FLAGS | scenes.FLAT_SHADING),
    "ref-cube-800x600-frame157-notex": lambda: model_scene("cube", 157, scenes.DEFAULT_FLAGS & ~scenes.SHOW_TEXTURES),
    "ref-suzanne-800x600-frame0": lambda: model_scene("suzanne", 0),
    "ref-suzanne-800x600-frame60": lambda: model_scene("suzanne", 60),
    "ref-suzanne-800x600-frame30-edges": lambda: model_scene("suzanne", 30, scenes.DEFAULT_FLAGS | scenes.SHOW_EDGES),
    "ref-suzanne-800x600-frame200-nocull": lambda: model_scene("suzanne", 200,
                                                               scenes.DEFAULT_FLAGS & ~scenes.BACKFACE_CULLING),
}
