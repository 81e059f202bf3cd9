"""Small seeded scenes shared by the golden fixtures and the GPU parity tests."""
import dataclasses

import numpy as np

from gorender_gb300 import scenes
from tests.reference_models import REFERENCE_MODEL_SCENES


def uvsphere():
    return scenes.scene_uvsphere_640x360()


def heightfield_small():
    sc = scenes.scene_heightfield_1280x720(n=97)
    return dataclasses.replace(sc, width=320, height=180)


def icospheres_small():
    sc = scenes.scene_icospheres_1920x1080(count=6, levels=(2, 3))
    return dataclasses.replace(sc, width=320, height=240)


def textures_mixed():
    m = scenes.heightfield(33, extent=1.5, seed=3)
    tex_img = scenes.random_texture(12, 10, seed=5, scale=3.0)
    solid = scenes.TextureData.solid((10, 200, 30, 255))
    m.tex = (np.arange(m.nf) % 3 - 1).astype(np.int32)
    cam = scenes.CameraData((0.0, 0.6, 1.8), (0.0, -0.5, -1.0), (0.0, 1.0, 0.0))
    return scenes.SceneData("textures-mixed", 160, 120, [scenes.ObjectData(m)], cam, [tex_img, solid],
                            scenes.DEFAULT_FLAGS | scenes.FLAT_SHADING)


def inside_sphere():
    # winding flipped so the faces point inward: seen from the camera inside,
    # they are front-facing and every one crosses or nears the near plane
    m = scenes.icosphere(3)
    m = dataclasses.replace(m, vidx=np.ascontiguousarray(m.vidx[:, [0, 2, 1]]),
                            nidx=np.ascontiguousarray(m.nidx[:, [0, 2, 1]]))
    return scenes.SceneData("inside", 160, 120, [scenes.ObjectData(m, scale=(2.0, 2.0, 2.0))],
                            scenes.CameraData((0.1, 0.2, 0.3), (0.3, -0.2, -1.0), (0.0, 1.0, 0.0)), [],
                            scenes.DEFAULT_FLAGS & ~scenes.BACKFACE_CULLING)


def overlays_uvsphere():
    sc = scenes.scene_uvsphere_640x360()
    return dataclasses.replace(sc, name="overlays", width=320, height=180,
                               flags=sc.flags | scenes.SHOW_EDGES | scenes.SHOW_VERTICES)


def overlays_wire_heightfield():
    # ShowFaces off: white edges only, no fills, no centroid marks
    sc = heightfield_small()
    return dataclasses.replace(sc, name="wire", flags=(sc.flags | scenes.SHOW_EDGES) & ~scenes.SHOW_FACES)


GOLDEN_SCENES = {
    "uvsphere960-640x360": uvsphere,
    "heightfield97-320x180": heightfield_small,
    "icospheres6-320x240": icospheres_small,
    "textures-mixed-160x120": textures_mixed,
    "inside-sphere-160x120": inside_sphere,
    "overlays-uvsphere-320x180": overlays_uvsphere,
    "wire-heightfield97-320x180": overlays_wire_heightfield,
}
GOLDEN_SCENES.update(REFERENCE_MODEL_SCENES)
