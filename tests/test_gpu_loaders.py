"""A scene read by the host loaders (manifest + OBJ/MTL + a PNG texture with
alpha, premultiplied as the reference loads it) renders on the GPU bit for
bit like the oracle."""
import json

import numpy as np
import pytest

import gorender_gb300 as gr
from gorender_gb300 import loaders, scenes
from tests import png_writer
from tests.test_gpu_parity import compare

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = gr.Context(0)
    yield c
    c.close()


def test_loaded_manifest_scene(ctx, tmp_path):
    rng = np.random.default_rng(11)
    (tmp_path / "tex.png").write_bytes(png_writer.encode(rng.integers(0, 256, (16, 16, 4)), 6, 8, interlace=True))
    (tmp_path / "odd.png").write_bytes(png_writer.encode(rng.integers(0, 256, (10, 12, 3)), 2, 8))
    sphere = scenes.icosphere(3, noise=0.05, seed=4)
    uv = scenes.spherical_uvs(sphere)
    lines = ["mtllib m.mtl", "o ball"]
    lines += [f"v {x:.6f} {y:.6f} {z:.6f}" for x, y, z in sphere.pos[:, :3]]
    lines += [f"vt {u:.6f} {v:.6f}" for u, v in uv.reshape(-1, 2)]
    lines += [f"vn {x:.4f} {y:.4f} {z:.4f}" for x, y, z in sphere.vnrm[:, :3]]
    lines.append("usemtl A")
    for f, (a, b, c) in enumerate(sphere.vidx + 1):
        t = 3 * f + 1
        lines.append(f"f {a}/{t}/{a} {b}/{t + 1}/{b} {c}/{t + 2}/{c}")
    (tmp_path / "ball.obj").write_text("\n".join(lines) + "\n")
    (tmp_path / "m.mtl").write_text("newmtl A\nmap_Kd tex.png\n")
    (tmp_path / "scene.json").write_text(json.dumps({
        "name": "loaded",
        "meshes": [{"id": "ball", "objFile": "ball.obj"},
                   {"id": "ball2", "objFile": "ball.obj", "texture": "odd.png", "textureScale": 3}],
        "objects": [{"meshID": "ball", "position": [-1.2, 0, 0], "rotation": [10, 20, 30], "scale": [1, 1, 1]},
                    {"meshID": "ball2", "position": [1.2, 0, 0], "rotation": [0, 45, 0], "scale": [1, 1, 1]}]}))
    ls = loaders.load_scene(str(tmp_path / "scene.json"))
    cam = scenes.CameraData((0.0, 0.5, 5.0), (0.0, -0.1, -1.0), (0.0, 1.0, 0.0))
    for flags in (scenes.DEFAULT_FLAGS, scenes.DEFAULT_FLAGS | scenes.FLAT_SHADING):
        sc = ls.scene(400, 240, cam, flags=flags)
        rgba, z, tpf = compare(ctx, sc)
        assert tpf > 0 and (z > -1).sum() > 5000
    # the OBJ's own material (the interlaced PNG) through load_obj directly
    meshes, texs = loaders.load_obj(str(tmp_path / "ball.obj"))
    sc = scenes.SceneData("obj", 320, 200, [scenes.ObjectData(meshes[0])], cam, texs, scenes.DEFAULT_FLAGS)
    compare(ctx, sc)


from tests.reference_models import REFERENCE_MODEL_SCENES  # noqa: E402


@pytest.mark.parametrize("name", sorted(REFERENCE_MODEL_SCENES))
def test_reference_sample_models(ctx, name):
    """The reference's own cube (textured from its 512x512 atlas) and Suzanne,
    drawn as its viewer draws them, bit for bit against the oracle."""
    sc = REFERENCE_MODEL_SCENES[name]()
    rgba, z, tpf = compare(ctx, sc)
    assert tpf > 0 and (z > -1).sum() > 40000
