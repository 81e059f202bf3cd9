"""The host loaders (OBJ/MTL, scene manifests, PNG textures) against the
reference's behaviour, on hand-written fixtures (CPU only)."""
import json
import os

import numpy as np
import pytest

from gorender_gb300 import loaders
from tests import png_writer

REF_MODELS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_models")


# ---- numbers: strconv.ParseFloat(s, 32) ----

@pytest.mark.parametrize("text,bits", [
    ("0.1", 0x3DCCCCCD),
    ("1.000000", 0x3F800000),
    ("-2.5e-3", 0xBB23D70A),
    ("16777217", 0x4B800000),   # tie between 2^24 and 2^24 + 2: the even one
    ("16777219", 0x4B800002),   # tie between 2^24 + 2 and 2^24 + 4: the even one
    # just above the midpoint of 1 and 1 + 2^-23: a double rounds it onto the
    # midpoint (then to 1.0 by ties-to-even); the correct float32 is 1 + 2^-23
    ("1.000000059604644775390625000000001", 0x3F800001),
])
def test_parse_float32(text, bits):
    assert int(loaders.parse_float32(text).view(np.uint32)) == bits


# ---- PNG ----

RNG = np.random.default_rng(5)


@pytest.mark.parametrize("ct,depth", [(0, 1), (0, 2), (0, 4), (0, 8), (0, 16), (2, 8), (2, 16), (3, 1), (3, 2),
                                      (3, 4), (3, 8), (4, 8), (4, 16), (6, 8), (6, 16)])
@pytest.mark.parametrize("interlace", [False, True])
def test_png_round_trip_samples(ct, depth, interlace):
    h, w = 13, 11
    ch = png_writer.CHANNELS[ct]
    s = RNG.integers(0, 1 << depth, (h, w, ch))
    pal = None
    if ct == 3:
        pal = RNG.integers(0, 256, (1 << depth, 3))
    data = png_writer.encode(s, ct, depth, palette=pal, interlace=interlace)
    out = loaders.decode_png(data)
    # expected: Go's color.RGBAModel of the decoded image
    if ct == 0:
        y = s[..., 0] * {1: 255, 2: 85, 4: 17, 8: 1}[depth] if depth <= 8 else s[..., 0] >> 8
        exp = np.stack([y, y, y, np.full_like(y, 255)], -1)
    elif ct == 2:
        exp = np.concatenate([s if depth == 8 else s >> 8, np.full((h, w, 1), 255)], -1)
    elif ct == 3:
        exp = np.concatenate([pal[s[..., 0]], np.full((h, w, 1), 255)], -1)
    elif ct == 4:
        if depth == 8:
            y = ((s[..., 0] * 257 * s[..., 1]) // 255) >> 8
            exp = np.stack([y, y, y, s[..., 1]], -1)
        else:
            y = ((s[..., 0] * s[..., 1]) // 65535) >> 8
            exp = np.stack([y, y, y, s[..., 1] >> 8], -1)
    else:
        if depth == 8:
            c = ((s[..., :3] * 257 * s[..., 3:]) // 255) >> 8
            exp = np.concatenate([c, s[..., 3:]], -1)
        else:
            c = ((s[..., :3] * s[..., 3:]) // 65535) >> 8
            exp = np.concatenate([c, s[..., 3:] >> 8], -1)
    assert np.array_equal(out, exp.astype(np.uint8))


def test_png_premultiply_hand_computed():
    # NRGBA (200, 100, 50, 128): 200*257*128//255 = 25800 -> 25800 >> 8 = 100;
    # 100*257*128//255 = 12900 -> 50; 50*257*128//255 = 6450 -> 25
    s = np.array([[[200, 100, 50, 128], [10, 20, 30, 0], [1, 2, 3, 255]]])
    out = loaders.decode_png(png_writer.encode(s, 6, 8))
    assert out[0].tolist() == [[100, 50, 25, 128], [0, 0, 0, 0], [1, 2, 3, 255]]


def test_png_palette_with_transparency_and_short_palette():
    s = np.array([[[0], [1], [3]]])  # index 3 is past a 2-entry palette: opaque black
    data = png_writer.encode(s, 3, 8, palette=[[200, 100, 50], [9, 9, 9]], trns=bytes([128]))
    out = loaders.decode_png(data)
    assert out[0].tolist() == [[100, 50, 25, 128], [9, 9, 9, 255], [0, 0, 0, 255]]


def test_png_rgb_transparent_key():
    s = np.array([[[1, 2, 3], [4, 5, 6]]])
    out = loaders.decode_png(png_writer.encode(s, 2, 8, trns=bytes([0, 4, 0, 5, 0, 6])))
    assert out[0].tolist() == [[1, 2, 3, 255], [0, 0, 0, 0]]


def test_png_bad_crc_rejected():
    data = bytearray(png_writer.encode(np.zeros((2, 2, 4), np.int64), 6, 8))
    data[-13] ^= 1  # inside the IDAT body
    with pytest.raises(ValueError):
        loaders.decode_png(bytes(data))


# ---- OBJ / MTL ----

def _write(path, text):
    with open(path, "w") as f:
        f.write(text)


@pytest.fixture
def objdir(tmp_path):
    tex = RNG.integers(0, 256, (4, 8, 4))
    (tmp_path / "t.png").write_bytes(png_writer.encode(tex, 6, 8))
    _write(tmp_path / "m.mtl", "newmtl A\nmap_Kd t.png\n\nnewmtl B\nKd 1 1 1\nnewmtl C\nmap_Kd t.png\n")
    _write(tmp_path / "two.obj", """# two objects
mtllib m.mtl
o First
v 0 0 0
v 1 0 0
v 0 1 0
v 0.1 0.2 0.3
vt 0.25 0.5
vt 0.75 0.5
vt 0.5 1
vn 0 0 1
vn 0 1 0
usemtl A
f 1/1/1 2/2/1 3/3/2
usemtl B
f 1/1 2/2 4/3
usemtl nothing
f 1 3 4
o Second
v 0 0 1
v 1 0 1
v 0 1 1
vt 0 0
vn 1 0 0
vn 0 1 0
vn 0 0 1
usemtl C
f 5//3 6//4 7//5
""")
    return tmp_path, tex


def test_obj_two_objects_offsets_materials(objdir):
    d, tex = objdir
    meshes, texs = loaders.load_obj(str(d / "two.obj"))
    assert len(meshes) == 2
    a, b = meshes
    assert a.nv == 4 and a.nf == 3 and b.nv == 3 and b.nf == 1
    assert a.vidx.tolist() == [[0, 1, 2], [0, 1, 3], [0, 2, 3]]
    assert a.nidx.tolist() == [[0, 0, 1], [0, 0, 0], [0, 0, 0]]
    assert np.allclose(a.uv[0], [0.25, 0.5, 0.75, 0.5, 0.5, 1.0])
    assert np.allclose(a.uv[2], 0.0)
    # materials: A -> the PNG, B (no map_Kd) -> solid magenta, unknown -> none;
    # C names the same file as A: loaded once
    assert texs[a.tex[0]].kind == 2 and texs[a.tex[0]].pixels.shape == (4, 8, 4)
    assert texs[a.tex[1]].kind == 0 and texs[a.tex[1]].color == (255, 0, 255, 255)
    assert a.tex[2] == -1
    assert b.tex[0] == a.tex[0]
    # the second object's indices are relative to the vertices read so far;
    # v//vn keeps the reference's scan of the third normal into the second slot
    assert b.vidx.tolist() == [[0, 1, 2]]
    assert b.nidx.tolist() == [[0, 2, -3]]
    assert b.vnrm.shape == (3, 4) and (b.vnrm[:, 3] == 1).all()
    fixed, _ = loaders.load_obj(str(d / "two.obj"), fix_normal_indices=True)
    assert fixed[1].nidx.tolist() == [[0, 1, 2]]


def test_obj_single_mesh_and_errors(objdir, tmp_path):
    d, _ = objdir
    meshes, _ = loaders.load_obj(str(d / "two.obj"), single_mesh=True)
    assert len(meshes) == 1 and meshes[0].nv == 7 and meshes[0].nf == 4
    _write(tmp_path / "quad.obj", "v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nf 1 2 3 4\n")
    with pytest.raises(ValueError, match="not triangulated"):
        loaders.load_obj(str(tmp_path / "quad.obj"))
    _write(tmp_path / "empty.obj", "# nothing\n")
    with pytest.raises(ValueError, match="vertices"):
        loaders.load_obj(str(tmp_path / "empty.obj"))
    _write(tmp_path / "bad.obj", "v 0 0 0\nf 1 2 3\n")
    with pytest.raises(ValueError, match="out of range"):
        loaders.load_obj(str(tmp_path / "bad.obj"))


# ---- scene manifests ----

def test_scene_manifest(objdir):
    d, _ = objdir
    _write(d / "scene.json", json.dumps({
        "name": "demo",
        "meshes": [{"id": "a", "objFile": "two.obj", "texture": "t.png", "textureScale": 4},
                   {"ID": "b", "objfile": "two.obj"}],
        "objects": [{"meshID": "a", "position": [1, 2, 3], "rotation": [90, 0, 45], "scale": [1, 1, 1]},
                    {"meshid": "b", "position": [0, 0, 0.1], "rotation": [0, 180, 0], "scale": [2, 2, 2]}],
    }))
    ls = loaders.load_scene(str(d / "scene.json"))
    assert ls.name == "demo" and len(ls.objects) == 2
    a, b = ls.objects
    # single-mesh load of the whole file; every face takes the manifest's texture
    assert a.mesh.nf == 4 and (a.mesh.tex == a.mesh.tex[0]).all()
    ta, tb = ls.textures[a.mesh.tex[0]], ls.textures[b.mesh.tex[0]]
    assert ta.kind == 2 and ta.scale == 4.0
    assert tb.kind == 0 and tb.color == (200, 200, 200, 255)
    # degrees -> radians as float32(deg) * float32(pi32 / 180)
    f = np.float32(np.float32(np.pi) / np.float32(180))
    assert np.float32(a.rotation[0]) == np.float32(np.float32(90) * f)
    assert np.float32(b.rotation[1]) == np.float32(np.float32(180) * f)
    assert b.translation == (0.0, 0.0, float(np.float32(0.1)))


def test_scene_unknown_mesh(objdir):
    d, _ = objdir
    _write(d / "bad.json", json.dumps({"meshes": [], "objects": [{"meshID": "zz"}]}))
    with pytest.raises(ValueError, match="mesh id not found"):
        loaders.load_scene(str(d / "bad.json"))


def test_reference_sample_models_load():
    meshes, texs = loaders.load_obj(os.path.join(REF_MODELS, "cube.obj"))
    assert len(meshes) == 1 and meshes[0].nv == 8 and meshes[0].nf == 12
    assert len(texs) == 1 and texs[0].kind == 2 and texs[0].pixels.shape == (512, 512, 4)
    # premultiplied: no colour channel above its alpha
    px = texs[0].pixels.astype(int)
    assert (px[..., :3] <= px[..., 3:]).all()
    meshes, texs = loaders.load_obj(os.path.join(REF_MODELS, "suzanne.obj"))
    assert meshes[0].nv == 507 and meshes[0].nf == 967 and texs == []


def test_jpeg_texture_rejected_clearly(tmp_path):
    p = tmp_path / "t.jpg"
    p.write_bytes(b"\xff\xd8\xff\xe0" + bytes(60))
    with pytest.raises(ValueError, match="JPEG"):
        loaders.load_texture(str(p))
