"""GPU parity of the frame's post effects: FrameBuffer.Fog (rasterizer.go:
193-207) standalone (gr_fog) and fused into the raster write-back
(gr_context_set_fog), and FrameBuffer.CrossHair (rasterizer.go:209-217,
drawn when the reference's demoMode is off) — bit for bit against the oracle."""
import dataclasses

import numpy as np
import pytest

import gorender_gb300 as gr
from gorender_gb300 import renderer as R
from gorender_gb300 import scenes
from oracle import oracle

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

FOG = (0.100, 0.033, (100, 100, 100, 255))  # the reference's commented-out call, renderer.go:479


@pytest.fixture(scope="module")
def ctx():
    c = gr.Context(0)
    yield c
    c.close()


def _oracle(scene, up, flags=None):
    rgba, z, tpf, st = oracle.draw_scene(scene, items_override=up.matrices, flags=flags, nthreads=4)
    assert st == 0
    return rgba, z


def _fog_scene():
    # z spans the fog range: an icosphere at distance ~12 (zRec ~ 1/12 .. 1/9)
    m = scenes.icosphere(3, noise=0.05, seed=2)
    objs = [scenes.ObjectData(m, scale=(3.0, 3.0, 3.0))]
    cam = scenes.CameraData((0.0, 0.0, 12.0), (0.0, 0.0, -1.0), (0.0, 1.0, 0.0))
    return scenes.SceneData("fog", 321, 203, objs, cam, [], scenes.DEFAULT_FLAGS)


def test_fog_standalone_matches_oracle(ctx):
    sc = _fog_scene()
    up = gr.UploadedScene(ctx, sc)
    rgba = torch.zeros((sc.height, sc.width, 4), dtype=torch.uint8, device="cuda")
    z = torch.zeros((sc.height, sc.width), dtype=torch.float32, device="cuda")
    up.draw(rgba.data_ptr(), z.data_ptr())
    ctx.fog(rgba.data_ptr(), z.data_ptr(), sc.width, sc.height, *FOG)
    ref_rgba, ref_z = _oracle(sc, up)
    ref = oracle.fog(ref_rgba, ref_z, *FOG)
    got = rgba.cpu().numpy()
    assert np.array_equal(got, ref)
    assert not np.array_equal(ref, ref_rgba)  # the fog changed something


@pytest.mark.parametrize("flags_extra", [0, R.CROSSHAIR, R.CROSSHAIR | gr.SHOW_EDGES | gr.SHOW_VERTICES])
def test_fog_fused_matches_draw_then_fog(flags_extra):
    ctx = gr.Context(0)
    try:
        sc = _fog_scene()
        sc = dataclasses.replace(sc, flags=sc.flags | flags_extra)
        ctx.set_fog(True, *FOG)
        up = gr.UploadedScene(ctx, sc)
        rgba, z, _ = up.render()
        ref_rgba, ref_z = _oracle(sc, up)
        assert np.array_equal(z.view(np.uint32), ref_z.view(np.uint32))
        assert np.array_equal(rgba, oracle.fog(ref_rgba, ref_z, *FOG))
        ctx.set_fog(False)
        rgba2, _, _ = up.render()
        assert np.array_equal(rgba2, ref_rgba)
    finally:
        ctx.close()


@pytest.mark.parametrize("size", [(640, 360), (9, 7), (12, 5), (33, 21)])
def test_crosshair_matches_oracle(ctx, size):
    sc = scenes.scene_uvsphere_640x360()
    sc = dataclasses.replace(sc, width=size[0], height=size[1], flags=sc.flags | R.CROSSHAIR)
    up = gr.UploadedScene(ctx, sc)
    rgba, z, _ = up.render()
    ref_rgba, ref_z = _oracle(sc, up)
    assert np.array_equal(rgba, ref_rgba)
    assert np.array_equal(z.view(np.uint32), ref_z.view(np.uint32))
    assert ((rgba[..., 0] == 255) & (rgba[..., 1] == 255) & (rgba[..., 2] == 0)).any()


def test_renderer_fog(ctx):
    sc = _fog_scene()
    r = gr.Renderer(ctx, sc.width, sc.height)
    mesh = ctx.mesh(sc.objects[0].mesh)
    r.set_fov(gr.fov_radians(60.0))
    o = gr.Object(mesh, scale=sc.objects[0].scale)
    cam = gr.Camera(sc.camera.position, sc.camera.direction, sc.camera.up)
    r.draw([o], cam)
    before = r.pixels()
    r.fog(*FOG)
    ref = oracle.fog(before, r.zbuffer(), *FOG)
    assert np.array_equal(r.pixels(), ref)


def test_unknown_flag_bits_rejected(ctx):
    sc = scenes.scene_uvsphere_640x360()
    for bad in (0x200, 0x80000000):
        up = gr.UploadedScene(ctx, dataclasses.replace(sc, flags=sc.flags | bad))
        with pytest.raises(gr.GrError) as e:
            up.render()
        assert e.value.code == R.N.GR_ERR_INVALID_ARGUMENT
