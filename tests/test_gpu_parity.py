"""GPU parity: the CUDA frame pipeline against the CPU oracle, through the C-ABI.

Framebuffer (RGBA8) and z-buffer (float32 bit patterns) must be identical,
and TPF (binned triangles) must match.  Inputs are seeded synthetic scenes
small enough for the oracle to finish in seconds.
"""
import dataclasses

import numpy as np
import pytest

import gorender_gb300 as gr
from gorender_gb300 import renderer as R
from gorender_gb300 import scenes
from oracle import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = gr.Context(0)
    yield c
    c.close()


def compare(ctx, scene, flags=None, light=None):
    """Render scene on the GPU and with the oracle using the same matrices."""
    if flags is not None:
        scene = dataclasses.replace(scene, flags=flags)
    up = gr.UploadedScene(ctx, scene)
    if light is not None:
        up.params = gr.make_params(scene.width, scene.height, scene.flags, light)
    rgba, z, tpf = up.render()
    ref_rgba, ref_z, ref_tpf, st = oracle.draw_scene(scene, items_override=up.matrices,
                                                     light=light, nthreads=4)
    assert st == 0
    diff = (rgba != ref_rgba).any(axis=2)
    zdiff = z.view(np.uint32) != ref_z.view(np.uint32)
    assert tpf == ref_tpf, f"TPF {tpf} vs oracle {ref_tpf}"
    assert not diff.any(), f"{int(diff.sum())} RGBA pixels differ, first at {np.argwhere(diff)[:5].tolist()}"
    assert not zdiff.any(), f"{int(zdiff.sum())} z values differ, first at {np.argwhere(zdiff)[:5].tolist()}"
    return rgba, z, tpf


def test_uvsphere_gouraud(ctx):
    rgba, z, tpf = compare(ctx, scenes.scene_uvsphere_640x360())
    assert (z > -1).sum() > 10000


@pytest.mark.parametrize("flags", [
    gr.FLAGS_DEFAULT,
    gr.FLAGS_DEFAULT & ~gr.BACKFACE_CULLING,
    gr.FLAGS_DEFAULT & ~gr.LIGHTING,
    gr.FLAGS_DEFAULT | gr.FLAT_SHADING,
    gr.FLAGS_DEFAULT & ~gr.FRUSTUM_CLIPPING,
    gr.FLAGS_DEFAULT & ~gr.SHOW_FACES,
])
def test_uvsphere_flags(ctx, flags):
    sc = scenes.scene_uvsphere_640x360()
    compare(ctx, sc, flags=flags)


def test_heightfield_textured_clipped(ctx):
    rgba, z, tpf = compare(ctx, scenes.scene_heightfield_1280x720())
    assert (z > -1).sum() > 100000


def test_heightfield_small_textures_off(ctx):
    sc = scenes.scene_heightfield_1280x720(n=97)
    sc = dataclasses.replace(sc, width=643, height=357)  # width not a multiple of 4
    compare(ctx, sc, flags=sc.flags & ~gr.SHOW_TEXTURES)


def test_heightfield_no_cull_no_clip(ctx):
    sc = scenes.scene_heightfield_1280x720(n=129)
    compare(ctx, sc, flags=sc.flags & ~(gr.BACKFACE_CULLING | gr.FRUSTUM_CLIPPING))


def test_icospheres_vertex_colours(ctx):
    sc = scenes.scene_icospheres_1920x1080(count=12, levels=(2, 3))
    sc = dataclasses.replace(sc, width=960, height=540)
    compare(ctx, sc)


def test_camera_inside_sphere_near_plane(ctx):
    m = scenes.icosphere(3)
    sc = scenes.SceneData("inside", 320, 240, [scenes.ObjectData(m, scale=(2.0, 2.0, 2.0))],
                          scenes.CameraData((0.1, 0.2, 0.3), (0.3, -0.2, -1.0), (0.0, 1.0, 0.0)), [],
                          gr.FLAGS_DEFAULT & ~gr.BACKFACE_CULLING)
    compare(ctx, sc)


def test_non_pow2_and_solid_textures(ctx):
    m = scenes.heightfield(65, extent=1.5, seed=3)
    tex_img = scenes.random_texture(12, 10, seed=5, scale=3.0)  # not a power of two: % path
    solid = scenes.TextureData.solid((10, 200, 30, 255))
    m.tex = (np.arange(m.nf) % 3 - 1).astype(np.int32)  # -1 nil, 0 image, 1 solid
    cam = scenes.CameraData((0.0, 0.6, 1.8), (0.0, -0.5, -1.0), (0.0, 1.0, 0.0))
    sc = scenes.SceneData("textures", 400, 300, [scenes.ObjectData(m)], cam, [tex_img, solid],
                          gr.FLAGS_DEFAULT | gr.FLAT_SHADING)
    compare(ctx, sc)


def test_multi_object_depth_ties(ctx):
    # the same mesh drawn twice at the same place: every pixel is a depth tie and
    # the later object must win (rasterizer.go:156 uses >=)
    m = scenes.icosphere(2)
    m2 = dataclasses.replace(m, vcolor=np.full((m.nv, 3), 0.25, np.float32))
    objs = [scenes.ObjectData(m), scenes.ObjectData(m2)]
    sc = scenes.SceneData("ties", 256, 256, objs, scenes.CameraData((0, 0, 3.0), (0, 0, -1.0), (0, 1, 0)), [],
                          gr.FLAGS_DEFAULT)
    rgba, z, _ = compare(ctx, sc)
    covered = z > -1
    assert (rgba[covered][:, 3] == 255).all()


def test_empty_and_offscreen(ctx):
    m = scenes.icosphere(1)
    sc = scenes.SceneData("behind", 128, 96, [scenes.ObjectData(m, translation=(0.0, 0.0, 10.0))],
                          scenes.CameraData((0, 0, 0), (0, 0, -1.0), (0, 1, 0)), [], gr.FLAGS_DEFAULT)
    rgba, z, tpf = compare(ctx, sc)
    assert tpf == 0 and (z == -1).all()
    sc0 = dataclasses.replace(sc, objects=[])
    compare(ctx, sc0)


def test_renderer_api_matches_low_level(ctx):
    sc = scenes.scene_uvsphere_640x360()
    up = gr.UploadedScene(ctx, sc)
    rgba, z, tpf = up.render()
    r = gr.Renderer(ctx, sc.width, sc.height)
    r.set_fov(up.fov)
    assert r.BackfaceCulling and r.Lighting and not r.FlatShading
    r.draw([gr.Object(up.mesh_handles[0])], gr.Camera(*[getattr(sc.camera, k) for k in ("position", "direction", "up")]))
    assert r.TPF == tpf
    assert np.array_equal(r.pixels(), rgba)
    assert np.array_equal(r.zbuffer().view(np.uint32), z.view(np.uint32))
    r.close()


from tests.golden_scenes import GOLDEN_SCENES  # noqa: E402
import hashlib  # noqa: E402
import json  # noqa: E402
import os  # noqa: E402

_GOLDEN = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "frames.json")))


@pytest.mark.parametrize("name", sorted(GOLDEN_SCENES))
def test_gpu_matches_golden_digest(ctx, name):
    # the committed digests were produced by the oracle with the oracle's own
    # matrices; the library's host math yields the same matrices bit for bit
    sc = GOLDEN_SCENES[name]()
    up = gr.UploadedScene(ctx, sc)
    rgba, z, tpf = up.render()
    g = _GOLDEN[name]
    assert tpf == g["tpf"]
    assert hashlib.sha256(rgba.tobytes()).hexdigest() == g["rgba_sha256"]
    assert hashlib.sha256(z.tobytes()).hexdigest() == g["z_sha256"]


@pytest.mark.parametrize("tile", [16, 32])
def test_tile_sizes_and_tiny_bins(tile):
    # tiny bins force the overflow path: the first attempt overflows, the
    # library grows the bins and re-runs the frame with identical output
    c = gr.Context(0)
    try:
        c.set_tuning(tile, 8)
        sc = scenes.scene_heightfield_1280x720(n=129)
        up = gr.UploadedScene(c, sc)
        rgba, z, tpf = up.render()
        ref_rgba, ref_z, ref_tpf, st = oracle.draw_scene(sc, items_override=up.matrices, nthreads=4)
        assert st == 0 and tpf == ref_tpf
        assert np.array_equal(rgba, ref_rgba) and np.array_equal(z.view(np.uint32), ref_z.view(np.uint32))
        assert c.tuning()[1] > 8
    finally:
        c.close()


def test_alternating_scenes_replay_captured_frames(ctx):
    """Frames are replayed from captured CUDA graphs keyed by their arguments
    (an asynchronous draw's graph also by its staging slot); five scenes in
    turn, each drawn asynchronously and then synchronously (20 graphs, more
    than are kept), stay bit-exact."""
    scs = [GOLDEN_SCENES[name]() for name in sorted(GOLDEN_SCENES)][:5]
    ups = [gr.UploadedScene(ctx, sc) for sc in scs]
    first = []
    for sc, up in zip(scs, ups):
        rgba, z, tpf = up.render()
        ref_rgba, ref_z, ref_tpf, st = oracle.draw_scene(sc, items_override=up.matrices, nthreads=4)
        assert st == 0 and tpf == ref_tpf and np.array_equal(rgba, ref_rgba)
        first.append((rgba, z, tpf))
    for _ in range(3):
        for (rgba0, z0, tpf0), sc, up in zip(first, scs, ups):
            R.draw_async(ctx, up.items, len(sc.objects), up.params)
            rgba, z, tpf = up.render()
            assert tpf == tpf0 and np.array_equal(rgba, rgba0) and np.array_equal(z.view(np.uint32), z0.view(np.uint32))


def test_page_locked_host_outputs(ctx):
    """Outputs in page-locked host memory are written by the kernels through
    their device addresses (no copy after the frame); pageable outputs are
    copied.  Both give the oracle's frame, and both count as device-to-host
    bytes."""
    import ctypes as C

    from gorender_gb300 import _native as N

    L = N.lib()
    sc = scenes.scene_heightfield_1280x720(n=129)
    up = gr.UploadedScene(ctx, sc)
    npx = sc.width * sc.height
    hp = C.c_void_p()
    N.check(L.gr_host_alloc(npx * 8, C.byref(hp)))
    try:
        buf = (C.c_uint8 * (npx * 8)).from_address(hp.value)
        arr = np.frombuffer(buf, np.uint8)
        arr[:] = 0xAB
        tpf = C.c_int64()
        N.check(L.gr_draw(ctx.handle, up.items, len(sc.objects), C.byref(up.params), hp.value, hp.value + npx * 4,
                          C.byref(tpf)))
        rgba = arr[:npx * 4].reshape(sc.height, sc.width, 4).copy()
        z = arr[npx * 4:].view(np.float32).reshape(sc.height, sc.width).copy()
        h2d, d2h = C.c_int64(), C.c_int64()
        N.check(L.gr_context_last_transfer_bytes(ctx.handle, C.byref(h2d), C.byref(d2h)))
    finally:
        N.check(L.gr_host_free(hp))
    ref_rgba, ref_z, ref_tpf, st = oracle.draw_scene(sc, items_override=up.matrices, nthreads=4)
    assert st == 0 and tpf.value == ref_tpf
    assert np.array_equal(rgba, ref_rgba) and np.array_equal(z.view(np.uint32), ref_z.view(np.uint32))
    assert d2h.value >= npx * 8
    rgba2, z2, tpf2 = up.render()  # pageable numpy outputs: the copy path
    assert tpf2 == ref_tpf and np.array_equal(rgba2, ref_rgba)
