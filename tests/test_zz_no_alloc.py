"""gr_draw_noalloc: the frame draw for callers that cannot allocate device
memory (an engine or framework owning every allocation, or a frame loop with a
fixed memory budget).  It takes device pointers for every input and output
and keeps its working memory in a static device array, so it must produce the
same bytes as gr_draw on the same inputs -- here on two calls in a row, since
the array keeps the previous call's contents.

The caller-owned device buffers of this test are torch tensors (standing in
for the caller's own allocator); the entry point itself allocates nothing.
Collected last (file name) so that a stop-at-first-failure run has already
run every other test; it also passes when run alone in a fresh process.
"""
import ctypes as C
import dataclasses

import numpy as np
import pytest

import gorender_gb300 as gr
from gorender_gb300 import _native as N
from gorender_gb300 import scenes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _dev(a, dtype):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=dtype)).cuda()


def _ptr(t):
    return None if t is None else t.data_ptr()


def _noalloc_inputs(scene, up):
    """Device copies of the scene's meshes/textures and the noalloc tables."""
    keep = []

    def dev(a, dtype):
        if a is None:
            return None
        t = _dev(a, dtype)
        keep.append(t)
        return t

    objs = (N.NoallocObject * max(1, len(scene.objects)))()
    for i, o in enumerate(scene.objects):
        m = o.mesh
        d = objs[i].mesh
        pos = dev(m.pos, np.float32)
        d.positions = _ptr(pos)
        d.num_vertices = m.nv
        vn = dev(m.vnrm, np.float32)
        d.vertex_normals = _ptr(vn)
        d.num_normals = 0 if m.vnrm is None else m.vnrm.shape[0]
        d.vertex_indices = _ptr(dev(m.vidx, np.int32))
        d.normal_indices = _ptr(dev(m.nidx, np.int32))
        d.uvs = _ptr(dev(m.uv, np.float32))
        d.face_textures = _ptr(dev(m.tex, np.int32))
        d.face_normals = _ptr(dev(gr.face_normals(m.pos, m.vidx), np.float32))
        d.vertex_colors = _ptr(dev(m.vcolor, np.float32))
        d.num_faces = m.nf
        bb = np.zeros(32, np.float32)
        N.check(N.lib().gr_mesh_bounding_box(up.ctx.handle, up.mesh_handles[i], bb.ctypes.data_as(C.POINTER(C.c_float))))
        mvp, world = up.matrices[i]
        for k in range(32):
            objs[i].bbox[k] = float(bb[k])
        for k in range(16):
            objs[i].mvp[k] = float(mvp[k])
            objs[i].world[k] = float(world[k])
    texs = (N.NoallocTexture * max(1, len(scene.textures)))()
    for i, t in enumerate(scene.textures):
        texs[i].kind, texs[i].width, texs[i].height, texs[i].scale = t.kind, t.width, t.height, t.scale
        for k in range(4):
            texs[i].color[k] = t.color[k]
        texs[i].rgba = _ptr(dev(t.pixels, np.uint8)) if t.pixels is not None else None
    return objs, texs, keep


def _small_textured_heightfield():
    m = scenes.heightfield(33, extent=1.5, seed=3)
    img = scenes.random_texture(16, 8, seed=5, scale=3.0)
    solid = scenes.TextureData.solid((10, 200, 30, 255))
    m.tex = (np.arange(m.nf) % 3 - 1).astype(np.int32)  # nil, image, solid
    cam = scenes.CameraData((0.0, 0.35, 1.2), (0.0, -0.4, -1.0), (0.0, 1.0, 0.0))
    return scenes.SceneData("hf33-noalloc", 320, 240, [scenes.ObjectData(m)], cam, [img, solid],
                            scenes.DEFAULT_FLAGS | scenes.FLAT_SHADING)


@pytest.mark.parametrize("make", [
    lambda: dataclasses.replace(scenes.scene_uvsphere_640x360(), width=480, height=320),
    _small_textured_heightfield,
])
def test_noalloc_matches_gr_draw_twice(make):
    scene = make()
    ctx = gr.Context(0)
    try:
        up = gr.UploadedScene(ctx, scene)
        ref_rgba, ref_z, ref_tpf = up.render()  # the existing entry point
        assert (ref_z > -1).sum() > 1000
        objs, texs, keep = _noalloc_inputs(scene, up)
        H, W = scene.height, scene.width
        for call in range(2):
            rgba = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
            z = torch.zeros((H, W), dtype=torch.float32, device="cuda")
            tpf = C.c_int64(-1)
            st = N.lib().gr_draw_noalloc(0, objs, len(scene.objects), texs, len(scene.textures),
                                         C.byref(up.params), rgba.data_ptr(), z.data_ptr(), None, C.byref(tpf))
            N.check(st)
            out_rgba = rgba.cpu().numpy()
            out_z = z.cpu().numpy()
            assert tpf.value == ref_tpf, f"call {call}: TPF {tpf.value} vs {ref_tpf}"
            assert np.array_equal(out_rgba, ref_rgba), f"call {call}: RGBA differs"
            assert np.array_equal(out_z.view(np.uint32), ref_z.view(np.uint32)), f"call {call}: Z differs"
        del keep
    finally:
        ctx.close()


def test_noalloc_rejects_sizes_beyond_its_limits():
    p = gr.make_params(513, 512, gr.FLAGS_DEFAULT)
    rgba = torch.zeros((512, 513, 4), dtype=torch.uint8, device="cuda")
    z = torch.zeros((512, 513), dtype=torch.float32, device="cuda")
    st = N.lib().gr_draw_noalloc(0, None, 0, None, 0, C.byref(p), rgba.data_ptr(), z.data_ptr(), None, None)
    assert st == N.GR_ERR_UNSUPPORTED
    assert b"512x512" in N.lib().gr_last_error()
    big = scenes.heightfield(65)  # 8192 faces > 4096
    objs = (N.NoallocObject * 1)()
    objs[0].mesh.positions = rgba.data_ptr()  # never read: rejected before any GPU work
    objs[0].mesh.num_vertices = big.nv
    objs[0].mesh.vertex_indices = rgba.data_ptr()
    objs[0].mesh.face_normals = rgba.data_ptr()
    objs[0].mesh.num_faces = big.nf
    p2 = gr.make_params(256, 256, gr.FLAGS_DEFAULT)
    st = N.lib().gr_draw_noalloc(0, objs, 1, None, 0, C.byref(p2), rgba.data_ptr(), z.data_ptr(), None, None)
    assert st == N.GR_ERR_UNSUPPORTED
    assert b"4096" in N.lib().gr_last_error()


def _call(scene, up, objs, texs, flags=None):
    H, W = scene.height, scene.width
    rgba = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
    z = torch.zeros((H, W), dtype=torch.float32, device="cuda")
    tpf = C.c_int64(-1)
    params = up.params
    if flags is not None:
        params = gr.make_params(W, H, flags)
    st = N.lib().gr_draw_noalloc(0, objs, len(scene.objects), texs, len(scene.textures), C.byref(params),
                                 rgba.data_ptr(), z.data_ptr(), None, C.byref(tpf))
    return st, rgba, z, tpf.value


def _assert_matches(scene, up, objs, texs):
    ref_rgba, ref_z, ref_tpf = up.render()
    st, rgba, z, tpf = _call(scene, up, objs, texs)
    N.check(st)
    assert tpf == ref_tpf
    assert np.array_equal(rgba.cpu().numpy(), ref_rgba)
    assert np.array_equal(z.cpu().numpy().view(np.uint32), ref_z.view(np.uint32))


def test_noalloc_rejects_bad_device_indices_and_flags():
    """Indices in the caller's device buffers are checked on the GPU before the
    frame's kernels gather through them: an out-of-range face texture or
    vertex index returns GR_ERR_BAD_INDEX (no fault), unknown flag bits
    GR_ERR_INVALID_ARGUMENT, and the next good call still matches gr_draw."""
    scene = _small_textured_heightfield()
    ctx = gr.Context(0)
    try:
        up = gr.UploadedScene(ctx, scene)
        objs, texs, keep = _noalloc_inputs(scene, up)
        m = scene.objects[0].mesh
        good_tex, good_vidx = objs[0].mesh.face_textures, objs[0].mesh.vertex_indices
        bad_tex = m.tex.copy()
        bad_tex[m.nf // 2] = len(scene.textures)  # one past the last texture
        t_bad = _dev(bad_tex, np.int32)
        objs[0].mesh.face_textures = t_bad.data_ptr()
        st, *_ = _call(scene, up, objs, texs)
        assert st == N.GR_ERR_BAD_INDEX and b"texture" in N.lib().gr_last_error()
        objs[0].mesh.face_textures = good_tex
        bad_v = m.vidx.copy()
        bad_v.reshape(-1)[7] = m.nv
        v_bad = _dev(bad_v, np.int32)
        objs[0].mesh.vertex_indices = v_bad.data_ptr()
        st, *_ = _call(scene, up, objs, texs)
        assert st == N.GR_ERR_BAD_INDEX and b"vertex" in N.lib().gr_last_error()
        objs[0].mesh.vertex_indices = good_vidx
        st, *_ = _call(scene, up, objs, texs, flags=scene.flags | 0x80000000)
        assert st == N.GR_ERR_INVALID_ARGUMENT and b"flag" in N.lib().gr_last_error()
        _assert_matches(scene, up, objs, texs)
        del keep, t_bad, v_bad
    finally:
        ctx.close()


def test_noalloc_bin_overflow_then_next_call_matches():
    """A frame within the size limits whose triangles all fall into one raster
    tile overflows the fixed 1024-entry bins: GR_ERR_BIN_OVERFLOW.  The static
    array keeps what that frame left behind; the next call must still give
    gr_draw's bytes."""
    m = scenes.heightfield(46, extent=1.5, seed=3)  # 4050 faces, drawn a few pixels wide
    cam = scenes.CameraData((0.0, 0.35, 1.2), (0.0, -0.4, -1.0), (0.0, 1.0, 0.0))
    tiny = scenes.SceneData("hf46-one-tile", 256, 256, [scenes.ObjectData(m, scale=(0.01, 0.01, 0.01))], cam, [],
                            scenes.DEFAULT_FLAGS | scenes.FLAT_SHADING)
    ctx = gr.Context(0)
    try:
        up = gr.UploadedScene(ctx, tiny)
        objs, texs, keep = _noalloc_inputs(tiny, up)
        st, *_ = _call(tiny, up, objs, texs)
        assert st == N.GR_ERR_BIN_OVERFLOW, N.lib().gr_last_error()
        scene = _small_textured_heightfield()
        up2 = gr.UploadedScene(ctx, scene)
        objs2, texs2, keep2 = _noalloc_inputs(scene, up2)
        for _ in range(2):
            _assert_matches(scene, up2, objs2, texs2)
        del keep, keep2
    finally:
        ctx.close()
