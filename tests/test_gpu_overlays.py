"""GPU parity of the ShowEdges / ShowVertices overlays (renderer.go:191-216):
edge lines, centroid marks and vertex marks drawn in draw order over the
depth-tested fills, through the C-ABI, bit for bit against the oracle."""
import dataclasses

import numpy as np
import pytest

import gorender_gb300 as gr
from gorender_gb300 import renderer as R
from gorender_gb300 import scenes
from tests.test_gpu_parity import compare

pytestmark = pytest.mark.gpu

EDGES, VERTS = gr.SHOW_EDGES, gr.SHOW_VERTICES


@pytest.fixture(scope="module")
def ctx():
    c = gr.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("extra,drop", [
    (EDGES, 0), (VERTS, 0), (EDGES | VERTS, 0),
    (EDGES | VERTS, gr.SHOW_FACES),              # white edges, no centroid marks
    (EDGES, gr.BACKFACE_CULLING),                # back faces: edges but never a fill
    (EDGES | VERTS, gr.FRUSTUM_CLIPPING),
])
def test_uvsphere_overlays(ctx, extra, drop):
    sc = scenes.scene_uvsphere_640x360()
    rgba, _, _ = compare(ctx, sc, flags=(sc.flags | extra) & ~drop)
    assert ((rgba[..., 0] == 255) & (rgba[..., 1] == 161)).any() or not (extra & VERTS)


def test_heightfield_clipped_fans_with_overlays(ctx):
    # clipped faces fan into several triangles, each with its own marks
    sc = scenes.scene_heightfield_1280x720(n=97)
    compare(ctx, sc, flags=sc.flags | EDGES | VERTS)


def test_camera_inside_sphere_overlays(ctx):
    m = scenes.icosphere(3)
    sc = scenes.SceneData("inside", 320, 240, [scenes.ObjectData(m, scale=(2.0, 2.0, 2.0))],
                          scenes.CameraData((0.1, 0.2, 0.3), (0.3, -0.2, -1.0), (0.0, 1.0, 0.0)), [],
                          (gr.FLAGS_DEFAULT & ~gr.BACKFACE_CULLING) | EDGES | VERTS)
    compare(ctx, sc)


def test_icospheres_vertex_marks_and_depth_ties(ctx):
    sc = scenes.scene_icospheres_1920x1080(count=8, levels=(1, 2))
    sc = dataclasses.replace(sc, width=481, height=271)  # odd sizes: row wrap of marks
    compare(ctx, sc, flags=sc.flags | EDGES | VERTS)


@pytest.mark.parametrize("tile", [16, 32])
def test_overlays_every_tile_size_twice(tile):
    """Marks are cleared by the resolve: a second frame equals the first."""
    ctx = gr.Context(0)
    try:
        ctx.set_tuning(tile, 0)
        sc = scenes.scene_uvsphere_640x360()
        a = compare(ctx, sc, flags=sc.flags | EDGES | VERTS)
        b = compare(ctx, sc, flags=sc.flags | EDGES | VERTS)
        assert np.array_equal(a[0], b[0])
        # and a frame without overlays afterwards shows none
        c = compare(ctx, sc)
        assert not ((c[0][..., 0] == 255) & (c[0][..., 1] == 161)).any()
    finally:
        ctx.close()


# overlay flags per view k: every view marked, or only every third view (a
# warp of kept faces then mixes faces of views with and without marks)
OVERLAY_PATTERNS = {
    "all": lambda k: EDGES if k % 2 else VERTS,
    "some": lambda k: (EDGES | VERTS) if k % 3 == 1 else 0,
}


@pytest.mark.parametrize("pattern", sorted(OVERLAY_PATTERNS))
def test_batched_views_with_overlays(pattern):
    torch = pytest.importorskip("torch")
    ctx = gr.Context(0)
    try:
        vs = scenes.multiview_batch(6, seed=2, min_tris=100, max_tris=5000,
                                    resolutions=((96, 64), (128, 128), (130, 77)))
        vs = [dataclasses.replace(v, flags=v.flags | OVERLAY_PATTERNS[pattern](k)) for k, v in enumerate(vs)]
        views, entries, singles, bufs = [], [], [], []
        for v, sc in enumerate(vs):
            up = gr.UploadedScene(ctx, sc)
            rgba = torch.zeros((sc.height, sc.width, 4), dtype=torch.uint8, device="cuda")
            z = torch.zeros((sc.height, sc.width), dtype=torch.float32, device="cuda")
            bufs.append((rgba, z))
            views.append((up.params, rgba.data_ptr(), z.data_ptr()))
            entries += [(h, mvp, w, v) for h, (mvp, w) in zip(up.mesh_handles, up.matrices)]
            singles.append(up)
        R.draw_views(ctx, views, entries)
        try:
            ctx.sync()
        except gr.GrError:
            R.draw_views(ctx, views, entries)
            ctx.sync()
        for v, up in enumerate(singles):
            ref_rgba, ref_z, _ = up.render()
            assert np.array_equal(bufs[v][0].cpu().numpy(), ref_rgba), f"view {v}"
            assert np.array_equal(bufs[v][1].cpu().numpy().view(np.uint32), ref_z.view(np.uint32))
    finally:
        ctx.close()
