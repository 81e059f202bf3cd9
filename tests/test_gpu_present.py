"""Double-buffered headless present (gr_presenter_*): every frame returned one
call later is bit-identical to the synchronous Renderer.Draw of the same
objects, while the next frame renders (FrameBuffer.SwapBuffers and the
present loop of the reference, rasterizer.go:32-34, main.go:221-228)."""
import numpy as np
import pytest

import gorender_gb300 as gr
from gorender_gb300 import scenes

pytestmark = pytest.mark.gpu


def _renderer(ctx, w=320, h=200):
    """A renderer with the heightfield and a small ball, uploaded to ctx."""
    sc = scenes.scene_heightfield_1280x720(n=65)
    tex = [ctx.texture(t) for t in sc.textures]
    mesh = ctx.mesh(sc.objects[0].mesh, tex)
    ball = ctx.mesh(scenes.icosphere(2, noise=0.05, seed=3))
    cam = gr.Camera(sc.camera.position, sc.camera.direction, sc.camera.up)
    objs = [gr.Object(mesh), gr.Object(ball, scale=(0.3, 0.3, 0.3), translation=(0.0, 0.4, 1.5))]
    r = gr.Renderer(ctx, w, h)
    r.FlatShading = True
    r.set_fov(gr.fov_radians(60.0))
    return r, objs, cam


def _demo_step(objs):
    # main.go demo loop: obj.Rotation.Y += 0.01 (float32)
    for o in objs:
        o.Rotation = (o.Rotation[0], float(np.float32(o.Rotation[1]) + np.float32(0.01)), o.Rotation[2])


@pytest.mark.parametrize("tiny_bins", [False, True])
def test_presenter_frames_equal_synchronous_draws(tiny_bins):
    ctx = gr.Context(0)      # synchronous reference draws
    pctx = gr.Context(0)     # the presenter's context
    try:
        if tiny_bins:
            pctx.set_tuning(32, 8)  # the first frame overflows its bins: re-rendered before it is returned
        ref, objs, cam = _renderer(ctx)
        pres_r, pobjs, _ = _renderer(pctx)
        p = gr.Presenter(pres_r)
        expected = []
        got = []
        for k in range(6):
            ref.draw(objs, cam)
            expected.append((ref.pixels(), ref.TPF))
            rgba, tpf = p.frame(pobjs, cam)
            if k == 0:
                assert rgba is None and tpf == -1
            else:
                got.append((rgba, tpf))
            _demo_step(objs)
            _demo_step(pobjs)
        got.append(p.flush())
        assert p.flush() == (None, -1)
        assert len(got) == len(expected)
        for k, ((a, ta), (b, tb)) in enumerate(zip(got, expected)):
            assert ta == tb, f"frame {k}: TPF {ta} vs {tb}"
            assert np.array_equal(a, b), f"frame {k} differs"
        # the demo rotation changed the frames
        assert not np.array_equal(expected[0][0], expected[-1][0])
        p.close()
    finally:
        pctx.close()
        ctx.close()
