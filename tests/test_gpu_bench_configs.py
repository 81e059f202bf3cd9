"""Parity at exactly the configurations bench.py times, at full size.

* the 199,712-face heightfield at 1280x720 after the library autotuner, and
  forced to the tuning the bench has reported (16x16 tiles, raster slice cost
  4096, bin capacity 1024);
* the 64-icosphere 1920x1080 frame with per-vertex colours (5.0 M faces), at
  the default tuning and after the autotuner;
* every view of the 256-view batch (its CUDA graph, autotuned) against the
  oracle's frame of that view alone.

Each frame is compared with the oracle's, whose matrices come from its own
restatement of projectObject (renderer.go:255-262): RGBA8 and the z-buffer's
bit patterns must be identical and TPF must match.
"""
import ctypes as C
import os

import numpy as np
import pytest

import gorender_gb300 as gr
from gorender_gb300 import _native as N
from gorender_gb300 import renderer as R
from gorender_gb300 import scenes
from oracle import oracle

pytestmark = pytest.mark.gpu

THREADS = max(1, min(os.cpu_count() or 1, 64))


def _oracle(sc):
    rgba, z, tpf, st = oracle.draw_scene(sc, nthreads=THREADS)
    assert st == 0
    return rgba, z, tpf


def _same(got, ref, what):
    rgba, z, tpf = got
    ref_rgba, ref_z, ref_tpf = ref
    assert tpf == ref_tpf, f"{what}: TPF {tpf} vs oracle {ref_tpf}"
    d = (rgba != ref_rgba).any(axis=-1)
    assert not d.any(), f"{what}: {int(d.sum())} RGBA pixels differ, first at {np.argwhere(d)[:3].tolist()}"
    dz = z.view(np.uint32) != ref_z.view(np.uint32)
    assert not dz.any(), f"{what}: {int(dz.sum())} z values differ, first at {np.argwhere(dz)[:3].tolist()}"


@pytest.fixture(scope="module")
def heightfield():
    sc = scenes.scene_heightfield_1280x720()
    return sc, _oracle(sc)


@pytest.fixture(scope="module")
def icospheres():
    sc = scenes.scene_icospheres_1920x1080()
    return sc, _oracle(sc)


def _render_tuned(sc, tuning):
    ctx = gr.Context(0)
    try:
        up = gr.UploadedScene(ctx, sc)
        if tuning == "autotune":
            N.check(N.lib().gr_context_autotune(ctx.handle, up.items, len(sc.objects), C.byref(up.params)))
        elif tuning is not None:
            tile, bins, slice_cost = tuning
            ctx.set_tuning(tile, bins)
            N.check(N.lib().gr_context_set_raster(ctx.handle, slice_cost, 0))
        out = up.render()
        again = up.render()  # a graph replay of the same frame
        assert np.array_equal(out[0], again[0]) and np.array_equal(out[1].view(np.uint32), again[1].view(np.uint32))
        return out, ctx.tuning() + (ctx.raster()[0],)
    finally:
        ctx.close()


@pytest.mark.parametrize("tuning", ["autotune", (16, 1024, 4096), (32, 1024, 8192)],
                         ids=["autotuned", "tile16-bins1024-slice4096", "tile32-bins1024-slice8192"])
def test_heightfield_full_size(heightfield, tuning):
    sc, ref = heightfield
    got, used = _render_tuned(sc, tuning)
    if tuning != "autotune":
        assert used[0] == tuning[0] and used[2] == tuning[2]
    _same(got, ref, f"heightfield {used}")
    assert (got[1] > -1).sum() > 500_000


@pytest.mark.parametrize("tuning", [None, "autotune"], ids=["default", "autotuned"])
def test_icospheres_full_size_1080p(icospheres, tuning):
    sc, ref = icospheres
    assert sc.num_triangles > 3_000_000 and (sc.width, sc.height) == (1920, 1080)
    got, used = _render_tuned(sc, tuning)
    _same(got, ref, f"icospheres {used}")


def test_multiview_batch_256_every_view_against_oracle():
    vs = scenes.multiview_batch(256, seed=0)
    ctx = gr.Context(0)
    bufs = []
    try:
        views, entries = [], []
        for v, sc in enumerate(vs):
            up = R.UploadedScene(ctx, sc)
            rgba = ctx.device_buffer(sc.width * sc.height * 4)
            z = ctx.device_buffer(sc.width * sc.height * 4)
            bufs.append((rgba, z))
            views.append((up.params, rgba.ptr, z.ptr))
            entries += [(h, mvp, w, v) for h, (mvp, w) in zip(up.mesh_handles, up.matrices)]
        b = R.Batch(ctx, views, entries, autotune=True)
        b.run()
        b.sync()
        b.run()  # a replay of the captured graph
        b.sync()
        tpfs = b.view_tpf()
        for v, sc in enumerate(vs):
            rgba = bufs[v][0].download((sc.height, sc.width, 4), np.uint8)
            z = bufs[v][1].download((sc.height, sc.width), np.float32)
            _same((rgba, z, tpfs[v]), _oracle(sc), f"view {v} ({sc.name}, {sc.width}x{sc.height})")
        b.close()
    finally:
        for r, z in bufs:
            r.free()
            z.free()
        ctx.close()
