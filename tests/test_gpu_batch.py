"""Batched multi-view rendering: every view of a batch must be bit-identical
to rendering that view alone with the plain path (gr_draw), both for the
direct batched call (gr_draw_views) and for the autotuned CUDA-graph batch
(gr_batch_*), and the per-view TPF must match.

Device output buffers are torch tensors (the test's stand-in for the caller's
device memory)."""
import numpy as np
import pytest

import gorender_gb300 as gr
from gorender_gb300 import renderer as R
from gorender_gb300 import scenes

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _setup(ctx, views_scenes):
    views, entries, singles = [], [], []
    for v, sc in enumerate(views_scenes):
        up = gr.UploadedScene(ctx, sc)
        rgba = torch.zeros((sc.height, sc.width, 4), dtype=torch.uint8, device="cuda")
        z = torch.zeros((sc.height, sc.width), dtype=torch.float32, device="cuda")
        views.append((up.params, rgba.data_ptr(), z.data_ptr(), rgba, z))
        for h, (mvp, w) in zip(up.mesh_handles, up.matrices):
            entries.append((h, mvp, w, v))
        singles.append(up)
    return views, entries, singles


def _check(views, singles, tpfs):
    for v, (params, _, _, rgba, z) in enumerate(views):
        ref_rgba, ref_z, ref_tpf = singles[v].render()
        got_rgba = rgba.cpu().numpy()
        got_z = z.cpu().numpy()
        assert tpfs[v] == ref_tpf, f"view {v}: TPF {tpfs[v]} vs {ref_tpf}"
        assert np.array_equal(got_rgba, ref_rgba), f"view {v}: RGBA differs"
        assert np.array_equal(got_z.view(np.uint32), ref_z.view(np.uint32)), f"view {v}: Z differs"


def _small_views(n=12, seed=3):
    vs = scenes.multiview_batch(n, seed=seed, min_tris=100, max_tris=30000,
                                resolutions=((96, 64), (128, 128), (160, 90), (130, 77)))
    # one view with no objects: it must still be cleared and dot-gridded
    vs.append(scenes.SceneData("empty", 64, 48, [], scenes.CameraData(), [], scenes.DEFAULT_FLAGS))
    return vs


def test_draw_views_matches_single_views():
    ctx = gr.Context(0)
    try:
        views, entries, singles = _setup(ctx, _small_views())
        vs = [(p, r, z) for p, r, z, _, _ in views]
        R.draw_views(ctx, vs, entries)
        try:
            ctx.sync()
        except gr.GrError as e:
            # asynchronous draws report bin overflow at sync after growing the
            # bins; the documented remedy is to issue the frame again
            assert e.code == R.N.GR_ERR_BIN_OVERFLOW
            R.draw_views(ctx, vs, entries)
            ctx.sync()
        tpf = (R.C.c_int64 * len(views))()
        R.N.check(R.N.lib().gr_context_view_tpf(ctx.handle, tpf, len(views)))
        _check(views, singles, list(tpf))
    finally:
        ctx.close()


def test_graph_batch_autotuned_matches_single_views():
    ctx = gr.Context(0)
    try:
        views, entries, singles = _setup(ctx, _small_views(10, seed=5))
        b = R.Batch(ctx, [(p, r, z) for p, r, z, _, _ in views], entries, autotune=True)
        tuning = b.tuning()
        assert tuning["tile_size"] in (16, 32) and tuning["bin_capacity"] >= 256
        for _ in range(3):  # graph replays
            for _, _, _, rgba, z in views:
                rgba.zero_()
                z.zero_()
            torch.cuda.synchronize()
            b.run()
            b.sync()
            _check(views, singles, b.view_tpf())
        b.close()
    finally:
        ctx.close()


def test_batch_view_index_checked():
    ctx = gr.Context(0)
    try:
        views, entries, _ = _setup(ctx, _small_views(2, seed=9)[:2])
        bad = [(m, mvp, w, 7) for m, mvp, w, _ in entries]
        with pytest.raises(gr.GrError):
            R.draw_views(ctx, [(p, r, z) for p, r, z, _, _ in views], bad)
    finally:
        ctx.close()


def test_back_to_back_async_draws_keep_their_own_tables():
    """Plain asynchronous draws of different views issued without a sync in
    between: each must render its own items (the pinned staging of one draw is
    not overwritten by the next before its copy has run)."""
    ctx = gr.Context(0)
    try:
        views, entries, singles = _setup(ctx, _small_views(9, seed=11))
        per_view = [[] for _ in views]
        for m, mvp, w, v in entries:
            per_view[v].append((m, mvp, w))
        items = [R.make_items(e) for e in per_view]
        for _ in range(2):  # the first pass may grow buffers (reported at sync)
            for _, _, _, rgba, z in views:
                rgba.zero_()
                z.zero_()
            torch.cuda.synchronize()
            for v, (params, rp, zp, _, _) in enumerate(views):
                R.draw_async(ctx, items[v], len(per_view[v]), params, rp, zp)
            try:
                ctx.sync()
                break
            except gr.GrError as e:
                assert e.code == R.N.GR_ERR_BIN_OVERFLOW
        for v, (params, _, _, rgba, z) in enumerate(views):
            ref_rgba, ref_z, _ = singles[v].render()
            assert np.array_equal(rgba.cpu().numpy(), ref_rgba), f"view {v}: RGBA differs"
            assert np.array_equal(z.cpu().numpy().view(np.uint32), ref_z.view(np.uint32)), f"view {v}: Z differs"
    finally:
        ctx.close()


def test_device_buffers_through_the_c_abi():
    """gr_device_alloc / gr_copy / gr_device_free: the device memory a host
    without CUDA of its own uses for batch outputs and parameters."""
    ctx = gr.Context(0)
    try:
        a = np.arange(1000, dtype=np.float32)
        buf = ctx.device_buffer(a.nbytes).upload(a)
        assert np.array_equal(buf.download(a.shape, np.float32), a)
        other = ctx.device_buffer(a.nbytes)
        R.N.check(R.N.lib().gr_copy(ctx.handle, other.ptr, buf.ptr, a.nbytes))  # device to device
        assert np.array_equal(other.download(a.shape, np.float32), a)
        with pytest.raises(ValueError):
            buf.download((2000,), np.float32)
        p = R.C.c_void_p()
        assert R.N.lib().gr_device_alloc(ctx.handle, 0, R.C.byref(p)) == R.N.GR_ERR_INVALID_ARGUMENT
        assert R.N.lib().gr_copy(ctx.handle, None, buf.ptr, 4) == R.N.GR_ERR_INVALID_ARGUMENT
        assert R.N.lib().gr_copy(ctx.handle, None, None, 0) == R.N.GR_OK
        buf.free()
        other.free()
        assert R.N.lib().gr_device_free(ctx.handle, None) == R.N.GR_OK
    finally:
        ctx.close()
