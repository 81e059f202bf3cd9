"""Fuzz parity: seeded triangle soups (tests/fuzz_scenes.py) rendered through
the C-ABI and by the oracle, bit for bit (RGBA8, Z bit patterns, TPF), over
flag combinations, both raster tile sizes, odd framebuffer sizes, overlays
and a batch of soup views."""
import dataclasses

import numpy as np
import pytest

import gorender_gb300 as gr
from oracle import oracle
from tests import fuzz_scenes as fz

pytestmark = pytest.mark.gpu

D = gr.FLAGS_DEFAULT
FLAG_SETS = [
    ("default", D),
    ("flat", D | gr.FLAT_SHADING),
    ("no-cull", D & ~gr.BACKFACE_CULLING),
    ("no-clip", D & ~gr.FRUSTUM_CLIPPING),
    ("no-clip-no-cull", D & ~(gr.FRUSTUM_CLIPPING | gr.BACKFACE_CULLING)),
    ("unlit", D & ~gr.LIGHTING),
    ("untextured", D & ~gr.SHOW_TEXTURES),
]
SIZES = [(97, 61), (160, 120), (333, 211)]


@pytest.fixture(scope="module", params=[32, 16], ids=["tile32", "tile16"])
def ctx(request):
    c = gr.Context(0)
    c.set_tuning(request.param, 0)
    yield c
    c.close()


def _check(ctx, sc):
    up = gr.UploadedScene(ctx, sc)
    rgba, z, tpf = up.render()
    ref_rgba, ref_z, ref_tpf, st = oracle.draw_scene(sc, items_override=up.matrices, nthreads=4)
    assert st == 0
    diff = (rgba != ref_rgba).any(axis=2)
    zdiff = z.view(np.uint32) != ref_z.view(np.uint32)
    assert tpf == ref_tpf, f"TPF {tpf} vs oracle {ref_tpf}"
    assert not diff.any(), f"{int(diff.sum())} RGBA pixels differ, first at {np.argwhere(diff)[:5].tolist()}"
    assert not zdiff.any(), f"{int(zdiff.sum())} z values differ, first at {np.argwhere(zdiff)[:5].tolist()}"
    return rgba, z, tpf


@pytest.mark.parametrize("name,flags", FLAG_SETS, ids=[f[0] for f in FLAG_SETS])
@pytest.mark.parametrize("seed", [1, 2, 3])
def test_soup_flags(ctx, seed, name, flags):
    w, h = SIZES[seed - 1]
    _check(ctx, fz.soup_scene(seed, w, h, flags))


@pytest.mark.parametrize("seed", [4, 5])
def test_soup_vertex_colours_gouraud(ctx, seed):
    _check(ctx, fz.soup_scene(seed, 211, 149, D, vcolor=True))


@pytest.mark.parametrize("seed", [6, 7])
def test_soup_overlays(ctx, seed):
    # with clipping on the marks stay near the screen (clipped corners)
    _check(ctx, fz.soup_scene(seed, 150, 101, D | gr.SHOW_EDGES | gr.SHOW_VERTICES, n=400))
    _check(ctx, fz.soup_scene(seed, 150, 101, (D | gr.SHOW_VERTICES) & ~gr.SHOW_FACES, n=400))


def test_soup_many_objects_large(ctx):
    _check(ctx, fz.soup_scene(8, 640, 360, D, objects=6, n=3000))


def test_soup_batch_views():
    """Soup views of different sizes and flags in one batched draw: each view
    equals the oracle's frame of that view alone."""
    torch = pytest.importorskip("torch")
    from gorender_gb300 import renderer as R

    ctx = gr.Context(0)
    try:
        specs = [(11, 97, 61, D), (12, 160, 120, D & ~gr.FRUSTUM_CLIPPING), (13, 64, 200, D | gr.FLAT_SHADING),
                 (14, 333, 211, D & ~gr.BACKFACE_CULLING)]
        scs = [fz.soup_scene(s, w, h, f) for s, w, h, f in specs]
        views, entries, ups = [], [], []
        for v, sc in enumerate(scs):
            up = gr.UploadedScene(ctx, sc)
            rgba = torch.zeros((sc.height, sc.width, 4), dtype=torch.uint8, device="cuda")
            z = torch.zeros((sc.height, sc.width), dtype=torch.float32, device="cuda")
            views.append((up.params, rgba.data_ptr(), z.data_ptr(), rgba, z))
            for hnd, (mvp, w) in zip(up.mesh_handles, up.matrices):
                entries.append((hnd, mvp, w, v))
            ups.append(up)
        vs = [(p, r, z) for p, r, z, _, _ in views]
        R.draw_views(ctx, vs, entries)
        try:
            ctx.sync()
        except gr.GrError as e:  # bins grown after an overflow: issue the frame again
            assert e.code == R.N.GR_ERR_BIN_OVERFLOW
            R.draw_views(ctx, vs, entries)
            ctx.sync()
        tpf = (R.C.c_int64 * len(views))()
        R.N.check(R.N.lib().gr_context_view_tpf(ctx.handle, tpf, len(views)))
        for v, (sc, up) in enumerate(zip(scs, ups)):
            ref_rgba, ref_z, ref_tpf, st = oracle.draw_scene(sc, items_override=up.matrices, nthreads=4)
            assert st == 0 and tpf[v] == ref_tpf
            rgba, z = views[v][3].cpu().numpy(), views[v][4].cpu().numpy()
            assert np.array_equal(rgba, ref_rgba), f"view {v}: RGBA differs"
            assert np.array_equal(z.view(np.uint32), ref_z.view(np.uint32)), f"view {v}: Z differs"
    finally:
        ctx.close()


@pytest.mark.parametrize("flags", [D, D & ~gr.FRUSTUM_CLIPPING, D & ~(gr.FRUSTUM_CLIPPING | gr.BACKFACE_CULLING)],
                         ids=["default", "no-clip", "no-clip-no-cull"])
def test_soup_nan_inf_positions(ctx, flags):
    """Corners at NaN and +-Inf in model space: the comparisons the reference
    makes on them (facing test, clip planes, Go's NaN-propagating min/max in
    the bin test, int() of NaN) decide what is drawn, bit for bit."""
    sc = fz.soup_scene(21, 160, 120, flags, objects=1, n=600)
    m = sc.objects[0].mesh
    pos = m.pos.copy()
    bad = np.arange(0, pos.shape[0], 37)
    pos[bad[0::3], 0] = np.nan
    pos[bad[1::3], 1] = np.inf
    pos[bad[2::3], 2] = -np.inf
    m = dataclasses.replace(m, pos=pos)
    sc = dataclasses.replace(sc, objects=[dataclasses.replace(sc.objects[0], mesh=m)])
    _check(ctx, sc)
