"""Differentiable forward/backward on the GPU (gr_diff_*), through the C-ABI.

Visibility (the per-pixel face of the forward pass) must equal the oracle's
raster bit for bit.  The loss and the four gradients must agree with the FP64
adjoint of the oracle evaluated on the GPU's own per-pixel records (same
faces, same texels): relative error max|g - g64| / max|g64| <= 1e-4 per
gradient, 1e-5 for the loss."""
import numpy as np
import pytest

import gorender_gb300 as gr
from gorender_gb300 import renderer as R
from oracle import oracle
from tests import diff_cases as dc

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

GRAD_TOL = 1e-4
LOSS_TOL = 1e-5


class _DevArray:
    """A device buffer of the library seen by torch without a copy."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": shape, "typestr": typestr, "data": (ptr, False), "version": 3}


def _dev(a, dtype=torch.float32):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


class Run:
    """Forward (target, then parameters) and backward of a DiffSceneData."""

    def __init__(self, sc):
        self.sc = sc
        self.ctx = gr.Context(0)
        mesh = self.ctx.mesh(sc.mesh)
        world, views = R.diff_views(sc)
        self.diff = R.Diff(self.ctx, mesh, world, views, tex_size=sc.tex.shape[:2])
        self.npx = sum(w * h for w, h, _, _, _ in views)
        nv = sc.mesh.nv
        self.p = [_dev(sc.mesh.pos), _dev(sc.vcol), _dev(sc.tex)]
        tp = sc.target_params
        self.tp = [_dev(tp["pos"]), _dev(tp["vcol"]), _dev(tp["tex"])]
        self.target = torch.zeros((self.npx, 4), dtype=torch.float32, device="cuda")
        zeros = torch.zeros_like(self.target)
        self.diff.forward(self.tp[0].data_ptr(), self.tp[1].data_ptr(), self.tp[2].data_ptr(), tp["light"],
                          zeros.data_ptr(), self.target.data_ptr())
        self.image = torch.zeros_like(self.target)
        self.loss = self.diff.forward(self.p[0].data_ptr(), self.p[1].data_ptr(), self.p[2].data_ptr(), sc.light,
                                      self.target.data_ptr(), self.image.data_ptr())
        self.g = [torch.empty((nv, 4), device="cuda"), torch.empty((nv, 3), device="cuda"),
                  torch.empty(sc.tex.shape, device="cuda")]
        self.g_light = self.diff.backward(*(t.data_ptr() for t in self.g))
        ids_ptr, rec_ptr, n = self.diff.buffers()
        assert n == self.npx
        self.ids = torch.as_tensor(_DevArray(ids_ptr, (n,), "<u4"), device="cuda").cpu().numpy().copy()
        rec = torch.as_tensor(_DevArray(rec_ptr, (n, 4), "<u4"), device="cuda").cpu().numpy().copy()
        self.rec_face, self.rec_texel = rec[:, 0], rec[:, 1]
        self.rec_l = rec[:, 2:].view(np.float32)
        self.target_np = self.target.cpu().numpy()

    def close(self):
        self.ctx.close()


@pytest.fixture(scope="module")
def small(oracle_lib):
    r = Run(dc.small_case(views=3, size=96, level=4, tex_size=32, seed=1))
    yield r
    r.close()


def test_visibility_matches_oracle(small):
    ref = dc.oracle_ids(small.sc)
    assert (ref != dc.NO_FACE).sum() > 1000
    assert np.array_equal(small.ids, ref)


def test_records_follow_visibility(small):
    vis = small.ids != dc.NO_FACE
    # every visible pixel is shaded (no corner behind the camera in this scene)
    assert np.array_equal(small.rec_face, small.ids)
    assert (small.rec_texel[vis] < small.sc.tex.shape[0] * small.sc.tex.shape[1]).all()
    l0, l1 = small.rec_l[vis, 0], small.rec_l[vis, 1]
    # pixel centres of the visible face lie (up to the integer snapping of the
    # visibility pass) inside it: barycentrics close to [0, 1]
    assert (l0 > -0.5).all() and (l1 > -0.5).all() and (l0 + l1 < 1.5).all()


def _compare(run):
    sc = run.sc
    views, world = dc.oracle_views(sc)
    params = dc.params_of(sc, world)
    ref = oracle.diff_eval(sc.mesh, views, params, run.ids, run.target_np, texel_in=run.rec_texel, image=True)
    errs = {
        "loss": abs(run.loss - ref["loss"]) / abs(ref["loss"]),
        "image": dc.rel_err(run.image.cpu().numpy(), ref["image"]),
        "g_pos": dc.rel_err(run.g[0].cpu().numpy()[:, :3], ref["g_pos"][:, :3]),
        "g_vcol": dc.rel_err(run.g[1].cpu().numpy(), ref["g_vcol"]),
        "g_tex": dc.rel_err(run.g[2].cpu().numpy(), ref["g_tex"]),
        "g_light": dc.rel_err(run.g_light, ref["g_light"]),
    }
    print("relative errors against the FP64 adjoint:", {k: f"{v:.2e}" for k, v in errs.items()})
    assert errs["loss"] <= LOSS_TOL
    assert errs["image"] <= GRAD_TOL
    for k in ("g_pos", "g_vcol", "g_tex", "g_light"):
        assert errs[k] <= GRAD_TOL, (k, errs[k])
    assert np.abs(run.g[0].cpu().numpy()[:, 3]).max() == 0.0  # w is not a parameter


def test_gradients_match_fp64_adjoint(small):
    _compare(small)


def test_backward_is_repeatable(small):
    """Gradients are overwritten, not accumulated, by a second backward."""
    before = [t.clone() for t in small.g]
    gl = small.diff.backward(*(t.data_ptr() for t in small.g))
    for a, b in zip(before, small.g):
        assert torch.allclose(a, b, rtol=1e-5, atol=1e-6 * float(a.abs().max()))
    assert np.allclose(gl, small.g_light, rtol=1e-5)


def test_misaligned_texture_gradient_rejected(small):
    """Texel gradients are accumulated as float4: a texture gradient buffer
    that is not 16-byte aligned is refused before any kernel runs."""
    big = torch.empty(small.g[2].numel() + 4, device="cuda")
    with pytest.raises(gr.GrError) as e:
        small.diff.backward(small.g[0].data_ptr(), small.g[1].data_ptr(), big.data_ptr() + 4)
    assert e.value.code == R.N.GR_ERR_INVALID_ARGUMENT and "aligned" in str(e.value)


def test_full_size_workload(oracle_lib):
    """64 views at 512x512 of the 81,920-face icosphere (the benchmark workload)."""
    run = Run(dc.small_case(views=64, size=512, level=6, tex_size=256, seed=0))
    try:
        assert np.array_equal(run.rec_face, run.ids)
        _compare(run)
    finally:
        run.close()


def test_single_view(oracle_lib):
    """One view: its visibility pass goes through the per-pixel resolve
    kernel (face ids from the keys) instead of the in-place tile resolve."""
    run = Run(dc.small_case(views=1, size=128, level=4, tex_size=32, seed=7))
    try:
        ref = dc.oracle_ids(run.sc)
        assert (ref != dc.NO_FACE).sum() > 500
        assert np.array_equal(run.ids, ref)
        _compare(run)
    finally:
        run.close()
