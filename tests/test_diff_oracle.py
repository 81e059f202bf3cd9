"""The FP64 adjoint of the differentiable shading model (oracle) against
central finite differences of the FP64 loss, h = 1e-3 (and h = 1e-6 for
positions, whose h = 1e-3 differences carry an O(h^2) truncation error), with
visibility and texel choices frozen at the base point (the gradients are
defined for fixed visibility and texel choices).  CPU only."""
import numpy as np
import pytest

from oracle import oracle
from tests import diff_cases as dc

H = 1e-3


@pytest.fixture(scope="module")
def case(oracle_lib):
    sc = dc.small_case(views=2, size=64, level=2, tex_size=16, seed=3)
    views, world = dc.oracle_views(sc)
    ids = dc.oracle_ids(sc)
    # target: the perturbed parameters over their own visibility
    tgt_ids = dc.oracle_ids(sc, sc.target_params["pos"])
    tp = dc.params_of(sc, world, target=True)
    npx = ids.size
    tgt = oracle.diff_eval(sc.mesh, views, tp, tgt_ids, np.zeros((npx, 4), np.float32), grads=False, image=True)
    target = tgt["image"].astype(np.float32)
    params = {k: (np.array(v, np.float64) if k != "world" else v) for k, v in dc.params_of(sc, world).items()}
    base = oracle.diff_eval(sc.mesh, views, params, ids, target)
    return sc, views, ids, target, params, base


def _loss(case, params):
    sc, views, ids, target, _, base = case
    return oracle.diff_eval(sc.mesh, views, params, ids, target, texel_in=base["texel"], grads=False)["loss"]


def _fd(case, key, index, h=H):
    params = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in case[4].items()}
    flat = params[key].reshape(-1)
    x0 = flat[index]
    flat[index] = x0 + h
    lp = _loss(case, params)
    flat[index] = x0 - h
    lm = _loss(case, params)
    return (lp - lm) / (2 * h)


def test_case_has_visible_shaded_pixels(case):
    sc, views, ids, target, params, base = case
    assert (ids != dc.NO_FACE).sum() > 1000
    assert base["loss"] > 0
    assert (base["texel"] != dc.NO_FACE).sum() > 1000


@pytest.mark.parametrize("key,gkey", [("vcol", "g_vcol"), ("tex", "g_tex"), ("light", "g_light"),
                                      ("pos", "g_pos")])
def test_adjoint_matches_finite_differences(case, key, gkey):
    g = case[5][gkey].reshape(-1)
    size = case[4][key].size
    if key == "pos":
        # x, y, z of vertices (w is not a parameter)
        cand = np.array([i for i in range(size) if i % 4 != 3 and g[i] != 0.0])
    else:
        cand = np.nonzero(g)[0]
    assert cand.size > 0
    rng = np.random.default_rng(7)
    picks = cand if cand.size <= 24 else rng.choice(cand, 24, replace=False)
    # include the largest entries, where the derivative matters most
    picks = np.unique(np.concatenate([picks, cand[np.argsort(-np.abs(g[cand]))[:4]]]))
    scale = np.abs(g).max()
    for i in picks:
        fd = _fd(case, key, int(i))
        if key != "pos":
            # the loss is quadratic in colours, texels and the light: central
            # differences are exact up to rounding
            assert abs(fd - g[i]) <= 1e-7 * scale, (key, int(i), fd, g[i], scale)
            continue
        # positions enter through the barycentrics (rational functions, with
        # kinks where the clip to the face switches a barycentric off): the
        # h = 1e-3 difference carries an O(h^2) truncation error and, near a
        # kink, a one-sided slope mix, so it is held to a loose bound; h = 1e-6
        # pins the adjoint.
        assert abs(fd - g[i]) <= 2e-2 * scale, (key, int(i), fd, g[i], scale)
        fd6 = _fd(case, key, int(i), 1e-6)
        assert abs(fd6 - g[i]) <= 1e-6 * scale, (key, int(i), fd6, g[i], scale)
