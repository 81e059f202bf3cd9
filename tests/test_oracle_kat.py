"""Known-answer tests of the CPU oracle, derived by hand from the Go sources.

The reference ships no golden vectors (its only test file holds two
benchmarks without assertions), so these cases restate, value by value, what
the Go code computes for small inputs: conversions, clipping, the top-left
rule, the degenerate-point quirk, texture wrapping and the matrices.
"""
import ctypes as C
import math

import numpy as np
import pytest

from oracle import oracle

L = None


@pytest.fixture(scope="module", autouse=True)
def lib(oracle_lib):
    global L
    L = oracle.lib()
    return L


def f32(x):
    return float(np.float32(x))


# ---- Go amd64 conversions (CVTTSS2SQ / CVTTSS2SL) ----

INT64_MIN = -(1 << 63)


@pytest.mark.parametrize("v,expect", [
    (1.9, 1), (-1.9, -1), (0.0, 0), (-0.0, 0), (1e10, 10000000000),
    (float("nan"), INT64_MIN), (float("inf"), INT64_MIN), (float("-inf"), INT64_MIN),
    (9.223372036854775808e18, INT64_MIN),       # 2^63 is out of range
    (-9.223372036854775808e18, INT64_MIN),      # -2^63 is in range and equals INT64_MIN
    (9.2233715e18, 9223371487098961920),        # largest float32 below 2^63
])
def test_go_int(v, expect):
    assert L.orc_go_int(v) == expect


@pytest.mark.parametrize("v,expect", [
    (255.9, 255), (256.5, 0), (0.99, 0), (-0.5, 0), (-1.5, 255), (-256.0, 0), (300.0, 44),
    (float("nan"), 0), (3e9, 0), (-3e9, 0), (2147483520.0, 128),
])
def test_go_uint8(v, expect):
    # uint8(float32) truncates to int32 (0x80000000 when out of range) and keeps the low byte
    assert L.orc_go_uint8(v) == expect


# ---- matrices (matrix.go) ----

def test_fov_constants():
    # float32(45 * (math.Pi / 180)) and float32(60 * (math.Pi / 180))
    assert np.float32(oracle.fov_radians(45)).view(np.uint32) == 0x3F490FDB
    assert np.float32(oracle.fov_radians(60)).view(np.uint32) == 0x3F860A92


def test_screen_matrix():
    m = oracle.screen_matrix(800, 600).reshape(4, 4)
    assert m.tolist() == [[400, 0, 0, 400], [0, 300, 0, 300], [0, 0, 0.5, 0.5], [0, 0, 0, 1]]


def test_perspective_matrix_znear_zero():
    # zNear = 0, zFar = 50: m22 = -1, m23 = -0 (matrix.go:97-98), so clip z = z_view
    # and clip w = -z_view exactly.
    fov = oracle.fov_radians(45)
    m = oracle.perspective_matrix(fov, f32(800 / 600), 0.0, 50.0).reshape(4, 4)
    th = np.float32(math.tan(np.float32(fov) / np.float32(2.0)))
    assert m[1, 1] == np.float32(1) / th
    assert m[0, 0] == np.float32(1) / (np.float32(f32(800 / 600)) * th)
    assert m[2, 2] == 1.0 and m[2, 3] == 0.0 and m[3, 2] == -1.0 and m[3, 3] == 0.0


def test_view_matrix_default_camera():
    # Camera{Position:(0,0,5), Direction:(0,0,-1), Up:(0,1,0)} (main.go): x axis = up x z = (-1,0,0)
    m = oracle.view_matrix((0, 0, 5), (0, 0, -1), (0, 1, 0)).reshape(4, 4)
    assert m[0, :3].tolist() == [-1, 0, 0] and m[1, :3].tolist() == [0, 1, 0]
    assert m[2].tolist() == [0, 0, -1, 5]


def test_world_matrix_identity_and_translation():
    w = oracle.world_matrix((1, 1, 1), (0, 0, 0), (1, 2, 3)).reshape(4, 4)
    assert w.tolist() == [[1, 0, 0, 1], [0, 1, 0, 2], [0, 0, 1, 3], [0, 0, 0, 1]]


def test_transform_batch_order():
    # ((m0*x + m1*y) + m2*z) + m3*w, no fused multiply-add
    m = np.eye(4, dtype=np.float32).reshape(-1).copy()
    m[0:4] = [1e8, 1.0, -1e8, 0.5]
    v = np.array([1.0, 3.0, 1.0, 1.0], np.float32)
    L.orc_transform_batch(oracle._fp(m), oracle._fp(v), 1)
    # 1e8 + 3 rounds back to 1e8 (ulp 8), so left-to-right gives 0.5; any
    # other association (or an FMA) would give 3.5 or 4.5
    x = np.float32(np.float32(np.float32(1e8) + np.float32(3.0)) + np.float32(-1e8)) + np.float32(0.5)
    assert v[0] == x == np.float32(0.5)


# ---- facing, frustum ----

def test_facing_camera():
    # clip-space triangle in front of the camera (w < 0 convention is irrelevant here:
    # facingCamera uses xyz only): normal . (0 - v0) > 0
    a = np.array([0, 0, 1, 1], np.float32)
    b = np.array([1, 0, 1, 1], np.float32)
    c = np.array([0, 1, 1, 1], np.float32)
    # (b-a) x (c-a) = (0,0,1); (0 - a) = (0,0,-1): dot = -1 -> not facing
    assert L.orc_facing_camera(oracle._fp(a), oracle._fp(b), oracle._fp(c)) == 0
    assert L.orc_facing_camera(oracle._fp(a), oracle._fp(c), oracle._fp(b)) == 1


def box(lo, hi, w):
    return np.array([[x, y, z, w] for x in (lo[0], hi[0]) for y in (lo[1], hi[1]) for z in (lo[2], hi[2])],
                    np.float32).reshape(-1)


def test_box_visibility():
    # inside: |x|,|y| <= -w ... with w = -2 (in front), x,y in [-1,1], z in [1,2]
    inside = box((-1, -1, 1), (1, 1, 2), -2.0)
    assert L.orc_box_visibility(oracle._fp(inside), 0.0, 50.0) == 2
    # behind the camera: z < 0 for every corner (Near plane) -> outside
    behind = box((-0.5, -0.5, -3), (0.5, 0.5, -1), 2.0)
    assert L.orc_box_visibility(oracle._fp(behind), 0.0, 50.0) == 0
    # straddling the near plane -> intersect
    straddle = box((-0.5, -0.5, -1), (0.5, 0.5, 1), -1.0)
    assert L.orc_box_visibility(oracle._fp(straddle), 0.0, 50.0) == 1


def clip(pts, uvs=None, inten=None):
    pts = np.asarray(pts, np.float32).reshape(-1)
    uvs = np.zeros(6, np.float32) if uvs is None else np.asarray(uvs, np.float32).reshape(-1)
    inten = np.zeros(3, np.float32) if inten is None else np.asarray(inten, np.float32)
    po = np.zeros(9 * 3 * 4, np.float32)
    uo = np.zeros(9 * 3 * 2, np.float32)
    io = np.zeros(9 * 3, np.float32)
    n = L.orc_clip_triangle(oracle._fp(pts), oracle._fp(uvs), oracle._fp(inten), None, 0.0, 50.0,
                            oracle._fp(po), oracle._fp(uo), oracle._fp(io), None)
    return n, po.reshape(9, 3, 4)[:max(n, 0)], uo.reshape(9, 3, 2)[:max(n, 0)], io.reshape(9, 3)[:max(n, 0)]


def test_clip_inside_is_identity():
    # a triangle inside every plane: six passes rotate [v0,v1,v2] back to itself
    tri = [[0.1, 0.1, 1, -1], [0.2, 0.1, 1, -1], [0.1, 0.3, 2, -2]]
    n, p, _, _ = clip(tri)
    assert n == 1 and np.array_equal(p[0], np.asarray(tri, np.float32))


def test_clip_behind_camera_hand_computed():
    # A0, A1 in front (w = -1), A2 behind (w = +1).  A point behind the camera
    # is outside the LEFT plane ((q-P).N = x + 1 + (w - 1) = 1 > 0), so the
    # left pass (the first) clips:
    #   edge A2->A1: u = A1-A2 = (.5,0,2,-2), w = A2-P = (1,0,-1,0),
    #     d = N.u = -1.5, n = -N.w = -1, f = float32(-1/-1.5) = 0.6666667,
    #     I1 = A2 + u*f = (0.33333334, 0, 0.33333337, -0.33333337)
    #   edge A0->A2: u = (0,0,-2,2), w = (1,0,1,-2), d = 2, n = 1, f = 0.5,
    #     I2 = (0, 0, 0, 0)
    # giving [A1, I1, I2, A0]; the other planes keep all four (rotating them)
    # and the fan is (I1, I2, A0), (I1, A0, A1).
    A0, A1, A2 = [0.0, 0.0, 1.0, -1.0], [0.5, 0.0, 1.0, -1.0], [0.0, 0.0, -1.0, 1.0]
    n, p, uv, inten = clip([A0, A1, A2], uvs=[[0, 0], [1, 0], [0, 1]], inten=[1.0, 1.0, 0.0])
    f = np.float32(-1.0) / np.float32(-1.5)
    I1 = [np.float32(0.5) * f, 0.0, np.float32(-1.0) + np.float32(2.0) * f, np.float32(1.0) - np.float32(2.0) * f]
    I2 = [0.0, 0.0, 0.0, 0.0]
    assert n == 2
    assert np.array_equal(p[0], np.array([I1, I2, A0], np.float32))
    assert np.array_equal(p[1], np.array([I1, A0, A1], np.float32))
    assert np.array_equal(inten, np.array([[f, 0.5, 1.0], [f, 1.0, 1.0]], np.float32))
    # lerpUV from A2 (0,1) toward A1 (1,0) by f; from A0 (0,0) toward A2 by 0.5
    assert np.array_equal(uv[0], np.array([[f, np.float32(1) + np.float32(-1) * f], [0, 0.5], [0, 0]], np.float32))


def test_clip_fully_outside_returns_zero():
    tri = [[0.0, 0.0, -1.0, 1.0], [0.5, 0.0, -2.0, 2.0], [0.0, 0.5, -1.5, 1.5]]
    n, _, _, _ = clip(tri)
    assert n == 0


# ---- rasterizer.go: Triangle ----

def raster(w, h, x0, y0, x1, y1, x2, y2, z=(-1.0, -1.0, -1.0), inten=(1.0, 1.0, 1.0), tex=None):
    rgba = np.zeros((h, w, 4), np.uint8)
    zb = np.full((h, w), -1.0, np.float32)
    L.orc_fb_triangle(rgba.ctypes.data, zb.ctypes.data, w, h,
                      x0, y0, z[0], 0.0, 0.0, x1, y1, z[1], 0.0, 0.0, x2, y2, z[2], 0.0, 0.0,
                      0, 0, w, h, inten[0], inten[1], inten[2], tex)
    return rgba, zb


def test_top_left_rule_square_split():
    # Two triangles sharing the diagonal of a 4x4 square, both wound so that
    # the inside has negative edge functions.  The top-left rule gives every
    # covered pixel to exactly one of them.
    W = H = 6
    ra, za = raster(W, H, 0, 0, 0, 4, 4, 0)
    rb, zb = raster(W, H, 4, 0, 0, 4, 4, 4)
    ca, cb = za > -1, zb > -1
    assert not (ca & cb).any()
    # hand count: (0,0),(0,4),(4,0): edge functions negative strictly inside or on
    # the kept edges
    assert ca.sum() + cb.sum() == 16
    # the opposite winding rasterises nothing
    _, zr = raster(W, H, 0, 0, 4, 0, 0, 4)
    assert (zr == -1).all()


def test_degenerate_point_quirk():
    # All three vertices at (3,3): every edge has dx = dy = 0, so the top-left
    # adjustment subtracts 1 from each and the single bbox pixel passes
    # fx < 0; alpha = beta = float32(-1)/float32(-3).
    rgba, zb = raster(8, 8, 3, 3, 3, 3, 3, 3, z=(-2.0, -2.0, -2.0), inten=(0.5, 0.5, 0.5))
    assert (zb > -1).sum() == 1 and zb[3, 3] > -1
    a = np.float32(-1.0) / np.float32(-3.0)
    g = np.float32(np.float32(1.0) - a) - a
    zr = -(np.float32(np.float32(a / np.float32(-2.0)) + np.float32(a / np.float32(-2.0))) + np.float32(g / np.float32(-2.0)))
    assert zb[3, 3] == np.float32(zr)
    i = np.float32(np.float32(a * np.float32(0.5)) + np.float32(a * np.float32(0.5))) + np.float32(g * np.float32(0.5))
    assert rgba[3, 3, 0] == int(np.float32(200.0) * i) and rgba[3, 3, 3] == 255


def test_depth_test_is_greater_equal():
    # the same triangle twice with different intensity: the second wins (>=)
    W = H = 8
    rgba = np.zeros((H, W, 4), np.uint8)
    zb = np.full((H, W), -1.0, np.float32)
    for inten in (1.0, 0.5):
        L.orc_fb_triangle(rgba.ctypes.data, zb.ctypes.data, W, H, 0, 0, -1.0, 0.0, 0.0, 0, 6, -1.0, 0.0, 0.0,
                          6, 0, -1.0, 0.0, 0.0, 0, 0, W, H, inten, inten, inten, None)
    cov = zb > -1
    assert cov.any() and (rgba[cov][:, 0] == 100).all()


# ---- texture.go ----

def make_tex(w, h, kind, scale=1.0):
    px = np.arange(w * h * 4, dtype=np.uint32).astype(np.uint8).reshape(h, w, 4)
    t = oracle.Texture()
    t.type, t.width, t.height, t.scale = kind, w, h, scale
    t.pixels = px.ctypes.data
    return t, px


def sample(t, u, v):
    out = (C.c_uint8 * 4)()
    L.orc_texture_sample(C.byref(t), u, v, out)
    return list(out)


def test_texture_fast_path_mask():
    t, px = make_tex(4, 4, 2)
    # x = int((1-u)*1*4) & 3; y = int(v*1*4) & 3
    assert sample(t, 0.0, 0.0) == px[0, int(4) & 3].tolist()
    assert sample(t, 0.6, 0.3) == px[int(np.float32(0.3) * 4) & 3, int((np.float32(1) - np.float32(0.6)) * 4) & 3].tolist()
    # u > 1 gives a negative x; the mask wraps it
    assert sample(t, 1.3, 0.0) == px[0, (-1) & 3].tolist()


def test_texture_modulo_path_negative_clamp():
    t, px = make_tex(3, 2, 1)
    flat = px.reshape(-1, 4)
    # (1 - 1.5)*3 = -1.5 -> int -1 -> % 3 = -1 (Go keeps the dividend's sign);
    # y = 0 -> idx = -1 -> clamped to 0
    assert sample(t, 1.5, 0.0) == flat[0].tolist()
    # y = int(0.6*2) = 1, x = int(0.5*3) % 3 = 1 -> idx 4
    assert sample(t, 0.5, 0.6) == flat[4].tolist()
    # x = -1, y = 1 -> idx = 1*3 - 1 = 2 (previous row's pixel, not clamped)
    assert sample(t, 1.5, 0.6) == flat[2].tolist()


def test_texture_solid():
    t = oracle.Texture()
    t.type = 0
    for i, c in enumerate((1, 2, 3, 4)):
        t.color[i] = c
    assert sample(t, 0.3, 0.7) == [1, 2, 3, 4]
