"""Known-answer tests of the oracle's overlay primitives, derived by hand from
FrameBuffer.Pixel / Line / Rect (rasterizer.go:25-30, 54-79) and utils.go abs:

* Pixel writes by linear index y*W + x: index 0 is never written, and an x
  outside the row wraps into a neighbouring row;
* Line steps x and y by float32(d)/float32(side) accumulated one add at a
  time and truncates each point with int();
* Rect returns early only for x >= W or y >= H.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle

W, H = 8, 4
MARK = (C.c_uint8 * 4)(9, 9, 9, 255)


@pytest.fixture(scope="module", autouse=True)
def lib(oracle_lib):
    return oracle.lib()


def _buf():
    return np.zeros((H, W, 4), np.uint8)


def _marked(b):
    return {(int(x), int(y)) for y, x in zip(*np.nonzero(b[..., 0] == 9))}


def _line(x0, y0, x1, y1):
    b = _buf()
    st = oracle.lib().orc_fb_line(b.ctypes.data, W, H, x0, y0, x1, y1, MARK)
    return st, _marked(b)


def test_line_skips_index_zero():
    # (0,0)->(3,1): steps x 1, y 1/3 (0.33333334f); y reaches 1.0f exactly at the end
    st, px = _line(0, 0, 3, 1)
    assert st == 0 and px == {(1, 0), (2, 0), (3, 1)}


def test_line_wraps_negative_x_into_previous_row():
    # x = -3..-1 on row 1 are linear indices 5..7 of row 0
    st, px = _line(-3, 1, 3, 1)
    assert st == 0 and px == {(5, 0), (6, 0), (7, 0), (0, 1), (1, 1), (2, 1), (3, 1)}


def test_line_truncates_toward_zero():
    # (0,1)->(-2,0): points (0,1), (-1.0, 0.5) -> (-1, 0), (-2, 0): negative indices
    st, px = _line(0, 1, -2, 0)
    assert st == 0 and px == {(0, 1)}


def test_line_single_point():
    # side 0: the steps are 0/0 (NaN) but only the first point is plotted
    st, px = _line(2, 2, 2, 2)
    assert st == 0 and px == {(2, 2)}


def test_line_too_long_is_refused():
    st, px = _line(0, 0, 1 << 23, 0)
    assert st == -6 and px == set()


def test_line_steep():
    # (1,0)->(2,3): side 3, x step 1/3, y step 1
    st, px = _line(1, 0, 2, 3)
    assert st == 0 and px == {(1, 0), (1, 1), (1, 2), (2, 3)}


def test_rect_wraps_and_clips_by_index():
    b = _buf()
    oracle.lib().orc_fb_rect(b.ctypes.data, W, H, -1, 2, 3, 3, MARK)
    # rows 2..4, x -1..1 -> indices 15..17, 23..25, 31..33; x = -1 wraps to the
    # row above, and of row 4 only index 31 (x = -1) is inside the buffer
    assert _marked(b) == {(7, 1), (0, 2), (1, 2), (7, 2), (0, 3), (1, 3), (7, 3)}


def test_rect_early_return():
    b = _buf()
    oracle.lib().orc_fb_rect(b.ctypes.data, W, H, W, 0, 3, 3, MARK)
    oracle.lib().orc_fb_rect(b.ctypes.data, W, H, 0, H, 3, 3, MARK)
    assert _marked(b) == set()


def test_rect_at_origin_skips_index_zero():
    b = _buf()
    oracle.lib().orc_fb_rect(b.ctypes.data, W, H, -1, -1, 3, 3, MARK)
    # y = -1: indices -9..-7 (none); y = 0: -1 (none), 0 (skipped), 1; y = 1: 7, 8, 9
    assert _marked(b) == {(1, 0), (7, 0), (0, 1), (1, 1)}


# ---- FrameBuffer.Fog (rasterizer.go:185-207) ----

def test_fog_hand_computed():
    # start 1.0, end 0.0: depth 0.25 blends with f = 1 - (0 - 0.25) / (0 - 1) = 0.75 (exact)
    rgba = np.array([[[200, 100, 50, 255], [200, 100, 50, 255], [200, 100, 50, 255], [200, 100, 50, 255],
                      [10, 20, 30, 40]]], np.uint8)
    z = np.array([[0.25, 1.0, 0.0, -1.0, float("nan")]], np.float32)
    out = oracle.fog(rgba, z, 1.0, 0.0, (100, 100, 100, 255))
    # 200*.25 + 100*.75 = 125; 100; 50*.25 + 75 = 87.5 -> 87; 255*.25 + 255*.75 = 255
    assert out[0, 0].tolist() == [125, 100, 87, 255]
    assert out[0, 1].tolist() == [200, 100, 50, 255]   # depth >= start: unchanged
    assert out[0, 2].tolist() == [100, 100, 100, 255]  # depth <= end: fog colour
    assert out[0, 3].tolist() == [100, 100, 100, 255]  # background (Z = -1)
    assert out[0, 4].tolist() == [0, 0, 0, 0]          # NaN depth: f = NaN, uint8(NaN) = 0
