"""Go's math.Sin / math.Cos / math.Tan as restated in the oracle (and, through
the matrices, in the library's host math): math32.go:15-25 round them to
float32 for the rotation (matrix.go:32-72) and perspective (matrix.go:93)
matrices.  No Go toolchain exists here, so the restatement is checked against
what the published algorithm guarantees: its error against correctly rounded
values (mpmath at 300 bits), exact octants of the Payne-Hanek reduction, the
special cases, and the float32 values of the angles the scenes use."""
import ctypes as C
import math
import struct
from fractions import Fraction

import numpy as np
import pytest

from oracle import oracle

mpmath = pytest.importorskip("mpmath")


@pytest.fixture(scope="module")
def L(oracle_lib):
    lib = C.CDLL(oracle.LIB_PATH)
    for n in ("orc_go_sin", "orc_go_cos", "orc_go_tan"):
        getattr(lib, n).restype = C.c_double
        getattr(lib, n).argtypes = [C.c_double]
    return lib


def ulps(a, b):
    ia = struct.unpack("<q", struct.pack("<d", a))[0]
    ib = struct.unpack("<q", struct.pack("<d", b))[0]
    return abs(ia - ib)


def angles():
    rng = np.random.default_rng(5)
    xs = rng.uniform(-8.0, 8.0, 3000).astype(np.float32).tolist()
    xs += [float(np.float32(k * np.float32(0.01))) for k in range(-700, 700, 7)]
    # fov/2 of the reference's 45 degrees (renderer.go:118) and of 60 degrees
    for deg in (45.0, 60.0, 75.0):
        xs.append(float(np.float32(np.float32(oracle.fov_radians(deg)) / np.float32(2.0))))
    xs += [float(np.float32(math.pi / 4)), float(np.float32(math.pi / 2)), float(np.float32(math.pi))]
    return xs


def test_error_against_correctly_rounded(L):
    mpmath.mp.prec = 300
    for name, ref, bound in (("orc_go_sin", mpmath.sin, 1), ("orc_go_cos", mpmath.cos, 1), ("orc_go_tan", mpmath.tan, 2)):
        f = getattr(L, name)
        for x in angles():
            t = ref(mpmath.mpf(x))
            if x == 0.0:
                assert f(x) == float(t)
                continue
            if name == "orc_go_tan" and min(abs(t), 1 / abs(t)) < 1.1e-7:
                # z*z <= 1e-14: tan returns the reduced argument z (or -1/z)
                # itself, without its cubic term: relative error z^2/3
                assert abs(f(x) - float(t)) <= 1e-14 * abs(float(t)), x
                continue
            assert ulps(f(x), float(t)) <= bound, f"{name}({x})"


def test_special_cases(L):
    for f in (L.orc_go_sin, L.orc_go_tan):
        assert struct.pack("<d", f(0.0)) == struct.pack("<d", 0.0)
        assert struct.pack("<d", f(-0.0)) == struct.pack("<d", -0.0)
        assert math.isnan(f(math.inf)) and math.isnan(f(-math.inf)) and math.isnan(f(math.nan))
    assert L.orc_go_cos(0.0) == 1.0 and L.orc_go_cos(-0.0) == 1.0
    assert math.isnan(L.orc_go_cos(math.inf)) and math.isnan(L.orc_go_cos(math.nan))


def test_huge_arguments_payne_hanek(L):
    """From 2^29 Go reduces with the bits of 4/pi (Payne-Hanek): the result is
    within a few 1e-16 of the true value in absolute terms (the reduced
    argument is truncated to 53 bits of a fraction of pi/4)."""
    mpmath.mp.prec = 300
    rng = np.random.default_rng(9)
    xs = [float(np.float32(2.0 ** e)) for e in rng.uniform(29, 127, 400)]
    xs += [float(np.float32(2.0 ** 29)), float(np.finfo(np.float32).max)]
    for x in xs:
        for f, ref in ((L.orc_go_sin, mpmath.sin), (L.orc_go_cos, mpmath.cos)):
            assert abs(f(x) - float(ref(mpmath.mpf(x)))) < 5e-16, x
            assert abs(f(-x) + (f(x) if f is L.orc_go_sin else -f(x))) == 0.0


def test_float32_results_of_scene_angles(L):
    """float32(Go's sin/cos/tan) of the angles the scenes pass, against the
    correctly rounded float32 (the double-rounding hazard of a different libm
    shows up here first)."""
    mpmath.mp.prec = 300
    for x in angles():
        for f, ref in ((L.orc_go_sin, mpmath.sin), (L.orc_go_cos, mpmath.cos), (L.orc_go_tan, mpmath.tan)):
            got = np.float32(f(x))
            exact = Fraction(str(ref(mpmath.mpf(x))))
            lo, hi = np.nextafter(got, np.float32(-np.inf)), np.nextafter(got, np.float32(np.inf))
            # got is the float32 nearest the true value, or a neighbour of it
            # only when the true value lies within 2^-50 of a rounding midpoint
            assert abs(Fraction(float(got)) - exact) <= max(abs(Fraction(float(lo)) - exact),
                                                           abs(Fraction(float(hi)) - exact)), x
