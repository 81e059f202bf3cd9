"""CPU-only checks of the product library and the host side: the C-ABI loads
and exports every declared symbol, the host matrix/mesh math (matrix.go,
mesh.go restated in C++) equals the oracle's restatement bit for bit, and the
scene generators are deterministic."""
import ctypes as C
import hashlib
import os
import re

import numpy as np
import pytest

import gorender_gb300 as gr
from gorender_gb300 import _native as N
from gorender_gb300 import scenes
from oracle import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def built(oracle_lib):
    from gorender_gb300 import build
    build.build()
    return N.lib()


def header_functions():
    src = open(os.path.join(ROOT, "include", "gorender_cuda.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(gr_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    L = N.lib()
    names = header_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(names) == set(N.EXPORTS)


def test_version_and_errors_without_gpu():
    L = N.lib()
    assert b"sm_103a" in L.gr_version()
    # NULL arguments are rejected with a status, never a crash
    assert L.gr_context_sync(None) == N.GR_ERR_INVALID_ARGUMENT
    assert L.gr_draw(None, None, 0, None, None, None, None) == N.GR_ERR_INVALID_ARGUMENT
    assert b"NULL" in L.gr_last_error()


def test_context_create_reports_missing_device():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    h = C.c_void_p()
    st = N.lib().gr_context_create(0, C.byref(h))
    assert st in (N.GR_ERR_NO_DEVICE, N.GR_ERR_CUDA)


def test_object_matrices_match_oracle():
    rng = np.random.default_rng(7)
    for _ in range(50):
        s = rng.uniform(0.2, 2.0, 3).astype(np.float32)
        r = rng.uniform(-3, 3, 3).astype(np.float32)
        r[rng.integers(0, 3)] = 0.0  # zero angles take the identity branch
        t = rng.uniform(-5, 5, 3).astype(np.float32)
        eye = rng.uniform(-5, 5, 3).astype(np.float32)
        d = rng.normal(size=3).astype(np.float32)
        W, H = int(rng.integers(64, 2000)), int(rng.integers(64, 2000))
        fov = oracle.fov_radians(float(rng.uniform(30, 90)))
        mvp, world = gr.object_matrices(s, r, t, eye, d, (0, 1, 0), W, H, fov)
        obj = scenes.ObjectData(None, tuple(s), tuple(r), tuple(t))
        cam = scenes.CameraData(tuple(eye), tuple(d), (0.0, 1.0, 0.0))
        mvp2, world2 = oracle.object_matrices(obj, cam, W, H, fov)
        assert np.array_equal(mvp.view(np.uint32), mvp2.view(np.uint32))
        assert np.array_equal(world.view(np.uint32), world2.view(np.uint32))


def test_object_matrices_match_oracle_large_and_demo_angles():
    """Rotation angles beyond 2^29 (Go's Payne-Hanek reduction), negative ones
    and the demo mode's accumulated turns: the library's restatement of Go's
    sin/cos/tan gives the oracle's matrices bit for bit."""
    rng = np.random.default_rng(17)
    big = [float(np.float32(s * 2.0 ** e)) for s, e in zip(rng.choice([-1, 1], 60), rng.uniform(20, 120, 60))]
    demo = [float(np.float32(k * 0.01)) for k in range(0, 700, 23)]
    for a in big + demo:
        r = np.array([a, -a * 0.5, a * 0.25], np.float32)
        fov = oracle.fov_radians(45.0)
        mvp, world = gr.object_matrices((1, 1, 1), r, (0, 0, 0), (0, 0, 5), (0, 0, -1), (0, 1, 0), 800, 600, fov)
        obj = scenes.ObjectData(None, (1.0, 1.0, 1.0), tuple(r), (0.0, 0.0, 0.0))
        cam = scenes.CameraData((0.0, 0.0, 5.0), (0.0, 0.0, -1.0), (0.0, 1.0, 0.0))
        mvp2, world2 = oracle.object_matrices(obj, cam, 800, 600, fov)
        assert np.array_equal(mvp.view(np.uint32), mvp2.view(np.uint32)), a
        assert np.array_equal(world.view(np.uint32), world2.view(np.uint32)), a


def _box_corners(lo, hi):
    """Mesh.BoundingBox's 8 corners (x outermost, then y, then z; w = 1)."""
    c = np.zeros((8, 4), np.float32)
    for k in range(8):
        c[k] = [hi[0] if k & 4 else lo[0], hi[1] if k & 2 else lo[1], hi[2] if k & 1 else lo[2], 1.0]
    return c


def test_box_visibility_matches_oracle():
    """Frustum.BoxVisibility of a transformed bounding box (clipping.go:131-154,
    renderer.go:268-275), which gr_draw now decides on the host for each draw
    item: the library's function against the oracle's transform + classify,
    on object matrices around a camera (boxes inside, straddling each plane,
    behind the camera, beyond zFar) and on raw matrices with extreme and
    non-finite entries."""
    L = N.lib()
    O = oracle.lib()
    rng = np.random.default_rng(23)
    seen = set()

    def fptr(a):
        return a.ctypes.data_as(C.POINTER(C.c_float))

    def check(mvp, box):
        mvp = np.ascontiguousarray(mvp, np.float32)
        box = np.ascontiguousarray(box, np.float32)
        out = C.c_int32()
        assert L.gr_box_visibility(fptr(mvp), fptr(box), C.byref(out)) == N.GR_OK
        corners = box.copy()  # the oracle transforms the corners in place, then classifies them
        O.orc_transform_batch(fptr(mvp), fptr(corners), 8)
        ref = O.orc_box_visibility(fptr(corners), C.c_float(0.0), C.c_float(50.0))
        assert out.value == ref, (mvp, box, out.value, ref)
        seen.add(ref)

    for _ in range(3000):
        s = rng.uniform(0.05, 4.0, 3).astype(np.float32)
        r = rng.uniform(-3, 3, 3).astype(np.float32)
        t = rng.uniform(-30, 30, 3).astype(np.float32)
        eye = rng.uniform(-10, 10, 3).astype(np.float32)
        d = rng.normal(size=3).astype(np.float32)
        fov = oracle.fov_radians(float(rng.uniform(30, 90)))
        mvp, _ = gr.object_matrices(s, r, t, eye, d, (0, 1, 0), 1280, 720, fov)
        lo = rng.uniform(-2, 0, 3).astype(np.float32)
        check(mvp, _box_corners(lo, lo + rng.uniform(0, 3, 3).astype(np.float32)))
    assert seen == {0, 1, 2}
    for _ in range(500):
        mvp = rng.normal(size=16).astype(np.float32) * np.float32(10.0) ** rng.integers(-6, 7, 16)
        mvp[rng.integers(0, 16)] = rng.choice([np.inf, -np.inf, np.nan, 0.0, 1e38])
        lo = rng.uniform(-1e3, 1e3, 3).astype(np.float32)
        check(mvp, _box_corners(lo, lo + np.float32(rng.uniform(0, 1e3))))


def test_screen_matrix_light_fov_match_oracle():
    for w, h in [(640, 360), (1280, 720), (1920, 1080), (643, 357)]:
        assert np.array_equal(gr.screen_matrix(w, h), oracle.screen_matrix(w, h))
    assert np.array_equal(gr.default_light(), oracle.normalize3([-1.0, 1.0, 1.0]))
    for deg in (45, 60, 75):
        assert gr.fov_radians(deg) == oracle.fov_radians(deg)


@pytest.mark.parametrize("make", [lambda: scenes.uv_sphere(32, 16), lambda: scenes.heightfield(65, seed=3),
                                  lambda: scenes.icosphere(3, noise=0.05, seed=2)])
def test_face_normals_match_oracle_and_numpy(make):
    m = make()
    a = gr.face_normals(m.pos, m.vidx)
    b = oracle.face_normals(m.pos, m.vidx)
    c = m.face_normals()
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert np.array_equal(a.view(np.uint32), c.view(np.uint32))


def test_bad_indices_rejected_on_host():
    pos = np.ones((3, 4), np.float32)
    bad = np.array([[0, 1, 3]], np.int32)
    out = np.zeros((1, 4), np.float32)
    st = N.lib().gr_mesh_face_normals(pos.ctypes.data, 3, bad.ctypes.data, 1, out.ctypes.data)
    assert st == N.GR_ERR_BAD_INDEX


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        if a is not None:
            h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()[:16]


def test_generators_deterministic():
    # fixed digests: the generators use splitmix64 and a fixed Taylor series,
    # so x86 and Arm hosts build identical meshes
    sph = scenes.uv_sphere(32, 16)
    assert sph.nf == 960 and sph.nv == 482
    hf = scenes.heightfield(317, seed=0)
    assert hf.nf == 199712 and hf.nv == 100489
    ico5 = scenes.icosphere(5)
    assert ico5.nf == 20480 and ico5.nv == 10242
    assert scenes.icosphere(6).nf == 81920
    assert digest(sph.pos, sph.vidx) == digest(scenes.uv_sphere(32, 16).pos, scenes.uv_sphere(32, 16).vidx)
    tex = scenes.random_texture(16, 16, seed=1)
    assert tex.kind == 2 and (tex.pixels[..., 3] == 255).all()


def test_splitmix64_reference_values():
    # splitmix64 with seed 0: first outputs of the published generator
    z = scenes.SplitMix64(0).next_u64(3)
    assert [int(v) for v in z] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]


def test_oracle_threads_identical():
    sc = scenes.scene_heightfield_1280x720(n=97)
    a = oracle.draw_scene(sc, nthreads=1)
    b = oracle.draw_scene(sc, nthreads=7)
    assert a[3] == 0 and b[3] == 0 and a[2] == b[2]
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32))
