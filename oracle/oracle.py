"""ctypes binding of the CPU oracle (liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and the CPU
baseline leg of bench.py.  The product never imports this module.

Parity status: unpinned against the reference's own outputs (the reference has
no golden vectors and no Go toolchain exists here); see gorender_oracle.h.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import List, Optional, Sequence, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
SRC = os.path.join(HERE, "gorender_oracle.c")

CFLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread", "-Wall"]


def build(force: bool = False) -> str:
    """Compile the restatement with contraction disabled (gcc, any host arch)."""
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "gorender_oracle.h"))):
        tmp = LIB_PATH + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", *CFLAGS, "-o", tmp, SRC, "-lm"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


class Texture(C.Structure):
    _fields_ = [("type", C.c_int32), ("width", C.c_int32), ("height", C.c_int32),
                ("scale", C.c_float), ("color", C.c_uint8 * 4), ("pixels", C.c_void_p)]


class Mesh(C.Structure):
    _fields_ = [("pos", C.c_void_p), ("nv", C.c_int32), ("vnrm", C.c_void_p), ("nn", C.c_int32),
                ("fnrm", C.c_void_p), ("vidx", C.c_void_p), ("nidx", C.c_void_p),
                ("uv", C.c_void_p), ("tex", C.c_void_p), ("vcolor", C.c_void_p),
                ("nf", C.c_int32), ("bbox", C.c_float * 32)]


class Item(C.Structure):
    _fields_ = [("mesh", C.POINTER(Mesh)), ("mvp", C.c_float * 16), ("world", C.c_float * 16)]


class Frame(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("screen", C.c_float * 16),
                ("light", C.c_float * 3), ("flags", C.c_uint32),
                ("textures", C.POINTER(Texture)), ("ntextures", C.c_int32)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        fp = C.POINTER(C.c_float)
        L.orc_draw.argtypes = [C.POINTER(Item), C.c_int32, C.POINTER(Frame), C.c_void_p, C.c_void_p,
                               C.POINTER(C.c_int64), C.c_int32]
        L.orc_draw.restype = C.c_int
        L.orc_project.argtypes = [C.POINTER(Item), C.c_int32, C.POINTER(Frame), C.c_void_p, C.c_void_p, C.c_int64]
        L.orc_project.restype = C.c_int64
        L.orc_transform_batch.argtypes = [fp, fp, C.c_int64]
        L.orc_facing_camera.argtypes = [fp, fp, fp]
        L.orc_facing_camera.restype = C.c_int
        L.orc_box_visibility.argtypes = [fp, C.c_float, C.c_float]
        L.orc_box_visibility.restype = C.c_int
        L.orc_clip_triangle.argtypes = [fp, fp, fp, C.c_void_p, C.c_float, C.c_float, fp, fp, fp, C.c_void_p]
        L.orc_clip_triangle.restype = C.c_int
        L.orc_go_int.argtypes = [C.c_float]
        L.orc_go_int.restype = C.c_int64
        L.orc_go_uint8.argtypes = [C.c_float]
        L.orc_go_uint8.restype = C.c_uint8
        L.orc_texture_sample.argtypes = [C.POINTER(Texture), C.c_float, C.c_float, C.c_void_p]
        L.orc_fb_triangle.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32,
                                      C.c_int64, C.c_int64, C.c_float, C.c_float, C.c_float,
                                      C.c_int64, C.c_int64, C.c_float, C.c_float, C.c_float,
                                      C.c_int64, C.c_int64, C.c_float, C.c_float, C.c_float,
                                      C.c_int64, C.c_int64, C.c_int64, C.c_int64,
                                      C.c_float, C.c_float, C.c_float, C.POINTER(Texture)]
        L.orc_mesh_face_normals.argtypes = [fp, C.c_void_p, C.c_int32, fp]
        L.orc_mesh_bbox.argtypes = [fp, C.c_int32, fp]
        L.orc_world_matrix.argtypes = [fp, fp, fp, fp]
        L.orc_view_matrix.argtypes = [fp, fp, fp, fp]
        L.orc_perspective_matrix.argtypes = [C.c_float, C.c_float, C.c_float, C.c_float, fp]
        L.orc_screen_matrix.argtypes = [C.c_int32, C.c_int32, fp]
        L.orc_matrix_multiply.argtypes = [fp, fp, fp]
        L.orc_normalize3.argtypes = [fp, fp]
        _lib = L
    return _lib


def _fp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


# ---- matrices (matrix.go) ----

def world_matrix(scale, rot, trans) -> np.ndarray:
    out = np.zeros(16, np.float32)
    s, r, t = (np.asarray(v, np.float32) for v in (scale, rot, trans))
    lib().orc_world_matrix(_fp(s), _fp(r), _fp(t), _fp(out))
    return out


def view_matrix(eye, direction, up) -> np.ndarray:
    out = np.zeros(16, np.float32)
    e, d, u = (np.asarray(v, np.float32) for v in (eye, direction, up))
    lib().orc_view_matrix(_fp(e), _fp(d), _fp(u), _fp(out))
    return out


def perspective_matrix(fov: float, aspect: float, znear: float, zfar: float) -> np.ndarray:
    out = np.zeros(16, np.float32)
    lib().orc_perspective_matrix(fov, aspect, znear, zfar, _fp(out))
    return out


def screen_matrix(w: int, h: int) -> np.ndarray:
    out = np.zeros(16, np.float32)
    lib().orc_screen_matrix(w, h, _fp(out))
    return out


def matmul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    out = np.zeros(16, np.float32)
    lib().orc_matrix_multiply(_fp(np.ascontiguousarray(a, np.float32)),
                              _fp(np.ascontiguousarray(b, np.float32)), _fp(out))
    return out


def normalize3(v) -> np.ndarray:
    a = np.asarray(v, np.float32)
    out = np.zeros(3, np.float32)
    lib().orc_normalize3(_fp(a), _fp(out))
    return out


def fov_radians(deg: float) -> float:
    """float32(deg * (math.Pi / 180)) as the Go constant expression rounds it."""
    import fractions
    # pi to 40 digits; the exact rational product rounds once to float32
    pi = fractions.Fraction("3.141592653589793238462643383279502884197")
    val = fractions.Fraction(deg).limit_denominator(10 ** 12) * pi / 180
    f = np.float32(float(val))
    cands = [np.nextafter(f, np.float32(-np.inf)), f, np.nextafter(f, np.float32(np.inf))]
    return float(min(cands, key=lambda c: abs(fractions.Fraction(float(c)) - val)))


def object_matrices(obj, cam, width: int, height: int, fov: float) -> Tuple[np.ndarray, np.ndarray]:
    """(mvp, world) as projectObject builds them (renderer.go:255-262)."""
    aspect = np.float32(np.float32(width) / np.float32(height))
    w = world_matrix(obj.scale, obj.rotation, obj.translation)
    v = view_matrix(cam.position, cam.direction, cam.up)
    p = perspective_matrix(fov, float(aspect), 0.0, 50.0)
    ident = np.eye(4, dtype=np.float32).reshape(-1)
    mvp = matmul(ident, p)
    mvp = matmul(mvp, v)
    mvp = matmul(mvp, w)
    return mvp, w


# ---- meshes and draw ----

class _Keep:
    """Keeps numpy buffers alive while ctypes structs point at them."""

    def __init__(self):
        self.refs = []

    def arr(self, a, dtype):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=dtype)
        self.refs.append(a)
        return a


def face_normals(pos: np.ndarray, vidx: np.ndarray) -> np.ndarray:
    pos = np.ascontiguousarray(pos, np.float32)
    vidx = np.ascontiguousarray(vidx, np.int32)
    out = np.zeros((vidx.shape[0], 4), np.float32)
    lib().orc_mesh_face_normals(_fp(pos), vidx.ctypes.data, vidx.shape[0], _fp(out))
    return out


def bbox(pos: np.ndarray) -> np.ndarray:
    pos = np.ascontiguousarray(pos, np.float32)
    out = np.zeros((8, 4), np.float32)
    lib().orc_mesh_bbox(_fp(pos), pos.shape[0], _fp(out))
    return out


def make_mesh(m, keep: _Keep) -> Mesh:
    s = Mesh()
    pos = keep.arr(m.pos, np.float32)
    vidx = keep.arr(m.vidx, np.int32)
    s.pos = _ptr(pos)
    s.nv = pos.shape[0]
    vn = keep.arr(m.vnrm, np.float32)
    s.vnrm = _ptr(vn)
    s.nn = 0 if vn is None else vn.shape[0]
    fn = keep.arr(face_normals(pos, vidx), np.float32)
    s.fnrm = _ptr(fn)
    s.vidx = _ptr(vidx)
    s.nidx = _ptr(keep.arr(m.nidx, np.int32))
    s.uv = _ptr(keep.arr(m.uv, np.float32))
    s.tex = _ptr(keep.arr(m.tex, np.int32))
    s.vcolor = _ptr(keep.arr(m.vcolor, np.float32))
    s.nf = vidx.shape[0]
    bb = bbox(pos)
    for i in range(32):
        s.bbox[i] = float(bb.reshape(-1)[i])
    return s


def make_texture(t, keep: _Keep) -> Texture:
    s = Texture()
    s.type = t.kind
    s.width = t.width
    s.height = t.height
    s.scale = t.scale
    for i in range(4):
        s.color[i] = t.color[i]
    px = keep.arr(t.pixels, np.uint8)
    s.pixels = _ptr(px)
    return s


def _setup(scene, flags, light, items_override, keep):
    fov = fov_radians(scene.fov_deg)
    meshes = {}
    items = (Item * max(1, len(scene.objects)))()
    for i, o in enumerate(scene.objects):
        key = id(o.mesh)
        if key not in meshes:
            meshes[key] = make_mesh(o.mesh, keep)
        items[i].mesh = C.pointer(meshes[key])
        if items_override is not None:
            mvp, w = items_override[i]
        else:
            mvp, w = object_matrices(o, scene.camera, scene.width, scene.height, fov)
        for k in range(16):
            items[i].mvp[k] = float(mvp[k])
            items[i].world[k] = float(w[k])
    keep.refs.append(meshes)
    fr = Frame()
    fr.width = scene.width
    fr.height = scene.height
    sm = screen_matrix(scene.width, scene.height)
    for k in range(16):
        fr.screen[k] = float(sm[k])
    L = normalize3([-1.0, 1.0, 1.0]) if light is None else np.asarray(light, np.float32)
    for k in range(3):
        fr.light[k] = float(L[k])
    fr.flags = scene.flags if flags is None else flags
    texs = (Texture * max(1, len(scene.textures)))()
    for i, t in enumerate(scene.textures):
        texs[i] = make_texture(t, keep)
    keep.refs.append(texs)
    fr.textures = texs
    fr.ntextures = len(scene.textures)
    return items, fr


def project_scene(scene, flags=None, light=None, items_override=None):
    """Binned triangles of a scene: (xy int64 (n,3,2), w float32 (n,3))."""
    keep = _Keep()
    items, fr = _setup(scene, flags, light, items_override, keep)
    cap = 8 * max(1, scene.num_triangles)
    xy = np.zeros((cap, 3, 2), np.int64)
    w = np.zeros((cap, 3), np.float32)
    n = lib().orc_project(items, len(scene.objects), C.byref(fr), xy.ctypes.data, w.ctypes.data, cap)
    if n < 0:
        raise RuntimeError(f"orc_project failed: {n}")
    return xy[:n], w[:n]


def draw_scene(scene, nthreads: int = 1, flags: Optional[int] = None, light=None,
               items_override: Optional[Sequence[Tuple[np.ndarray, np.ndarray]]] = None):
    """Render a scenes.SceneData with the oracle.  Returns (rgba HxWx4, z HxW, tpf, status)."""
    keep = _Keep()
    fov = fov_radians(scene.fov_deg)
    meshes = {}
    items = (Item * max(1, len(scene.objects)))()
    for i, o in enumerate(scene.objects):
        key = id(o.mesh)
        if key not in meshes:
            meshes[key] = make_mesh(o.mesh, keep)
        items[i].mesh = C.pointer(meshes[key])
        if items_override is not None:
            mvp, w = items_override[i]
        else:
            mvp, w = object_matrices(o, scene.camera, scene.width, scene.height, fov)
        for k in range(16):
            items[i].mvp[k] = float(mvp[k])
            items[i].world[k] = float(w[k])
    fr = Frame()
    fr.width = scene.width
    fr.height = scene.height
    sm = screen_matrix(scene.width, scene.height)
    for k in range(16):
        fr.screen[k] = float(sm[k])
    L = normalize3([-1.0, 1.0, 1.0]) if light is None else np.asarray(light, np.float32)
    for k in range(3):
        fr.light[k] = float(L[k])
    fr.flags = scene.flags if flags is None else flags
    texs = (Texture * max(1, len(scene.textures)))()
    for i, t in enumerate(scene.textures):
        texs[i] = make_texture(t, keep)
    fr.textures = texs
    fr.ntextures = len(scene.textures)
    rgba = np.zeros((scene.height, scene.width, 4), np.uint8)
    z = np.zeros((scene.height, scene.width), np.float32)
    tpf = C.c_int64(0)
    st = lib().orc_draw(items, len(scene.objects), C.byref(fr), rgba.ctypes.data, z.ctypes.data,
                        C.byref(tpf), nthreads)
    return rgba, z, int(tpf.value), int(st)
