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
SOURCES = [SRC, os.path.join(HERE, "gorender_diff.c")]

CFLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread", "-Wall"]


def build(force: bool = False) -> str:
    """Compile the restatement with contraction disabled (gcc, any host arch)."""
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(
            [os.path.getmtime(f) for f in SOURCES] + [os.path.getmtime(os.path.join(HERE, "gorender_oracle.h"))]):
        tmp = LIB_PATH + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", *CFLAGS, "-o", tmp, *SOURCES, "-lm"])
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


class DiffScene(C.Structure):
    _fields_ = [("nv", C.c_int32), ("nf", C.c_int32), ("nn", C.c_int32), ("pos", C.c_void_p),
                ("vcol", C.c_void_p), ("vidx", C.c_void_p), ("nidx", C.c_void_p), ("vnrm", C.c_void_p),
                ("uv", C.c_void_p), ("tex", C.c_void_p), ("tw", C.c_int32), ("th", C.c_int32),
                ("light", C.c_double * 3), ("world", C.c_double * 16)]


class DiffView(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("screen", C.c_double * 16),
                ("mvp", C.c_double * 16)]


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
        L.orc_draw_ids.argtypes = [C.POINTER(Item), C.c_int32, C.POINTER(Frame), C.c_void_p, C.c_void_p,
                                   C.c_void_p, C.POINTER(C.c_int64), C.c_int32]
        L.orc_draw_ids.restype = C.c_int
        L.orc_diff_eval.argtypes = [C.POINTER(DiffScene), C.POINTER(DiffView), C.c_int32, C.c_void_p,
                                    C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_void_p]
        L.orc_diff_eval.restype = C.c_double
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
        L.orc_fb_line.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int64, C.c_int64, C.c_int64, C.c_int64,
                                  C.c_void_p]
        L.orc_fb_line.restype = C.c_int
        L.orc_fb_rect.argtypes = [C.c_void_p, C.c_int32, C.c_int32, C.c_int64, C.c_int64, C.c_int64, C.c_int64,
                                  C.c_void_p]
        L.orc_fog.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, C.c_float, C.c_float, C.c_void_p]
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
               items_override: Optional[Sequence[Tuple[np.ndarray, np.ndarray]]] = None, face_ids: bool = False):
    """Render a scenes.SceneData with the oracle.  Returns (rgba HxWx4, z HxW, tpf, status), plus the
    per-pixel face ids (uint32 HxW) when face_ids is set."""
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
    if face_ids:
        ids = np.zeros((scene.height, scene.width), np.uint32)
        st = lib().orc_draw_ids(items, len(scene.objects), C.byref(fr), rgba.ctypes.data, z.ctypes.data,
                                ids.ctypes.data, C.byref(tpf), nthreads)
        return rgba, z, int(tpf.value), int(st), ids
    st = lib().orc_draw(items, len(scene.objects), C.byref(fr), rgba.ctypes.data, z.ctypes.data,
                        C.byref(tpf), nthreads)
    return rgba, z, int(tpf.value), int(st)


def fog(rgba: np.ndarray, z: np.ndarray, fog_start: float, fog_end: float, color) -> np.ndarray:
    """FrameBuffer.Fog on a copy of rgba (H x W x 4 uint8) with z (H x W float32)."""
    out = np.ascontiguousarray(rgba, np.uint8).copy()
    zz = np.ascontiguousarray(z, np.float32)
    col = (C.c_uint8 * 4)(*color)
    lib().orc_fog(out.ctypes.data, zz.ctypes.data, out.shape[1], out.shape[0], fog_start, fog_end, col)
    return out


# ---- differentiable shading extension (FP64) ----

def diff_eval(mesh, views, params, ids: np.ndarray, target: np.ndarray, texel_in: Optional[np.ndarray] = None,
              grads: bool = True, image: bool = False):
    """FP64 loss (and gradients) of the differentiable shading model.

    mesh: scenes.MeshData (vidx, nidx, vnrm, uv); views: list of (width, height, screen16, mvp16);
    params: dict with pos (nv x 4), vcol (nv x 3), tex (th x tw x 4 or None), light (3), world (16),
    any float dtype (converted to float64); ids, target: per pixel over all views.
    Returns dict(loss, texel, image?, g_pos, g_vcol, g_tex, g_light)."""
    keep = []

    def d64(a):
        if a is None:
            return None
        a = np.ascontiguousarray(np.asarray(a, np.float64))
        keep.append(a)
        return a

    def i32(a):
        a = np.ascontiguousarray(np.asarray(a, np.int32))
        keep.append(a)
        return a

    s = DiffScene()
    pos, vcol = d64(params["pos"]), d64(params["vcol"])
    tex = d64(params.get("tex"))
    s.nv = pos.shape[0]
    s.nf = mesh.vidx.shape[0]
    s.nn = mesh.vnrm.shape[0]
    s.pos, s.vcol = pos.ctypes.data, vcol.ctypes.data
    s.vidx = i32(mesh.vidx).ctypes.data
    s.nidx = i32(mesh.nidx).ctypes.data
    s.vnrm = d64(mesh.vnrm).ctypes.data
    uv = d64(mesh.uv) if mesh.uv is not None else None
    s.uv = None if uv is None else uv.ctypes.data
    s.tex = None if tex is None else tex.ctypes.data
    s.th, s.tw = (0, 0) if tex is None else (tex.shape[0], tex.shape[1])
    for k in range(3):
        s.light[k] = float(params["light"][k])
    for k in range(16):
        s.world[k] = float(params["world"][k])
    vs = (DiffView * len(views))()
    for i, (w, h, sm, mvp) in enumerate(views):
        vs[i].width, vs[i].height = w, h
        for k in range(16):
            vs[i].screen[k] = float(sm[k])
            vs[i].mvp[k] = float(mvp[k])
    npx = sum(w * h for w, h, _, _ in views)
    ids = np.ascontiguousarray(ids, np.uint32).reshape(-1)
    target = np.ascontiguousarray(target, np.float32).reshape(-1)
    assert ids.size == npx and target.size == 4 * npx
    texel = np.zeros(npx, np.uint32)
    tin = None if texel_in is None else np.ascontiguousarray(texel_in, np.uint32).reshape(-1)
    img = np.zeros((npx, 4), np.float64) if image else None
    out = {}
    gp = np.zeros((s.nv, 4)) if grads else None
    gc = np.zeros((s.nv, 3)) if grads else None
    gt = np.zeros_like(tex) if (grads and tex is not None) else None
    gl = np.zeros(3) if grads else None
    out["loss"] = lib().orc_diff_eval(C.byref(s), vs, len(views), ids.ctypes.data, _ptr(tin),
                                      texel.ctypes.data, target.ctypes.data, _ptr(img), _ptr(gp), _ptr(gc),
                                      _ptr(gt), _ptr(gl))
    out["texel"] = texel if tin is None else tin
    if image:
        out["image"] = img
    if grads:
        out.update(g_pos=gp, g_vcol=gc, g_tex=gt, g_light=gl)
    return out
