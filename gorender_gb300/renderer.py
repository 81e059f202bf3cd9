"""Host mirror of gorender's Renderer / FrameBuffer / Mesh / Object / Camera API
over the C-ABI (renderer.go, rasterizer.go, mesh.go, texture.go).

    ctx = Context(0)
    mesh = ctx.mesh(meshdata)                    # NewMesh + upload
    r = Renderer(ctx, 1280, 720)                 # NewFrameBuffer + NewRenderer
    r.FlatShading = True                         # the exported Renderer flags
    r.draw([Object(mesh)], Camera(...))          # (*Renderer).Draw
    rgba, z = r.pixels(), r.zbuffer()            # FrameBuffer.Pixels / ZBuffer
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _native as N
from .scenes import MeshData, SceneData, TextureData

FRUSTUM_CLIPPING = 0x01
SHOW_FACES = 0x02
BACKFACE_CULLING = 0x04
LIGHTING = 0x08
FLAT_SHADING = 0x10
SHOW_TEXTURES = 0x20
SHOW_EDGES = 0x40
SHOW_VERTICES = 0x80
CROSSHAIR = 0x100  # FrameBuffer.CrossHair after the scene (the reference's demoMode off)
FLAGS_DEFAULT = FRUSTUM_CLIPPING | SHOW_FACES | BACKFACE_CULLING | LIGHTING | SHOW_TEXTURES


def _ptr(a: Optional[np.ndarray]):
    return None if a is None else a.ctypes.data


def _fp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


# ---- host math (matrix.go restated in C++ inside the library) ----

def object_matrices(scale, rotation, translation, cam_pos, cam_dir, cam_up, width: int, height: int,
                    fov_y: float) -> Tuple[np.ndarray, np.ndarray]:
    o = N.Object()
    for k in range(3):
        o.scale[k] = scale[k]
        o.rotation[k] = rotation[k]
        o.translation[k] = translation[k]
    cam = N.Camera()
    for k in range(3):
        cam.position[k] = cam_pos[k]
        cam.direction[k] = cam_dir[k]
        cam.up[k] = cam_up[k]
    mvp = np.zeros(16, np.float32)
    world = np.zeros(16, np.float32)
    N.check(N.lib().gr_object_matrices(C.byref(o), C.byref(cam), width, height, fov_y, _fp(mvp), _fp(world)))
    return mvp, world


def screen_matrix(width: int, height: int) -> np.ndarray:
    out = np.zeros(16, np.float32)
    N.check(N.lib().gr_screen_matrix(width, height, _fp(out)))
    return out


def normalize3(v) -> np.ndarray:
    a = np.asarray(v, np.float32)
    out = np.zeros(3, np.float32)
    N.check(N.lib().gr_normalize3(_fp(a), _fp(out)))
    return out


def face_normals(pos: np.ndarray, vidx: np.ndarray) -> np.ndarray:
    pos = np.ascontiguousarray(pos, np.float32)
    vidx = np.ascontiguousarray(vidx, np.int32)
    out = np.zeros((vidx.shape[0], 4), np.float32)
    N.check(N.lib().gr_mesh_face_normals(pos.ctypes.data, pos.shape[0], vidx.ctypes.data, vidx.shape[0],
                                         out.ctypes.data))
    return out


DEFAULT_LIGHT = None


def default_light() -> np.ndarray:
    """Vec3{X: -1, Y: 1, Z: 1}.Normalize() (renderer.go:265)."""
    return normalize3([-1.0, 1.0, 1.0])


def fov_radians(deg: float) -> float:
    """float32(deg * (math.Pi / 180)), rounded once as Go's constant arithmetic does."""
    import fractions
    pi = fractions.Fraction("3.141592653589793238462643383279502884197")
    val = fractions.Fraction(deg).limit_denominator(10 ** 12) * pi / 180
    f = np.float32(float(val))
    cands = [np.nextafter(f, np.float32(-np.inf)), f, np.nextafter(f, np.float32(np.inf))]
    return float(min(cands, key=lambda c: abs(fractions.Fraction(float(c)) - val)))


# ---- device objects ----

class DeviceBuffer:
    """Device memory owned through the C-ABI (gr_device_alloc / gr_device_free),
    with host copies through gr_copy: outputs of batched views and the
    differentiable parameters for hosts without a CUDA allocator of their own."""

    def __init__(self, ctx: "Context", nbytes: int):
        self.ctx = ctx
        self.nbytes = int(nbytes)
        self._p = C.c_void_p()
        N.check(N.lib().gr_device_alloc(ctx.handle, self.nbytes, C.byref(self._p)))

    @property
    def ptr(self) -> int:
        return int(self._p.value)

    def upload(self, a: np.ndarray) -> "DeviceBuffer":
        a = np.ascontiguousarray(a)
        if a.nbytes > self.nbytes:
            raise ValueError(f"{a.nbytes} bytes do not fit a {self.nbytes}-byte buffer")
        N.check(N.lib().gr_copy(self.ctx.handle, self.ptr, a.ctypes.data, a.nbytes))
        return self

    def download(self, shape, dtype) -> np.ndarray:
        out = np.empty(shape, dtype)
        if out.nbytes > self.nbytes:
            raise ValueError(f"{out.nbytes} bytes exceed the {self.nbytes}-byte buffer")
        N.check(N.lib().gr_copy(self.ctx.handle, out.ctypes.data, self.ptr, out.nbytes))
        return out

    @staticmethod
    def download_from(ctx: "Context", ptr: int, shape, dtype) -> np.ndarray:
        """A host copy of device memory at ptr (any device pointer of ctx's GPU)."""
        out = np.empty(shape, dtype)
        N.check(N.lib().gr_copy(ctx.handle, out.ctypes.data, int(ptr), out.nbytes))
        return out

    def free(self):
        if self._p and self._p.value and self.ctx.handle:
            N.check(N.lib().gr_device_free(self.ctx.handle, self._p))
        self._p = C.c_void_p()


class Context:
    """A gr_context: one device, one stream, resident meshes and textures."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        # objects living on this context (batches, diffs, renderers, presenters):
        # closed before it, newest first, since none may outlive the context
        self._batches = []
        N.check(N.lib().gr_context_create(device, C.byref(self._h)))

    @property
    def handle(self):
        return self._h

    def close(self):
        for b in reversed(list(self._batches)):
            b.close()
        self._batches = []
        if self._h:
            N.lib().gr_context_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def device_buffer(self, nbytes: int) -> "DeviceBuffer":
        """A device allocation on this context's GPU (gr_device_alloc)."""
        return DeviceBuffer(self, nbytes)

    def texture(self, t: TextureData) -> int:
        out = C.c_int32()
        px = None if t.pixels is None else np.ascontiguousarray(t.pixels, np.uint8)
        col = (C.c_uint8 * 4)(*t.color)
        N.check(N.lib().gr_texture_create(self._h, t.kind, t.width, t.height, _ptr(px), t.scale,
                                          C.cast(col, C.c_void_p), C.byref(out)))
        return int(out.value)

    def mesh(self, m: MeshData, texture_map: Optional[Sequence[int]] = None) -> int:
        """Uploads a mesh; texture_map translates m.tex slots to texture handles."""
        keep = []

        def arr(a, dt):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dt)
            keep.append(a)
            return a

        d = N.MeshDesc()
        pos = arr(m.pos, np.float32)
        d.positions = _ptr(pos)
        d.num_vertices = pos.shape[0]
        vn = arr(m.vnrm, np.float32)
        d.vertex_normals = _ptr(vn)
        d.num_normals = 0 if vn is None else vn.shape[0]
        vidx = arr(m.vidx, np.int32)
        d.vertex_indices = _ptr(vidx)
        d.normal_indices = _ptr(arr(m.nidx, np.int32))
        d.uvs = _ptr(arr(m.uv, np.float32))
        tex = m.tex
        if tex is not None and texture_map is not None:
            tm = np.asarray(texture_map, np.int32)
            if len(tm) == 0:
                if (tex >= 0).any():
                    raise ValueError("faces name textures but the scene has none")
                tex = np.full(tex.shape, -1, np.int32)
            else:
                tex = np.where(tex >= 0, tm[np.clip(tex, 0, len(tm) - 1)], -1).astype(np.int32)
        d.face_textures = _ptr(arr(tex, np.int32))
        d.face_normals = None
        d.vertex_colors = _ptr(arr(m.vcolor, np.float32))
        d.num_faces = vidx.shape[0]
        out = C.c_int32()
        N.check(N.lib().gr_mesh_create(self._h, C.byref(d), C.byref(out)))
        return int(out.value)

    def sync(self):
        N.check(N.lib().gr_context_sync(self._h))

    # timing helpers
    def event(self, slot: int):
        N.check(N.lib().gr_context_event_record(self._h, slot))

    def elapsed_ms(self, a: int, b: int) -> float:
        ms = C.c_float()
        N.check(N.lib().gr_context_event_elapsed(self._h, a, b, C.byref(ms)))
        return float(ms.value)

    def flush_l2(self, nbytes: int = 512 << 20):
        N.check(N.lib().gr_context_flush_l2(self._h, nbytes))

    def set_fog(self, enable: bool, fog_start: float = 0.0, fog_end: float = 0.0, color=(0, 0, 0, 0)):
        """Fog fused into every later frame (gr_context_set_fog)."""
        col = (C.c_uint8 * 4)(*color)
        N.check(N.lib().gr_context_set_fog(self._h, 1 if enable else 0, fog_start, fog_end, C.cast(col, C.c_void_p)))

    def fog(self, rgba_dev: int, z_dev: int, width: int, height: int, fog_start: float, fog_end: float, color):
        """FrameBuffer.Fog on a device framebuffer (gr_fog)."""
        col = (C.c_uint8 * 4)(*color)
        N.check(N.lib().gr_fog(self._h, int(rgba_dev), int(z_dev), width, height, fog_start, fog_end,
                               C.cast(col, C.c_void_p)))

    def set_tuning(self, tile_size: int = 0, bin_capacity: int = 0):
        N.check(N.lib().gr_context_set_tuning(self._h, tile_size, bin_capacity))

    def tuning(self) -> Tuple[int, int]:
        t, b = C.c_int32(), C.c_int32()
        N.check(N.lib().gr_context_get_tuning(self._h, C.byref(t), C.byref(b)))
        return int(t.value), int(b.value)

    def raster(self) -> Tuple[int, int]:
        """(raster cost per slice, persistent-raster waves)."""
        s, w = C.c_int32(), C.c_int32()
        N.check(N.lib().gr_context_get_raster(self._h, C.byref(s), C.byref(w)))
        return int(s.value), int(w.value)

    def last_launches(self) -> int:
        n = C.c_int32()
        N.check(N.lib().gr_context_last_launches(self._h, C.byref(n)))
        return int(n.value)


def make_items(entries: Sequence[Tuple[int, np.ndarray, np.ndarray]]):
    """gr_draw_item array from (mesh handle, mvp, world) tuples."""
    items = (N.DrawItem * max(1, len(entries)))()
    for i, (mesh, mvp, world) in enumerate(entries):
        items[i].mesh = mesh
        for k in range(16):
            items[i].mvp[k] = float(mvp[k])
            items[i].world[k] = float(world[k])
    return items


def make_params(width: int, height: int, flags: int, light=None) -> N.FrameParams:
    p = N.FrameParams()
    p.width = width
    p.height = height
    p.flags = flags
    sm = screen_matrix(width, height)
    for k in range(16):
        p.screen[k] = float(sm[k])
    lv = default_light() if light is None else np.asarray(light, np.float32)
    for k in range(3):
        p.light[k] = float(lv[k])
    return p


def draw(ctx: Context, items, n: int, params: N.FrameParams, rgba_out=None, z_out=None) -> int:
    """gr_draw with host numpy outputs (or raw device pointers as ints)."""
    tpf = C.c_int64()

    def p(x):
        if x is None:
            return None
        if isinstance(x, np.ndarray):
            return x.ctypes.data
        return int(x)

    N.check(N.lib().gr_draw(ctx.handle, items, n, C.byref(params), p(rgba_out), p(z_out), C.byref(tpf)))
    return int(tpf.value)


def draw_async(ctx: Context, items, n: int, params: N.FrameParams, rgba_dev=None, z_dev=None) -> None:
    N.check(N.lib().gr_draw_async(ctx.handle, items, n, C.byref(params),
                                  None if rgba_dev is None else int(rgba_dev),
                                  None if z_dev is None else int(z_dev)))


class Camera:
    """Camera (renderer.go:22-26)."""

    def __init__(self, position=(0.0, 0.0, 5.0), direction=(0.0, 0.0, -1.0), up=(0.0, 1.0, 0.0)):
        self.Position, self.Direction, self.Up = tuple(position), tuple(direction), tuple(up)


class Object:
    """Object (mesh.go:71-79) referencing an uploaded mesh handle."""

    def __init__(self, mesh: int, scale=(1.0, 1.0, 1.0), rotation=(0.0, 0.0, 0.0), translation=(0.0, 0.0, 0.0)):
        self.Mesh, self.Scale, self.Rotation, self.Translation = mesh, scale, rotation, translation


def _c_objects(objects: Sequence[Object]):
    objs = (N.Object * max(1, len(objects)))()
    for i, o in enumerate(objects):
        objs[i].mesh = o.Mesh
        for k in range(3):
            objs[i].scale[k] = o.Scale[k]
            objs[i].rotation[k] = o.Rotation[k]
            objs[i].translation[k] = o.Translation[k]
    return objs


def _c_camera(camera: Camera):
    cam = N.Camera()
    for k in range(3):
        cam.position[k] = camera.Position[k]
        cam.direction[k] = camera.Direction[k]
        cam.up[k] = camera.Up[k]
    return cam


class Renderer:
    """NewFrameBuffer(width, height) + NewRenderer(fb) (rasterizer.go:15, renderer.go:114)."""

    _FLAG_NAMES = {"FrustumClipping": FRUSTUM_CLIPPING, "ShowFaces": SHOW_FACES,
                   "BackfaceCulling": BACKFACE_CULLING, "Lighting": LIGHTING,
                   "FlatShading": FLAT_SHADING, "ShowTextures": SHOW_TEXTURES,
                   "ShowEdges": SHOW_EDGES, "ShowVertices": SHOW_VERTICES}

    def __init__(self, ctx: Context, width: int, height: int):
        object.__setattr__(self, "_ctx", ctx)
        h = C.c_void_p()
        N.check(N.lib().gr_renderer_create(ctx.handle, width, height, C.byref(h)))
        object.__setattr__(self, "_h", h)
        object.__setattr__(self, "width", width)
        object.__setattr__(self, "height", height)
        ctx._batches.append(self)

    def _flags(self) -> int:
        f = C.c_uint32()
        N.check(N.lib().gr_renderer_get_flags(self._h, C.byref(f)))
        return int(f.value)

    def __getattr__(self, name):
        if name in Renderer._FLAG_NAMES:
            return bool(self._flags() & Renderer._FLAG_NAMES[name])
        raise AttributeError(name)

    def __setattr__(self, name, value):
        if name in Renderer._FLAG_NAMES:
            f = self._flags()
            bit = Renderer._FLAG_NAMES[name]
            f = (f | bit) if value else (f & ~bit)
            N.check(N.lib().gr_renderer_set_flags(self._h, f))
        else:
            object.__setattr__(self, name, value)

    def set_fov(self, fov_y_radians: float):
        N.check(N.lib().gr_renderer_set_fov(self._h, fov_y_radians))

    def set_light(self, direction):
        d = np.asarray(direction, np.float32)
        N.check(N.lib().gr_renderer_set_light(self._h, _fp(d)))

    def draw(self, objects: Sequence[Object], camera: Camera) -> None:
        """(*Renderer).Draw (renderer.go:443-483)."""
        objs, cam = _c_objects(objects), _c_camera(camera)
        N.check(N.lib().gr_renderer_draw(self._h, objs, len(objects), C.byref(cam)))

    @property
    def TPF(self) -> int:
        t = C.c_int64()
        N.check(N.lib().gr_renderer_tpf(self._h, C.byref(t)))
        return int(t.value)

    def pixels(self) -> np.ndarray:
        out = np.empty((self.height, self.width, 4), np.uint8)
        N.check(N.lib().gr_renderer_read(self._h, out.ctypes.data, None))
        return out

    def zbuffer(self) -> np.ndarray:
        out = np.empty((self.height, self.width), np.float32)
        N.check(N.lib().gr_renderer_read(self._h, None, out.ctypes.data))
        return out

    def fog(self, fog_start: float, fog_end: float, color) -> None:
        """FrameBuffer.Fog (rasterizer.go:193-207) on the last frame."""
        col = (C.c_uint8 * 4)(*color)
        N.check(N.lib().gr_renderer_fog(self._h, fog_start, fog_end, C.cast(col, C.c_void_p)))

    def close(self):
        if self._h:
            N.lib().gr_renderer_destroy(self._h)
            object.__setattr__(self, "_h", C.c_void_p())
        if self in self._ctx._batches:
            self._ctx._batches.remove(self)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- scenes ----

class UploadedScene:
    """A SceneData resident on a context, with per-object matrices."""

    def __init__(self, ctx: Context, scene: SceneData):
        self.ctx = ctx
        self.scene = scene
        self.tex_handles = [ctx.texture(t) for t in scene.textures]
        cache = {}
        self.mesh_handles = []
        for o in scene.objects:
            key = id(o.mesh)
            if key not in cache:
                cache[key] = ctx.mesh(o.mesh, self.tex_handles)
            self.mesh_handles.append(cache[key])
        self.fov = fov_radians(scene.fov_deg)
        self.matrices = [object_matrices(o.scale, o.rotation, o.translation, scene.camera.position,
                                         scene.camera.direction, scene.camera.up, scene.width,
                                         scene.height, self.fov) for o in scene.objects]
        self.items = make_items([(h, m[0], m[1]) for h, m in zip(self.mesh_handles, self.matrices)])
        self.params = make_params(scene.width, scene.height, scene.flags)

    def draw(self, rgba_out=None, z_out=None) -> int:
        return draw(self.ctx, self.items, len(self.scene.objects), self.params, rgba_out, z_out)

    def render(self) -> Tuple[np.ndarray, np.ndarray, int]:
        rgba = np.empty((self.scene.height, self.scene.width, 4), np.uint8)
        z = np.empty((self.scene.height, self.scene.width), np.float32)
        tpf = self.draw(rgba, z)
        return rgba, z, tpf


# ---- batched multi-view ----

class Batch:
    """A fixed set of views rendered by one CUDA graph (gr_batch_*).

    ``views`` is a list of (FrameParams, rgba device pointer, z device pointer);
    ``entries`` a list of (mesh handle, mvp, world, view index).
    """

    def __init__(self, ctx: Context, views, entries, autotune: bool = True):
        self.ctx = ctx
        self._views = (N.View * len(views))()
        for i, (params, rgba, z) in enumerate(views):
            self._views[i].params = params
            self._views[i].rgba_dev = int(rgba)
            self._views[i].z_dev = int(z)
        self._items = make_items([(m, mvp, w) for m, mvp, w, _ in entries])
        for i, (_, _, _, v) in enumerate(entries):
            self._items[i].reserved = v
        self.nviews = len(views)
        self._h = C.c_void_p()
        N.check(N.lib().gr_batch_create(ctx.handle, self._views, len(views), self._items, len(entries),
                                        1 if autotune else 0, C.byref(self._h)))
        ctx._batches.append(self)

    def run(self):
        N.check(N.lib().gr_batch_run(self._h))

    def sync(self):
        N.check(N.lib().gr_batch_sync(self._h))

    def tuning(self):
        t, s, w, b = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        ms = C.c_float()
        N.check(N.lib().gr_batch_tuning(self._h, C.byref(t), C.byref(s), C.byref(w), C.byref(b), C.byref(ms)))
        return {"tile_size": t.value, "slice_cost": s.value, "raster_waves": w.value,
                "bin_capacity": b.value, "tuned_ms": ms.value}

    def profile(self) -> Tuple[float, float, float]:
        """Stage durations in ms (project, multi-tile binning, raster) of one
        run of the batch's frame outside its graph (gr_batch_profile)."""
        ms = (C.c_float * 3)()
        N.check(N.lib().gr_batch_profile(self._h, ms))
        return float(ms[0]), float(ms[1]), float(ms[2])

    def view_tpf(self):
        out = (C.c_int64 * self.nviews)()
        N.check(N.lib().gr_context_view_tpf(self.ctx.handle, out, self.nviews))
        return list(out)

    def close(self):
        if self._h:
            N.lib().gr_batch_destroy(self._h)
            self._h = C.c_void_p()
        if self in self.ctx._batches:
            self.ctx._batches.remove(self)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def draw_views(ctx: Context, views, entries) -> None:
    """gr_draw_views: views = [(FrameParams, rgba_dev, z_dev)], entries = [(mesh, mvp, world, view)]."""
    vs = (N.View * len(views))()
    for i, (params, rgba, z) in enumerate(views):
        vs[i].params = params
        vs[i].rgba_dev = int(rgba)
        vs[i].z_dev = int(z)
    items = make_items([(m, mvp, w) for m, mvp, w, _ in entries])
    for i, (_, _, _, v) in enumerate(entries):
        items[i].reserved = v
    N.check(N.lib().gr_draw_views(ctx.handle, vs, len(views), items, len(entries)))


# ---- differentiable forward/backward (extension) ----

def diff_views(scene) -> Tuple[np.ndarray, list]:
    """(world matrix, [(width, height, flags, screen16, mvp16)]) of a scenes.DiffSceneData,
    with the host matrix code (matrix.go restated in the library)."""
    fov = fov_radians(scene.fov_deg)
    sm = screen_matrix(scene.width, scene.height)
    views, world = [], None
    for cam in scene.cameras:
        mvp, world = object_matrices((1.0, 1.0, 1.0), (0.0, 0.0, 0.0), (0.0, 0.0, 0.0), cam.position,
                                     cam.direction, cam.up, scene.width, scene.height, fov)
        views.append((scene.width, scene.height, scene.flags, sm, mvp))
    return world, views


class Diff:
    """gr_diff_*: differentiable shading of one mesh over several views.

    Parameters, targets, images and gradients are device pointers (ints):
    ``forward(pos, vcol, tex, light, target, image=None) -> loss`` and
    ``backward(g_pos, g_vcol, g_tex) -> light gradient``."""

    def __init__(self, ctx: Context, mesh: int, world, views, tex_size: Tuple[int, int] = (0, 0)):
        self.ctx = ctx
        vs = (N.DiffView * len(views))()
        for i, (w, h, flags, sm, mvp) in enumerate(views):
            vs[i].width, vs[i].height, vs[i].flags = w, h, flags
            for k in range(16):
                vs[i].screen[k] = float(sm[k])
                vs[i].mvp[k] = float(mvp[k])
        wm = np.ascontiguousarray(world, np.float32)
        self._h = C.c_void_p()
        N.check(N.lib().gr_diff_create(ctx.handle, mesh, _fp(wm), int(tex_size[1]), int(tex_size[0]), vs,
                                       len(views), C.byref(self._h)))
        self.nviews = len(views)
        ctx._batches.append(self)

    def forward(self, pos, vcol, tex, light, target, image=None) -> float:
        p = N.DiffParams()
        p.positions, p.vertex_colors = int(pos), int(vcol)
        p.texture = None if tex is None else int(tex)
        for k in range(3):
            p.light[k] = float(light[k])
        loss = C.c_double()
        N.check(N.lib().gr_diff_forward(self._h, C.byref(p), int(target), None if image is None else int(image),
                                        C.byref(loss)))
        return float(loss.value)

    def backward(self, g_pos, g_vcol, g_tex=None) -> np.ndarray:
        g = N.DiffGrads()
        g.positions, g.vertex_colors = int(g_pos), int(g_vcol)
        g.texture = None if g_tex is None else int(g_tex)
        N.check(N.lib().gr_diff_backward(self._h, C.byref(g)))
        return np.array(g.light[:], np.float64)

    def buffers(self):
        """(face ids device pointer, records device pointer, pixels)."""
        ids, rec, n = C.c_void_p(), C.c_void_p(), C.c_int64()
        N.check(N.lib().gr_diff_buffers(self._h, C.byref(ids), C.byref(rec), C.byref(n)))
        return ids.value, rec.value, int(n.value)

    def close(self):
        if self._h:
            N.lib().gr_diff_destroy(self._h)
            self._h = C.c_void_p()
        if self in self.ctx._batches:
            self.ctx._batches.remove(self)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Presenter:
    """Double-buffered headless present (gr_presenter_*): ``frame(objects, camera)``
    queues a Draw and returns the previous frame (a copy of its pixels, H x W x 4,
    and its TPF), or (None, -1) on the first call; ``flush()`` returns the last."""

    def __init__(self, renderer: "Renderer"):
        self.renderer = renderer
        self._h = C.c_void_p()
        N.check(N.lib().gr_presenter_create(renderer._h, C.byref(self._h)))
        renderer._ctx._batches.append(self)

    def _take(self, ptr, tpf, copy):
        if not ptr:
            return None, -1
        n = self.renderer.width * self.renderer.height * 4
        arr = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(C.c_uint8)), shape=(n,))
        arr = arr.reshape(self.renderer.height, self.renderer.width, 4)
        return (arr.copy() if copy else arr), int(tpf.value)

    def frame(self, objects: Sequence[Object], camera: Camera, copy: bool = True):
        """copy=False returns a view of the library's page-locked buffer, valid until the next call."""
        ptr, tpf = C.c_void_p(), C.c_int64()
        N.check(N.lib().gr_presenter_frame(self._h, _c_objects(objects), len(objects), C.byref(_c_camera(camera)),
                                           C.byref(ptr), C.byref(tpf)))
        return self._take(ptr.value, tpf, copy)

    def flush(self, copy: bool = True):
        ptr, tpf = C.c_void_p(), C.c_int64()
        N.check(N.lib().gr_presenter_flush(self._h, C.byref(ptr), C.byref(tpf)))
        return self._take(ptr.value, tpf, copy)

    def close(self):
        if self._h:
            N.lib().gr_presenter_destroy(self._h)
            self._h = C.c_void_p()
        if self in self.renderer._ctx._batches:
            self.renderer._ctx._batches.remove(self)

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
