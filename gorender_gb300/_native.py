"""ctypes binding of libgorender_cuda.so (the C-ABI in include/gorender_cuda.h).

Loading fails loudly when the library is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libgorender_cuda.so")

GR_OK = 0
GR_ERR_INVALID_ARGUMENT = 1
GR_ERR_CUDA = 2
GR_ERR_OUT_OF_MEMORY = 3
GR_ERR_BAD_INDEX = 4
GR_ERR_BIN_OVERFLOW = 5
GR_ERR_CLIP_OVERFLOW = 6
GR_ERR_NO_DEVICE = 7
GR_ERR_UNSUPPORTED = 8
GR_CROSSHAIR = 0x100

STATUS_NAMES = {0: "GR_OK", 1: "GR_ERR_INVALID_ARGUMENT", 2: "GR_ERR_CUDA", 3: "GR_ERR_OUT_OF_MEMORY",
                4: "GR_ERR_BAD_INDEX", 5: "GR_ERR_BIN_OVERFLOW", 6: "GR_ERR_CLIP_OVERFLOW",
                7: "GR_ERR_NO_DEVICE", 8: "GR_ERR_UNSUPPORTED"}

# Every entry point the header declares.
EXPORTS = [
    "gr_last_error", "gr_version", "gr_context_create", "gr_context_destroy", "gr_context_sync",
    "gr_mesh_create", "gr_mesh_destroy", "gr_mesh_bounding_box", "gr_texture_create", "gr_draw",
    "gr_draw_async", "gr_object_matrices", "gr_screen_matrix", "gr_normalize3", "gr_box_visibility",
    "gr_mesh_face_normals",
    "gr_renderer_create", "gr_renderer_destroy", "gr_renderer_set_flags", "gr_renderer_get_flags",
    "gr_renderer_set_fov", "gr_renderer_set_light", "gr_renderer_draw", "gr_renderer_read",
    "gr_renderer_tpf", "gr_context_event_record", "gr_context_event_elapsed", "gr_context_flush_l2",
    "gr_context_last_launches", "gr_context_last_transfer_bytes", "gr_draw_profiled", "gr_host_alloc",
    "gr_host_free", "gr_context_set_tuning", "gr_context_get_tuning", "gr_draw_noalloc",
    "gr_draw_views", "gr_context_view_tpf", "gr_batch_create", "gr_batch_run", "gr_batch_sync",
    "gr_batch_tuning", "gr_batch_destroy", "gr_context_set_raster", "gr_context_get_raster",
    "gr_context_autotune", "gr_diff_create", "gr_diff_forward", "gr_diff_backward", "gr_diff_buffers",
    "gr_diff_destroy", "gr_fog", "gr_context_set_fog", "gr_renderer_fog", "gr_presenter_create",
    "gr_presenter_frame", "gr_presenter_flush", "gr_presenter_destroy", "gr_device_alloc", "gr_device_free",
    "gr_copy", "gr_batch_profile",
]


class GrError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


class MeshDesc(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("num_vertices", C.c_int32),
                ("vertex_normals", C.c_void_p), ("num_normals", C.c_int32),
                ("vertex_indices", C.c_void_p), ("normal_indices", C.c_void_p),
                ("uvs", C.c_void_p), ("face_textures", C.c_void_p), ("face_normals", C.c_void_p),
                ("vertex_colors", C.c_void_p), ("num_faces", C.c_int32)]


class DrawItem(C.Structure):
    _fields_ = [("mesh", C.c_int32), ("reserved", C.c_int32), ("mvp", C.c_float * 16),
                ("world", C.c_float * 16)]


class FrameParams(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("flags", C.c_uint32),
                ("reserved", C.c_int32), ("screen", C.c_float * 16), ("light", C.c_float * 3)]


class Object(C.Structure):
    _fields_ = [("mesh", C.c_int32), ("scale", C.c_float * 3), ("rotation", C.c_float * 3),
                ("translation", C.c_float * 3)]


class Camera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("direction", C.c_float * 3), ("up", C.c_float * 3)]


class View(C.Structure):
    """gr_view: one view of a batch."""
    _fields_ = [("params", FrameParams), ("rgba_dev", C.c_void_p), ("z_dev", C.c_void_p)]


class DiffView(C.Structure):
    """gr_diff_view: one view of the differentiable object."""
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("flags", C.c_uint32), ("reserved", C.c_int32),
                ("screen", C.c_float * 16), ("mvp", C.c_float * 16)]


class DiffParams(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("vertex_colors", C.c_void_p), ("texture", C.c_void_p),
                ("light", C.c_float * 3), ("reserved", C.c_int32)]


class DiffGrads(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("vertex_colors", C.c_void_p), ("texture", C.c_void_p),
                ("light", C.c_double * 3)]


class NoallocObject(C.Structure):
    """gr_noalloc_object: a mesh given by device pointers plus its matrices."""
    _fields_ = [("mesh", MeshDesc), ("bbox", C.c_float * 32), ("mvp", C.c_float * 16),
                ("world", C.c_float * 16)]


class NoallocTexture(C.Structure):
    _fields_ = [("kind", C.c_int32), ("width", C.c_int32), ("height", C.c_int32), ("scale", C.c_float),
                ("color", C.c_uint8 * 4), ("rgba", C.c_void_p)]


_lib = None


def lib() -> C.CDLL:
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with gorender_gb300.build.build() "
                               "(the frame pipeline has no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        vp, i32, fp = C.c_void_p, C.c_int32, C.POINTER(C.c_float)
        L.gr_last_error.restype = C.c_char_p
        L.gr_version.restype = C.c_char_p
        sig = {
            "gr_context_create": [i32, C.POINTER(vp)],
            "gr_context_destroy": [vp],
            "gr_context_sync": [vp],
            "gr_mesh_create": [vp, C.POINTER(MeshDesc), C.POINTER(i32)],
            "gr_mesh_destroy": [vp, i32],
            "gr_mesh_bounding_box": [vp, i32, fp],
            "gr_texture_create": [vp, i32, i32, i32, vp, C.c_float, vp, C.POINTER(i32)],
            "gr_draw": [vp, C.POINTER(DrawItem), i32, C.POINTER(FrameParams), vp, vp, C.POINTER(C.c_int64)],
            "gr_draw_async": [vp, C.POINTER(DrawItem), i32, C.POINTER(FrameParams), vp, vp],
            "gr_object_matrices": [C.POINTER(Object), C.POINTER(Camera), i32, i32, C.c_float, fp, fp],
            "gr_screen_matrix": [i32, i32, fp],
            "gr_normalize3": [fp, fp],
            "gr_box_visibility": [fp, fp, vp],
            "gr_mesh_face_normals": [vp, i32, vp, i32, vp],
            "gr_renderer_create": [vp, i32, i32, C.POINTER(vp)],
            "gr_renderer_destroy": [vp],
            "gr_renderer_set_flags": [vp, C.c_uint32],
            "gr_renderer_get_flags": [vp, C.POINTER(C.c_uint32)],
            "gr_renderer_set_fov": [vp, C.c_float],
            "gr_renderer_set_light": [vp, fp],
            "gr_renderer_draw": [vp, C.POINTER(Object), i32, C.POINTER(Camera)],
            "gr_renderer_read": [vp, vp, vp],
            "gr_renderer_tpf": [vp, C.POINTER(C.c_int64)],
            "gr_context_event_record": [vp, i32],
            "gr_context_event_elapsed": [vp, i32, i32, fp],
            "gr_context_flush_l2": [vp, C.c_int64],
            "gr_context_last_launches": [vp, C.POINTER(i32)],
            "gr_context_last_transfer_bytes": [vp, C.POINTER(C.c_int64), C.POINTER(C.c_int64)],
            "gr_draw_profiled": [vp, C.POINTER(DrawItem), i32, C.POINTER(FrameParams), vp, vp, fp],
            "gr_host_alloc": [C.c_int64, C.POINTER(vp)],
            "gr_host_free": [vp],
            "gr_context_set_tuning": [vp, i32, i32],
            "gr_context_get_tuning": [vp, C.POINTER(i32), C.POINTER(i32)],
            "gr_draw_noalloc": [i32, C.POINTER(NoallocObject), i32, C.POINTER(NoallocTexture), i32,
                                C.POINTER(FrameParams), vp, vp, vp, C.POINTER(C.c_int64)],
            "gr_draw_views": [vp, C.POINTER(View), i32, C.POINTER(DrawItem), i32],
            "gr_context_view_tpf": [vp, C.POINTER(C.c_int64), i32],
            "gr_batch_create": [vp, C.POINTER(View), i32, C.POINTER(DrawItem), i32, i32, C.POINTER(vp)],
            "gr_batch_run": [vp],
            "gr_batch_sync": [vp],
            "gr_batch_tuning": [vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32), C.POINTER(i32), fp],
            "gr_batch_destroy": [vp],
            "gr_context_set_raster": [vp, i32, i32],
            "gr_context_get_raster": [vp, C.POINTER(i32), C.POINTER(i32)],
            "gr_context_autotune": [vp, C.POINTER(DrawItem), i32, C.POINTER(FrameParams)],
            "gr_diff_create": [vp, i32, fp, i32, i32, C.POINTER(DiffView), i32, C.POINTER(vp)],
            "gr_diff_forward": [vp, C.POINTER(DiffParams), vp, vp, C.POINTER(C.c_double)],
            "gr_diff_backward": [vp, C.POINTER(DiffGrads)],
            "gr_diff_buffers": [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(C.c_int64)],
            "gr_diff_destroy": [vp],
            "gr_fog": [vp, vp, vp, i32, i32, C.c_float, C.c_float, vp],
            "gr_context_set_fog": [vp, i32, C.c_float, C.c_float, vp],
            "gr_renderer_fog": [vp, C.c_float, C.c_float, vp],
            "gr_presenter_create": [vp, C.POINTER(vp)],
            "gr_presenter_frame": [vp, C.POINTER(Object), i32, C.POINTER(Camera), C.POINTER(vp), C.POINTER(C.c_int64)],
            "gr_presenter_flush": [vp, C.POINTER(vp), C.POINTER(C.c_int64)],
            "gr_presenter_destroy": [vp],
            "gr_device_alloc": [vp, C.c_int64, C.POINTER(vp)],
            "gr_device_free": [vp, vp],
            "gr_copy": [vp, vp, vp, C.c_int64],
            "gr_batch_profile": [vp, fp],
        }
        for name, args in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = C.c_int32
        _lib = L
    return _lib


def check(code: int) -> None:
    if code != GR_OK:
        raise GrError(code, lib().gr_last_error().decode(errors="replace"))
