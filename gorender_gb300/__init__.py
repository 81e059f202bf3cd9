"""gorender_gb300: gorender's frame pipeline as hand-written sm_103a kernels
behind a C-ABI (include/gorender_cuda.h), with a host mirror of the
reference's Renderer / FrameBuffer / Mesh / Object / Camera API."""
from . import scenes  # noqa: F401
from .renderer import (BACKFACE_CULLING, FLAGS_DEFAULT, FLAT_SHADING, FRUSTUM_CLIPPING, LIGHTING,  # noqa: F401
                       SHOW_EDGES, SHOW_FACES, SHOW_TEXTURES, SHOW_VERTICES, Camera, Context, Object,
                       Presenter, Renderer, UploadedScene, default_light, draw, draw_async, face_normals,
                       fov_radians, make_items, make_params, normalize3, object_matrices, screen_matrix)
from ._native import GrError  # noqa: F401
