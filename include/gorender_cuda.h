/*
 * gorender_cuda.h -- C-ABI of the GB300 frame pipeline (libgorender_cuda.so).
 *
 * This is the boundary a host program binds (cgo, ctypes, JNI ...).  It takes
 * plain pointers and sizes; no CUDA, C++ or PyTorch type appears here.  Every
 * entry point returns an int32 status (GR_OK == 0) and never aborts the
 * process; gr_last_error() gives a message for the calling thread.
 *
 * Reference interfaces replaced (file:line in the Go sources):
 *   NewFrameBuffer (rasterizer.go:15)     -> gr_renderer_create / gr_draw outputs
 *   NewRenderer + flags (renderer.go:90-148) -> gr_renderer_create/_set_flags/_set_fov
 *   (*Renderer).Draw (renderer.go:443-483) -> gr_renderer_draw, or gr_draw when
 *                                             the host builds the matrices itself
 *   NewMesh / Mesh (mesh.go:20-69)        -> gr_mesh_create
 *   NewImageTexture / NewColorTexture / SetScale (texture.go:28-67)
 *                                         -> gr_texture_create
 *   Renderer.TPF (renderer.go:98, 436-441) -> tpf_out of gr_draw / gr_renderer_tpf
 *   NewWorldMatrix/NewViewMatrix/NewPerspectiveMatrix/NewScreenMatrix
 *   (matrix.go:82-118, 133-144)           -> gr_object_matrices / gr_screen_matrix
 */
#ifndef GORENDER_CUDA_H
#define GORENDER_CUDA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define GR_OK 0
#define GR_ERR_INVALID_ARGUMENT 1 /* null pointer, bad size, unknown handle */
#define GR_ERR_CUDA 2             /* a CUDA runtime call failed */
#define GR_ERR_OUT_OF_MEMORY 3
#define GR_ERR_BAD_INDEX 4        /* a face references a missing vertex/normal/texture
                                     (the reference panics here) */
#define GR_ERR_BIN_OVERFLOW 5     /* a tile bin overflowed in an asynchronous draw;
                                     bins have been grown, re-issue the frame */
#define GR_ERR_CLIP_OVERFLOW 6    /* a clipped polygon exceeded 9 vertices
                                     (the reference panics here) */
#define GR_ERR_NO_DEVICE 7
#define GR_ERR_UNSUPPORTED 8      /* e.g. framebuffer larger than 16384 x 16384, or an edge
                                     overlay line of more than 2^22 steps */

/* ---- Renderer flags (renderer.go:90-98); defaults of NewRenderer are
 *      GR_FLAGS_DEFAULT (renderer.go:130-148). ---- */
#define GR_FRUSTUM_CLIPPING 0x01u
#define GR_SHOW_FACES 0x02u
#define GR_BACKFACE_CULLING 0x04u
#define GR_LIGHTING 0x08u
#define GR_FLAT_SHADING 0x10u
#define GR_SHOW_TEXTURES 0x20u
#define GR_SHOW_EDGES 0x40u    /* edge lines + centroid marks, drawn in draw order (renderer.go:191-209) */
#define GR_SHOW_VERTICES 0x80u /* vertex marks (renderer.go:212-216); both overlays: not in gr_draw_noalloc */
#define GR_FLAGS_DEFAULT (GR_FRUSTUM_CLIPPING | GR_SHOW_FACES | GR_BACKFACE_CULLING | GR_LIGHTING | GR_SHOW_TEXTURES)
/* Not a Renderer field: FrameBuffer.CrossHair (rasterizer.go:209-217) after
 * the scene, as Draw does when the reference's demoMode constant is false
 * (renderer.go:476-478; the reference ships with demoMode = true). */
#define GR_CROSSHAIR 0x100u

/* ---- texture kinds (texture.go:12-17) ---- */
#define GR_TEXTURE_SOLID 0
#define GR_TEXTURE_IMAGE 1
#define GR_TEXTURE_IMAGE_FAST 2 /* power-of-two sizes; chosen by NewImageTexture */

typedef struct gr_context gr_context;
typedef struct gr_renderer gr_renderer;

/* Thread-local message for the last failing call on this thread. */
const char* gr_last_error(void);
/* Library version string. */
const char* gr_version(void);

/* One context per device and per host thread that draws (Draw is not
 * reentrant, renderer.go:103-111).  All work runs on a stream the context
 * owns. */
int32_t gr_context_create(int32_t device, gr_context** out);
int32_t gr_context_destroy(gr_context* ctx);
/* Wait for all queued work; returns the first error an asynchronous draw hit. */
int32_t gr_context_sync(gr_context* ctx);

/* ---- meshes (mesh.go:20-69), resident in device memory ---- */
typedef struct {
  const float* positions;       /* num_vertices x 4 (x, y, z, w=1)  Mesh.Vertices */
  int32_t num_vertices;
  const float* vertex_normals;  /* num_normals x 4 (w=1) or NULL    Mesh.VertexNormals */
  int32_t num_normals;
  const int32_t* vertex_indices;/* num_faces x 3                     Face.VertexIndices */
  const int32_t* normal_indices;/* num_faces x 3 or NULL             Face.NormalIndices */
  const float* uvs;             /* num_faces x 6 or NULL             Face.UVs */
  const int32_t* face_textures; /* num_faces or NULL; texture handle, -1 = nil  Face.Texture */
  const float* face_normals;    /* num_faces x 4 or NULL: computed as NewMesh does */
  const float* vertex_colors;   /* num_vertices x 3 RGB in [0,1] or NULL (extension, no
                                   counterpart in the reference) */
  int32_t num_faces;
} gr_mesh_desc;

/* Uploads a mesh (host pointers).  Vertex indices are checked here; normal
 * indices are checked when a Gouraud-lit draw first uses them, matching the
 * reference, which only indexes them there (renderer.go:327-333). */
int32_t gr_mesh_create(gr_context* ctx, const gr_mesh_desc* desc, int32_t* mesh_out);
int32_t gr_mesh_destroy(gr_context* ctx, int32_t mesh);
/* Mesh.BoundingBox as stored at creation (8 x 4 floats). */
int32_t gr_mesh_bounding_box(gr_context* ctx, int32_t mesh, float* out32);

/* NewImageTexture (kind IMAGE or IMAGE_FAST; rgba = width*height*4 bytes,
 * already alpha-premultiplied as color.RGBAModel.Convert returns it) or
 * NewColorTexture (kind SOLID; color = 4 bytes).  scale = Texture.scale. */
int32_t gr_texture_create(gr_context* ctx, int32_t kind, int32_t width, int32_t height,
                          const uint8_t* rgba, float scale, const uint8_t* color,
                          int32_t* texture_out);

/* ---- low-level draw: the host supplies the matrices ---- */
typedef struct {
  int32_t mesh;
  int32_t reserved;
  float mvp[16];   /* row-major I*P*V*W as projectObject builds it (renderer.go:259-262) */
  float world[16]; /* row-major NewWorldMatrix (renderer.go:255) */
} gr_draw_item;

typedef struct {
  int32_t width, height;  /* framebuffer size, <= 16384 each */
  uint32_t flags;         /* GR_* renderer flags */
  int32_t reserved;
  float screen[16];       /* NewScreenMatrix(width, height) (renderer.go:264) */
  float light[3];         /* normalised light direction; the reference fixes
                             Vec3{-1,1,1}.Normalize() (renderer.go:265) */
} gr_frame_params;

/* Renders one frame: Clear + DotGrid + every item in order (renderer.go:443-483,
 * sequential order).  rgba_out (width*height*4 bytes, FrameBuffer.Pixels) and
 * z_out (width*height floats, FrameBuffer.ZBuffer) may be host or device
 * pointers; either may be NULL.  Blocks until the outputs are complete.
 * tpf_out (may be NULL) receives the number of binned triangles. */
int32_t gr_draw(gr_context* ctx, const gr_draw_item* items, int32_t num_items,
                const gr_frame_params* params, uint8_t* rgba_out, float* z_out,
                int64_t* tpf_out);

/* Same, enqueued on the context stream without waiting.  Outputs must be
 * device pointers (or NULL: the context framebuffer).  Errors and bin
 * overflow surface at the next gr_context_sync. */
int32_t gr_draw_async(gr_context* ctx, const gr_draw_item* items, int32_t num_items,
                      const gr_frame_params* params, uint8_t* rgba_dev, float* z_dev);

/* ---- batched multi-view drawing (no counterpart in the reference, whose
 * Draw renders one camera; each view here equals a separate gr_draw) ---- */
typedef struct {
  gr_frame_params params;
  uint8_t* rgba_dev;  /* device output, width*height*4 bytes */
  float* z_dev;       /* device output, width*height floats */
} gr_view;

/* Renders every view in one launch sequence; item i belongs to view
 * items[i].reserved.  Asynchronous on the context stream; errors and
 * overflow surface at gr_context_sync. */
int32_t gr_draw_views(gr_context* ctx, const gr_view* views, int32_t num_views,
                      const gr_draw_item* items, int32_t num_items);
/* Binned triangles per view of the last gr_draw_views / gr_batch_run
 * (waits for the stream). */
int32_t gr_context_view_tpf(gr_context* ctx, int64_t* tpf, int32_t num_views);

/* A fixed batch of views captured once as a CUDA graph.  With autotune != 0
 * the raster tile size, bin slice length and persistent-grid size are chosen
 * by timing each candidate on the batch, and the tile bins are sized to the
 * largest bin seen.  gr_batch_run launches the graph (asynchronous);
 * gr_batch_sync waits and, if a buffer overflowed, grows it, re-captures and
 * re-runs the batch before returning. */
typedef struct gr_batch gr_batch;
int32_t gr_batch_create(gr_context* ctx, const gr_view* views, int32_t num_views,
                        const gr_draw_item* items, int32_t num_items, int32_t autotune,
                        gr_batch** out);
int32_t gr_batch_run(gr_batch* batch);
int32_t gr_batch_sync(gr_batch* batch);
int32_t gr_batch_tuning(gr_batch* batch, int32_t* tile_size, int32_t* slice_cost,
                        int32_t* raster_waves, int32_t* bin_capacity, float* tuned_ms);
int32_t gr_batch_destroy(gr_batch* batch);
/* The batch's frame once outside its graph, at its tuning, with CUDA events
 * between the stages (as gr_draw_profiled): stage_ms3 receives the project,
 * multi-tile binning and raster stage durations.  Synchronous. */
int32_t gr_batch_profile(gr_batch* batch, float* stage_ms3);

/* ---- host math (R1: stays on the host, restated from matrix.go) ---- */
typedef struct {
  int32_t mesh;
  float scale[3];        /* Object.Scale */
  float rotation[3];     /* Object.Rotation, radians */
  float translation[3];  /* Object.Translation */
} gr_object;

typedef struct {
  float position[3];
  float direction[3];
  float up[3];
} gr_camera;

/* (mvp, world) exactly as projectObject computes them for a framebuffer of
 * width x height, field of view fov_y (radians), zNear 0 and zFar 50. */
int32_t gr_object_matrices(const gr_object* obj, const gr_camera* cam, int32_t width,
                           int32_t height, float fov_y, float* mvp_out16, float* world_out16);
int32_t gr_screen_matrix(int32_t width, int32_t height, float* out16);
/* Vec3.Normalize (vector.go:78-80). */
int32_t gr_normalize3(const float* v3, float* out3);
/* Frustum.BoxVisibility (clipping.go:131-154) of a mesh's bounding box
 * (Mesh.BoundingBox: 8 corners x 4 floats, mesh.go:28-51) transformed by mvp
 * as projectObject does (renderer.go:268-275), zNear 0 and zFar 50: *out =
 * 0 outside, 1 intersecting, 2 inside.  gr_draw computes it once per draw
 * item with this same function; k_cull skips the faces of an object outside. */
int32_t gr_box_visibility(const float* mvp16, const float* bbox32, int32_t* out);
/* NewMesh face normals (mesh.go:55-60): num_faces x 4 floats. */
int32_t gr_mesh_face_normals(const float* positions, int32_t num_vertices,
                             const int32_t* vertex_indices, int32_t num_faces, float* out);

/* ---- high-level Renderer: NewFrameBuffer + NewRenderer + Draw ---- */
int32_t gr_renderer_create(gr_context* ctx, int32_t width, int32_t height, gr_renderer** out);
int32_t gr_renderer_destroy(gr_renderer* r);
int32_t gr_renderer_set_flags(gr_renderer* r, uint32_t flags);
int32_t gr_renderer_get_flags(gr_renderer* r, uint32_t* flags);
/* Vertical field of view in radians (NewRenderer uses 45 degrees). */
int32_t gr_renderer_set_fov(gr_renderer* r, float fov_y);
int32_t gr_renderer_set_light(gr_renderer* r, const float* direction3);
/* Renderer.Draw: builds the matrices on the host and renders into the
 * renderer's device framebuffer. */
int32_t gr_renderer_draw(gr_renderer* r, const gr_object* objects, int32_t num_objects,
                         const gr_camera* camera);
/* Copies FrameBuffer.Pixels / ZBuffer of the last Draw to host or device
 * memory (either pointer may be NULL). */
int32_t gr_renderer_read(gr_renderer* r, uint8_t* rgba_out, float* z_out);
int32_t gr_renderer_tpf(gr_renderer* r, int64_t* tpf);
/* FrameBuffer.Fog (rasterizer.go:193-207) on the renderer's last frame. */
int32_t gr_renderer_fog(gr_renderer* r, float fog_start, float fog_end, const uint8_t* color4);

/* ---- headless present (double buffer) ----
 * FrameBuffer.SwapBuffers (rasterizer.go:32-34) and the reference's present
 * loop (main.go:221-228, 297): frames render into two device framebuffers in
 * turn; each finished frame is copied to page-locked host memory on a second
 * stream while the next frame renders.  The Z buffer stays single, as in the
 * reference. */
typedef struct gr_presenter gr_presenter;
int32_t gr_presenter_create(gr_renderer* r, gr_presenter** out);
/* Queues Draw(objects, camera) (the renderer's flags, FOV and light) and
 * returns the previous frame's pixels (host, width*height*4 bytes, valid
 * until the next call) and its TPF; on the first call *prev_rgba is NULL.
 * A frame whose buffers overflowed is rendered again before it is returned. */
int32_t gr_presenter_frame(gr_presenter* p, const gr_object* objects, int32_t num_objects, const gr_camera* camera,
                           const uint8_t** prev_rgba, int64_t* prev_tpf);
/* Waits for the last queued frame and returns it (NULL when none is queued). */
int32_t gr_presenter_flush(gr_presenter* p, const uint8_t** rgba, int64_t* tpf);
int32_t gr_presenter_destroy(gr_presenter* p);

/* ---- fog (rasterizer.go:185-207) ----
 * FrameBuffer.Fog: pixels with depth >= fog_start keep their colour, those
 * with depth <= fog_end take color4, the rest blend by
 * f = 1 - (fog_end - depth) / (fog_end - fog_start) (blendRGBA, alpha too).
 * The reference's Draw does not call it (renderer.go:479 is commented out). */
/* On any framebuffer in device memory (RGBA8 + Z of width x height). */
int32_t gr_fog(gr_context* ctx, uint8_t* rgba_dev, const float* z_dev, int32_t width, int32_t height,
               float fog_start, float fog_end, const uint8_t* color4);
/* Fused: every later frame of the context ends with Fog in the raster's
 * write-back (after overlays and the crosshair), as Draw followed by Fog
 * would; enable = 0 turns it off. */
int32_t gr_context_set_fog(gr_context* ctx, int32_t enable, float fog_start, float fog_end,
                           const uint8_t* color4);

/* ---- timing helpers (CUDA events on the context stream) ---- */
int32_t gr_context_event_record(gr_context* ctx, int32_t slot);  /* slot < 64 */
int32_t gr_context_event_elapsed(gr_context* ctx, int32_t start_slot, int32_t end_slot,
                                 float* ms);
/* Writes 'bytes' bytes of a scratch buffer on the context stream (flushes L2
 * between timed frames). */
int32_t gr_context_flush_l2(gr_context* ctx, int64_t bytes);
/* Raster tile size (16 or 32 pixels; 0 keeps the current one) and per-tile
 * bin capacity in triangles (0 keeps the automatic size).  A frame whose
 * bins overflow is re-run by gr_draw after the bins grow. */
int32_t gr_context_set_tuning(gr_context* ctx, int32_t tile_size, int32_t bin_capacity);
int32_t gr_context_get_tuning(gr_context* ctx, int32_t* tile_size, int32_t* bin_capacity);
/* Raster work split: estimated raster cost per slice (a tile's cost is the
 * sum over its bin entries of the entry's box clipped to the tile, in pixels,
 * plus 16; a costlier tile is shared by up to 32 CTAs) and persistent-raster
 * waves (CTAs = SMs x resident CTAs x waves); 0 keeps the current value. */
int32_t gr_context_set_raster(gr_context* ctx, int32_t slice_cost, int32_t raster_waves);
int32_t gr_context_get_raster(gr_context* ctx, int32_t* slice_cost, int32_t* raster_waves);
/* Autotunes tile size, slice length and raster waves for this frame (the
 * batch autotuner on a one-view batch) and sizes the bins; the choice stays
 * on the context. */
int32_t gr_context_autotune(gr_context* ctx, const gr_draw_item* items, int32_t num_items,
                            const gr_frame_params* params);
/* Number of kernels the last frame launched. */
int32_t gr_context_last_launches(gr_context* ctx, int32_t* launches);
/* Host<->device bytes the last gr_draw moved (draw items in; result words,
 * framebuffer and z-buffer out). */
int32_t gr_context_last_transfer_bytes(gr_context* ctx, int64_t* h2d_bytes, int64_t* d2h_bytes);
/* gr_draw with CUDA events around each kernel: kernel_ms3 receives the
 * durations of the project, multi-tile binning and raster kernels.
 * Synchronous; outputs must be device pointers or NULL. */
int32_t gr_draw_profiled(gr_context* ctx, const gr_draw_item* items, int32_t num_items,
                         const gr_frame_params* params, uint8_t* rgba_dev, float* z_dev,
                         float* kernel_ms3);
/* Page-locked host memory for framebuffers read back every frame. */
int32_t gr_host_alloc(int64_t bytes, void** out);
int32_t gr_host_free(void* p);
/* Device buffers on the context's GPU, for hosts without CUDA of their own
 * (a Go host that keeps batch outputs or differentiable parameters on the
 * device; no counterpart in the reference, whose framebuffers are Go slices,
 * rasterizer.go:15-23).  gr_device_free waits for the context's stream first.
 * gr_copy copies bytes between any two host or device pointers in the
 * context's stream order and returns when the copy is done. */
int32_t gr_device_alloc(gr_context* ctx, int64_t bytes, void** out);
int32_t gr_device_free(gr_context* ctx, void* p);
int32_t gr_copy(gr_context* ctx, void* dst, const void* src, int64_t bytes);

/* ---- draw without allocating: no counterpart in the reference ----
 * For callers that must not allocate device memory themselves or let a
 * library do it: an engine or framework that owns every device allocation,
 * or a frame loop with a fixed memory budget in which a cudaMalloc/cudaFree
 * (and the device synchronisation cudaFree implies) would stall the frame.
 * gr_draw_noalloc renders one frame like gr_draw, with every input and output
 * in caller-owned device memory, and takes all of its working memory from one
 * static device array of 8 MiB inside the library (held by every GPU that
 * loads the library until the process exits).  It allocates nothing.
 *
 * Limits, checked up front (GR_ERR_UNSUPPORTED): <= 4096 faces per frame,
 * <= 16 objects, <= 16 textures, <= 32768 vertex positions across objects
 * with faces, <= 16384 vertex normals across Gouraud-lit objects,
 * framebuffer <= 512 x 512; unknown flag bits are GR_ERR_INVALID_ARGUMENT and
 * the overlay flags (GR_SHOW_EDGES, GR_SHOW_VERTICES) GR_ERR_UNSUPPORTED.  A
 * frame that overflows the fixed bins or record buffers returns
 * GR_ERR_BIN_OVERFLOW (nothing can grow here).  The device-side vertex,
 * normal and face texture indices are checked on the GPU before the frame
 * runs: one out of range returns GR_ERR_BAD_INDEX and draws nothing.
 *
 * Concurrency: all calls share the static array, which keeps the previous
 * call's contents (each call clears what must start at zero).  Calls whose
 * GPU work overlapped would race on it, so calls on one device are
 * serialised by a lock held until the call's stream has drained; work the
 * caller queues elsewhere never touches the array.  The call is synchronous:
 * it waits for `stream` (a cudaStream_t; NULL = default stream) before
 * returning.  The first call on each device looks up the array's device
 * address (cudaGetSymbolAddress) with that device current; make it before
 * any stream capture. */
typedef struct {
  gr_mesh_desc mesh;  /* DEVICE pointers; face_normals is required (NewMesh normals);
                         face_textures index the `textures` array, -1 = nil */
  float bbox[32];     /* Mesh.BoundingBox, host memory (8 corners x 4) */
  float mvp[16];      /* as gr_draw_item */
  float world[16];
} gr_noalloc_object;

typedef struct {
  int32_t kind;           /* GR_TEXTURE_* */
  int32_t width, height;
  float scale;
  uint8_t color[4];       /* solid colour */
  const uint8_t* rgba;    /* DEVICE pointer, width*height*4 bytes (image kinds) */
} gr_noalloc_texture;

int32_t gr_draw_noalloc(int32_t device, const gr_noalloc_object* objects, int32_t num_objects,
                        const gr_noalloc_texture* textures, int32_t num_textures,
                        const gr_frame_params* params, uint8_t* rgba_dev, float* z_dev, void* stream,
                        int64_t* tpf_out);

/* ---- differentiable forward/backward ----
 * An extension with no counterpart in the reference renderer.  Visibility is
 * the exact frame pipeline's (the face FrameBuffer.Triangle leaves at each
 * pixel, rasterizer.go:90-183, with culling and clipping as the view flags
 * say); over it a smooth shading model is differentiated:
 *   l_i  perspective-correct barycentrics of pixel (x, y) from the unsnapped
 *        screen positions S * (clip_i / W_i) of the visible face's corners,
 *        clipped to the face (negative ones set to 0, the rest renormalised:
 *        visibility snaps corners to whole pixels, so a pixel can lie just
 *        outside the unsnapped face)
 *   c    = sum l_i c_i                  vertex RGB (parameter)
 *   I    = sum l_i (0.5 + 0.5 n_i . L)  n_i = xyz of Vec4.Normalize(world * vertex
 *                                       normal) (renderer.go:328-331), L a parameter
 *   t    = texel at (floor(v th) mod th, floor(u tw) mod tw), (u, v) = sum l_i uv_i
 *   out  = (I c_r t_r, I c_g t_g, I c_b t_b, t_a)   (t = 1 without UVs)
 *   loss = sum over views, pixels and channels of (out - target)^2
 * Gradients of the loss with respect to vertex colours, texels, the light and
 * vertex positions are exact for fixed visibility and texel choices (position
 * gradients flow through the barycentrics only).  Faces with a corner at or
 * behind the camera plane (W >= 0) are not shaded (out = 0, no gradient).
 * Per-pixel buffers hold all views back to back, view v starting at the sum
 * of the earlier views' W * H pixels. */
typedef struct {
  int32_t width, height;
  uint32_t flags;          /* GR_FRUSTUM_CLIPPING / GR_BACKFACE_CULLING for visibility;
                              shading flags are ignored */
  int32_t reserved;
  float screen[16];        /* NewScreenMatrix(width, height) */
  float mvp[16];           /* I*P*V*W of the object in this view */
} gr_diff_view;

typedef struct {
  const float* positions;      /* DEVICE num_vertices x 4 (w = 1); visibility uses them too */
  const float* vertex_colors;  /* DEVICE num_vertices x 3 */
  const float* texture;        /* DEVICE texture_height x texture_width x 4 RGBA, or NULL */
  float light[3];
  int32_t reserved;
} gr_diff_params;

typedef struct {
  float* positions;      /* DEVICE num_vertices x 4 (w gradient 0), overwritten */
  float* vertex_colors;  /* DEVICE num_vertices x 3, overwritten */
  float* texture;        /* DEVICE texture_height x texture_width x 4, overwritten (or NULL);
                            16-byte aligned (texels are accumulated as float4) */
  double light[3];       /* written */
} gr_diff_grads;

typedef struct gr_diff gr_diff;

/* One mesh (it needs vertex normals with normal indices; UVs optional) seen in
 * num_views views with one world matrix (host, 16 floats). */
int32_t gr_diff_create(gr_context* ctx, int32_t mesh, const float* world, int32_t texture_width,
                       int32_t texture_height, const gr_diff_view* views, int32_t num_views, gr_diff** out);
/* Renders the views with params, writes the per-pixel records (and the image,
 * RGBA fp32 per pixel, when image_dev is not NULL) and returns the loss
 * against target_dev (RGBA fp32 per pixel).  params and target must stay
 * unchanged until the matching gr_diff_backward. */
int32_t gr_diff_forward(gr_diff* d, const gr_diff_params* params, const float* target_dev, float* image_dev,
                        double* loss);
/* Gradients of the last forward's loss. */
int32_t gr_diff_backward(gr_diff* d, gr_diff_grads* grads);
/* Device buffers of the last forward: per pixel the visible face index
 * (view v's faces are v * num_faces + f; 0xFFFFFFFF = none) and a 16-byte
 * record {face, texel (y * width + x, or 0xFFFFFFFF), l0, l1}; pixels = total. */
int32_t gr_diff_buffers(gr_diff* d, const uint32_t** face_ids, const void** records, int64_t* pixels);
int32_t gr_diff_destroy(gr_diff* d);

#ifdef __cplusplus
}
#endif
#endif
