/*
 * gorender_oracle.h -- CPU restatement of gorender's frame pipeline.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path:
 * tests, the smoke check and the CPU-baseline leg of bench.py load it.  The
 * product (libgorender_cuda.so) never links, loads or calls it.
 *
 * It restates, in plain C, the sequential (single-tile) code path of the Go
 * reference: matrix.go, vector.go, clipping.go, renderer.go, rasterizer.go,
 * texture.go and mesh.go.  Arithmetic follows Go on amd64: float32 operations
 * in source order with no FMA contraction (build with -ffp-contract=off),
 * int(float32) and uint8(float32) with the x86 "integer indefinite" result
 * for NaN and out-of-range values, and Go `int` (int64) edge functions with
 * two's-complement wraparound.
 *
 * Parity status: UNPINNED against the reference's own outputs.  The reference
 * ships no golden vectors or correctness tests (its only test file holds two
 * benchmarks without assertions) and it cannot be built here (it is Go and no
 * Go toolchain exists in this environment).  The restatement is checked by
 * hand-derived known-answer tests and by the reference's sample models when
 * those are readable.
 */
#ifndef GORENDER_ORACLE_H
#define GORENDER_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Renderer flags (renderer.go:90-98).  Same bit values as the product ABI. */
#define ORC_FRUSTUM_CLIPPING 0x01u
#define ORC_SHOW_FACES 0x02u
#define ORC_BACKFACE_CULLING 0x04u
#define ORC_LIGHTING 0x08u
#define ORC_FLAT_SHADING 0x10u
#define ORC_SHOW_TEXTURES 0x20u
#define ORC_SHOW_EDGES 0x40u
#define ORC_SHOW_VERTICES 0x80u
/* Not a Renderer field: draws FrameBuffer.CrossHair after the scene, as Draw
 * does when the reference's demoMode constant is false (renderer.go:476-478). */
#define ORC_CROSSHAIR 0x100u

/* Texture kinds (texture.go:12-17). */
#define ORC_TEX_SOLID 0
#define ORC_TEX_IMAGE 1
#define ORC_TEX_IMAGE_FAST 2

typedef struct {
  int32_t type;           /* ORC_TEX_* */
  int32_t width, height;  /* texels */
  float scale;            /* Texture.scale (SetScale), 1 by default */
  uint8_t color[4];       /* solid colour */
  const uint8_t* pixels;  /* RGBA8, row-major, width*height*4 bytes */
} orc_texture;

typedef struct {
  const float* pos;       /* nv x 4   Mesh.Vertices            */
  int32_t nv;
  const float* vnrm;      /* nn x 4   Mesh.VertexNormals       */
  int32_t nn;
  const float* fnrm;      /* nf x 4   Mesh.FaceNormals (NewMesh) */
  const int32_t* vidx;    /* nf x 3   Face.VertexIndices       */
  const int32_t* nidx;    /* nf x 3   Face.NormalIndices or NULL */
  const float* uv;        /* nf x 6   Face.UVs or NULL          */
  const int32_t* tex;     /* nf       texture slot, -1 = nil; or NULL */
  const float* vcolor;    /* nv x 3   per-vertex RGB in [0,1] (extension) or NULL */
  int32_t nf;
  float bbox[8][4];       /* Mesh.BoundingBox */
} orc_mesh;

typedef struct {
  const orc_mesh* mesh;
  float mvp[16];          /* row-major, I*P*V*W (renderer.go:259-262) */
  float world[16];        /* row-major, NewWorldMatrix */
} orc_item;

typedef struct {
  int32_t width, height;
  float screen[16];       /* NewScreenMatrix */
  float light[3];         /* normalised light direction (renderer.go:265) */
  uint32_t flags;         /* ORC_* */
  const orc_texture* textures;
  int32_t ntextures;
} orc_frame;

/* One frame: Clear + DotGrid + projection of every item in order + raster of
 * every binned triangle in order (renderer.go:443-483 with parallel=false).
 * rgba: width*height*4 bytes; z: width*height floats.  tpf receives the
 * number of binned triangles (Renderer.TPF with one tile).  nthreads > 1
 * projects objects concurrently and rasterises in disjoint horizontal bands,
 * which yields the same bytes as nthreads == 1.  Returns 0, or a negative
 * error: -1 bad vertex index, -2 bad normal index, -3 clip polygon overflow,
 * -4 out of memory, -5 bad texture slot, -6 an overlay line of more than
 * 2^22 steps (ShowEdges on a triangle with far-away corners).  ShowEdges
 * and ShowVertices draw the reference's overlays in draw order
 * (renderer.go:191-216, FrameBuffer.Line/Rect/Pixel). */
int orc_draw(const orc_item* items, int32_t nitems, const orc_frame* fr,
             uint8_t* rgba, float* z, int64_t* tpf, int32_t nthreads);

/* orc_draw that also records, per pixel, the global face index (faces of
 * earlier items first) of the triangle that last wrote it, or 0xFFFFFFFF. */
int orc_draw_ids(const orc_item* items, int32_t nitems, const orc_frame* fr,
                 uint8_t* rgba, float* z, uint32_t* ids, int64_t* tpf, int32_t nthreads);

/* ---- differentiable shading extension (no counterpart in the reference) ----
 * FP64 restatement of the shading model the CUDA differentiable path
 * implements over fixed visibility (per-pixel face ids) and, optionally,
 * fixed texel choices.  Inputs are doubles so that finite differences can be
 * taken without float32 rounding of the perturbed parameter. */
typedef struct {
  int32_t nv, nf, nn;
  const double* pos;      /* nv x 4 (w = 1) */
  const double* vcol;     /* nv x 3 */
  const int32_t* vidx;    /* nf x 3 */
  const int32_t* nidx;    /* nf x 3 */
  const double* vnrm;     /* nn x 4 */
  const double* uv;       /* nf x 6, or NULL */
  const double* tex;      /* th x tw x 4, or NULL */
  int32_t tw, th;
  double light[3];
  double world[16];
} orc_diff_scene;

typedef struct {
  int32_t width, height;
  double screen[16];
  double mvp[16];
} orc_diff_view;

/* Loss of the views (pixels back to back) against target (RGBA per pixel).
 * ids: visible global face per pixel (view v's faces are v * nf + f).
 * texel_in: texel per pixel to use (NULL: choose from the UVs, writing the
 * choice to texel_out when that is not NULL).  image, g_pos (nv x 4),
 * g_vcol (nv x 3), g_tex (th x tw x 4) and g_light (3) are optional outputs;
 * gradients are written (not accumulated).  Returns the loss. */
double orc_diff_eval(const orc_diff_scene* s, const orc_diff_view* views, int32_t nviews, const uint32_t* ids,
                     const uint32_t* texel_in, uint32_t* texel_out, const float* target, double* image,
                     double* g_pos, double* g_vcol, double* g_tex, double* g_light);

/* Projection only: the binned triangles of every item in draw order, as
 * drawProjection passes them to FrameBuffer.Triangle (int x, int y per
 * vertex into xy_out, 6 per triangle; clip W into w_out, 3 per triangle).
 * Returns the triangle count (entries beyond cap are counted, not written)
 * or a negative error. */
int64_t orc_project(const orc_item* items, int32_t nitems, const orc_frame* fr, int64_t* xy_out,
                    float* w_out, int64_t cap);

/* ---- per-stage entry points used by the known-answer tests ---- */

/* matrixMultiplyVec4Batch (asm_amd64.s:7-50 / asm_purego.go:9-19), in place. */
void orc_transform_batch(const float* m, float* vecs, int64_t n);
/* facingCamera (renderer.go:246-250) on clip-space xyz of three Vec4. */
int orc_facing_camera(const float* v0, const float* v1, const float* v2);
/* Frustum.BoxVisibility (clipping.go:131-154) of 8 clip-space corners. */
int orc_box_visibility(const float* corners8x4, float znear, float zfar);
/* Frustum.ClipTriangle (clipping.go:167-236).  pts 3x4, uvs 3x2, inten 3,
 * col 3x3 (may be NULL).  Outputs sized for 9 triangles: pts_out 9x3x4,
 * uv_out 9x3x2, inten_out 9x3, col_out 9x3x3.  Returns the triangle count or
 * -3 on polygon overflow. */
int orc_clip_triangle(const float* pts, const float* uvs, const float* inten,
                      const float* col, float znear, float zfar,
                      float* pts_out, float* uv_out, float* inten_out,
                      float* col_out);
/* Go amd64 conversions: int(float32) and uint8(float32). */
int64_t orc_go_int(float f);
uint8_t orc_go_uint8(float f);
/* Texture.Sample (texture.go:69-89): writes 4 bytes. */
void orc_texture_sample(const orc_texture* t, float u, float v, uint8_t* out);
/* FrameBuffer.Triangle (rasterizer.go:90-183) on an existing buffer, with the
 * given tile bounds; texture may be NULL (faceColor). */
void orc_fb_triangle(uint8_t* rgba, float* z, int32_t width, int32_t height,
                     int64_t x0, int64_t y0, float z0, float u0, float v0,
                     int64_t x1, int64_t y1, float z1, float u1, float v1,
                     int64_t x2, int64_t y2, float z2, float u2, float v2,
                     int64_t tsx, int64_t tsy, int64_t tex_, int64_t tey,
                     float ia, float ib, float ic, const orc_texture* texture);
/* FrameBuffer.Line (rasterizer.go:65-79) and FrameBuffer.Rect (54-63) on an
 * existing buffer; both plot through FrameBuffer.Pixel (25-30).  orc_fb_line
 * returns -6 (and draws nothing) for more than 2^22 steps. */
int orc_fb_line(uint8_t* rgba, int32_t width, int32_t height, int64_t x0, int64_t y0, int64_t x1, int64_t y1,
                const uint8_t* color);
void orc_fb_rect(uint8_t* rgba, int32_t width, int32_t height, int64_t x, int64_t y, int64_t w, int64_t h,
                 const uint8_t* color);
/* FrameBuffer.Fog (rasterizer.go:193-207) on an existing frame. */
void orc_fog(uint8_t* rgba, const float* z, int32_t width, int32_t height, float fog_start, float fog_end,
             const uint8_t* color);
/* NewMesh face normals (mesh.go:53-60) and boundingBox (mesh.go:28-51). */
void orc_mesh_face_normals(const float* pos, const int32_t* vidx, int32_t nf,
                           float* fnrm_out);
void orc_mesh_bbox(const float* pos, int32_t nv, float* bbox_out);

/* Host matrix constructors (matrix.go), row-major 4x4 outputs. */
void orc_world_matrix(const float* scale3, const float* rot3,
                      const float* trans3, float* out);
void orc_view_matrix(const float* eye3, const float* dir3, const float* up3,
                     float* out);
void orc_perspective_matrix(float fov, float aspect, float znear, float zfar,
                            float* out);
void orc_screen_matrix(int32_t width, int32_t height, float* out);
void orc_matrix_multiply(const float* a, const float* b, float* out);
void orc_normalize3(const float* v, float* out);
/* Go's math.Sin / Cos / Tan on float64 (math32.go:15-25 round them to float32). */
double orc_go_sin(double x);
double orc_go_cos(double x);
double orc_go_tan(double x);

#ifdef __cplusplus
}
#endif
#endif
