// gr_internal.h -- structures shared by the host runtime and the sm_103a
// kernels of the frame pipeline.  Plain C++ (no device code) so both nvcc and
// the host translation units include it.
#pragma once

#include <cstdint>

#include <vector_types.h>

namespace gr {

constexpr int kDefaultTileShift = 5;          // 32 x 32 pixel raster tiles (16 x 16: shift 4)
constexpr int kMaxDim = 16384;                // narrow edge-function bound
constexpr int kNarrowLimit = 16384;           // |screen coordinate| < 2^14 => int32 edge math
constexpr int kMaxFan = 7;                    // a triangle clipped by 6 planes fans into <= 7
constexpr int kKeysPerFace = 8;               // order key = face * 8 + fan + 1
constexpr uint32_t kClipFace = 0x80000000u;   // rec_of_face: a clipped face, the low bits its first fan record
constexpr int kProjectThreads = 256;
// k_cull (and k_vertex / k_light): faces (vertices, normals) a thread, 1, 2
// or 4 by the frame's face count
__host__ __device__ constexpr int project_faces_per_lane(unsigned long long faces) {
  return faces >= 2000000ull ? 4 : faces >= 1000000ull ? 2 : 1;
}
constexpr int kBinDirectMax = 4;              // triangles spanning <= 4 tiles bin directly
constexpr int kStageSlots = 3;                // pinned staging slots for back-to-back async draws
constexpr int kRasterMaxSlices = 32;          // CTAs that may share one tile's bin
static_assert(kRasterMaxSlices <= 32, "a raster work item packs its slice into 5 bits");
constexpr int kDefaultSliceCost = 8192;       // raster cost per slice before a tile is split
constexpr int kEntryCost = 32;                // raster cost of a bin entry covering <= kSmallBox pixels
constexpr int kSmallBox = 64;                 // larger tile-clipped boxes add their area to the tile's cost
// k_setup: resident CTAs an SM by the frame's face count (its k_cull lane
// count): 2 (at most 104 registers a thread, no spills, room for a k_clip CTA
// beside them) below 1 M faces; 3 (at most 80 registers, 64 bytes spilled)
// from 1 M faces on, where more warps hide more of the gathers (same-box A/B:
// the 256-view batch 40 us faster, the 5 M-face frame 3 us; the 200k-face
// frame 1.5 us slower with 3)
__host__ __device__ constexpr int setup_ctas_per_sm(int project_g) { return project_g >= 2 ? 3 : 2; }
// k_setup grid (grid-stride over the kept faces)
__host__ __device__ constexpr int setup_blocks_max(int project_g) { return setup_ctas_per_sm(project_g) * 152; }
constexpr int kClipBlocks = 2 * 152;          // k_clip grid (grid-stride over the queue)
constexpr int kBigBlocks = 3 * 152;           // k_bin_big / k_overlay grid (grid-stride over the queue)

// Texture table entry (texture.go:19-26).
struct DevTex {
  int kind;             // 0 solid, 1 image (modulo), 2 image fast (mask)
  int width, height;
  float widthF, heightF, scale;
  uint32_t color;       // solid colour, RGBA little-endian
  const uint32_t* px;   // RGBA8 texels, row-major
};

// One view of a frame or batch: framebuffer, renderer flags, screen matrix,
// light and its range of raster tiles.
struct DevView {
  int W, H;
  uint32_t flags;                   // GR_* renderer flags
  int tiles_x, tiles_y;
  uint32_t tile_base;               // first global raster tile of this view
  int vec_ok;                       // outputs allow 16-byte vector stores
  int pad;
  float S[8];                       // screen matrix rows 0 and 1
  float L[4];                       // light direction (L[3] unused)
  uint32_t* out_rgba;               // H x W RGBA8
  float* out_z;                     // H x W
  unsigned long long pix_base;      // first pixel of this view in the overlay key buffer
  int fog_on;                       // FrameBuffer.Fog after the frame
  float fog_start, fog_end;
  uint32_t fog_color;               // RGBA little-endian
};

// One draw item in device memory: an Object with its matrices.
struct DevItem {
  float mvp[16];
  float world[16];
  float bbox[32];                   // Mesh.BoundingBox, 8 corners x 4
  const float* pos;                 // nv x 4
  const float* vnrm;                // nn x 4
  const float* fnrm;                // nf x 4
  const int* vidx;                  // nf x 3
  const int* nidx;                  // nf x 3 (may be null)
  const float* uv;                  // nf x 6 (may be null)
  const int* tex;                   // nf (may be null)
  const float* vcol;                // nv x 3 (may be null)
  int nv, nn, nf;
  uint32_t face_base;               // global face order of face 0
  int block_base;                   // first k_cull block of this item
  int light_base;                   // first entry of this item in FrameArgs::vlight
  int light_block_base;             // first k_light block of this item
  int view;                         // index into FrameArgs::views
  uint32_t vert_base;               // first entry of this item in FrameArgs::vclip / vscr
  int vert_block_base;              // first k_vertex block of this item
  int vis;                          // Frustum.BoxVisibility of bbox under mvp (box_visibility)
};

// Frustum.BoxVisibility (clipping.go:131-154) of a transformed bounding box
// (renderer.go:268-275): 0 outside, 1 intersecting, 2 inside.  bbox holds the
// 8 corners x 4 of Mesh.BoundingBox; each corner is transformed as
// matrixMultiplyVec4 does, ((m0 x + m1 y) + m2 z) + m3 w, and tested against
// the six planes (zNear = 0, zFar = 50) with DistanceToVertex = N.v - N.P.
// Plain float operations, one rounding each: device code is built with
// --fmad=false and host code with -ffp-contract=off, so host and device give
// the same bits.
__host__ __device__ inline int box_visibility(const float* m, const float* bbox) {
  const float P[6][4] = {{-1, 0, 0, 1}, {1, 0, 0, 1}, {0, -1, 0, 1}, {0, 1, 0, 1}, {0, 0, 0, 1}, {0, 0, 50, 1}};
  const float N[6][4] = {{1, 0, 0, 1}, {-1, 0, 0, 1}, {0, 1, 0, 1}, {0, -1, 0, 1}, {0, 0, -1, 0}, {0, 0, 1, 0}};
  unsigned out[8];
  for (int c = 0; c < 8; ++c) {
    const float* b = bbox + 4 * c;
    float v[4];
    for (int r = 0; r < 4; ++r) v[r] = ((m[4 * r] * b[0] + m[4 * r + 1] * b[1]) + m[4 * r + 2] * b[2]) + m[4 * r + 3] * b[3];
    unsigned bits = 0;
    for (int i = 0; i < 6; ++i) {
      const float nv = ((N[i][0] * v[0] + N[i][1] * v[1]) + N[i][2] * v[2]) + N[i][3] * v[3];
      const float np = ((N[i][0] * P[i][0] + N[i][1] * P[i][1]) + N[i][2] * P[i][2]) + N[i][3] * P[i][3];
      if (nv - np > 0.0f) bits |= 1u << i;
    }
    out[c] = bits;
  }
  for (int i = 0; i < 6; ++i) {
    int outside = 0;
    for (int c = 0; c < 8; ++c) outside += (out[c] >> i) & 1u;
    if (outside == 8) return 0;
    if (outside > 0) return 1;
  }
  return 2;
}

// Raster setup of one binned triangle (64 bytes, in registers and shared
// memory; stored as a TriPacked).  For "narrow" triangles
// (all screen coordinates within +-2^14) the three adjusted edge functions
// E(x,y) = a*x + b*y + c evaluate exactly in int32 over the screen.
struct alignas(16) TriRaster {
  int a01, b01, c01;
  int a12, b12, c12;
  int a20, b20, c20;
  float sumf;                       // float32(E01+E12+E20), constant over the triangle
  float w0, w1, w2;                 // clip-space W of the vertices (the rasteriser's z)
  uint32_t key;                     // bit 31: wide; bits 0..30: face*8 + fan + 1
  int16_t bx0, bx1, by0, by1;       // pixel bounding box clamped to the screen, inclusive
};
static_assert(sizeof(TriRaster) == 64, "TriRaster layout");

// int64 edge coefficients of a "wide" triangle (wraparound arithmetic) and
// its pixel box (its corners do not fit a TriPacked).
struct alignas(16) TriWide {
  long long a01, b01, c01, a12, b12, c12, a20, b20, c20;
  int16_t bx0, bx1, by0, by1;
};

// The raster record of one binned triangle as stored (32 bytes): what the
// raster needs of a narrow triangle follows from its integer screen corners
// (|coordinate| < 2^14), its three W's and its order key -- the edge
// functions, the top-left adjustment, the sum and the clamped pixel box are
// recomputed where the record is read (unpack_tri).  A wide triangle keeps
// its sum here and its int64 edges and box in TriWide.
struct alignas(16) TriPacked {
  int16_t x0, y0, x1, y1, x2, y2;   // narrow triangles only
  uint32_t key;                     // bit 31: wide; bits 0..30: face*8 + fan + 1
  float w0, w1, w2;                 // clip-space W of the vertices (the rasteriser's z)
  float sumf;                       // wide triangles only: float32(E01+E12+E20)
};
static_assert(sizeof(TriPacked) == 32, "TriPacked layout");

// Shading inputs of one binned triangle, in two arrays so that each frame
// writes only what its triangles use, in whole 32-byte sectors: the
// intensities and texture slot of every triangle (16 bytes) and, for
// textured triangles only, u/W and v/W per vertex (32 bytes).
struct alignas(16) TriShade {
  float i0, i1, i2;                   // light intensity per vertex
  int tex;                            // texture slot; -1 = faceColor; -2 = vertex colour from
                                      // TriColor (clipped fans); -3 = vertex colour of kept face r,
                                      // gathered again from the mesh (no TriColor written)
};
struct alignas(16) TriUV {
  float u0w, v0w, u1w, v1w, u2w, v2w; // u/W and v/W per vertex (rasterizer.go:132-137)
  float pad[2];
};

// Per-vertex RGB of a clipped fan triangle (vertex-colour extension), 3 x 3
// floats; the whole faces k_cull keeps are shaded from the mesh's own
// vertex colours instead (TriShade::tex == -3).
struct TriColor {
  float c[9];
};

// One binned triangle's overlay marks (ShowEdges / ShowVertices,
// renderer.go:191-216): its int() corners, its float corners (the centroid
// mark uses them) and its draw-order key.
struct Overlay {
  long long X[3], Y[3];
  float sx[3], sy[3];
  uint32_t key;                     // face * 8 + fan + 1
  uint32_t view;
};
constexpr long long kMaxLineSteps = 1ll << 22;  // longer overlay lines are refused (error bit 2)

// Counters the kernels append to.  Zeroed once at allocation; the raster
// kernel copies them into DevResult and zeroes them again.
struct DevWork {
  unsigned long long tpf;           // binned triangles (Renderer.TPF, one tile)
  unsigned int nrec;                // raster records written
  unsigned int nbig;                // records in the multi-tile queue
  unsigned int bin_need;            // max (bin position + 1) seen when over capacity
  unsigned int rec_need;            // records needed when over capacity
  unsigned int big_need;
  unsigned int error;               // bit 0 clip overflow, bit 1 bad normal index, bit 2 overlay line too long
  unsigned int nclip;               // faces queued for the general clipper
  unsigned int clip_need;
  unsigned int max_bin;             // largest tile bin of the frame (k_plan)
  unsigned int plan_front, plan_back;  // raster work items: split tiles, whole tiles
  unsigned int raster_next, raster_exit;  // persistent raster: next item, finished CTAs
  unsigned int novl, ovl_need;      // overlay records written / needed
  unsigned int nempty, clear_next;  // tiles without bin entries (k_plan); the next one k_raster clears
  unsigned int nkept;               // faces k_cull kept whole, for k_setup
};

struct alignas(8) DevResult {
  unsigned long long tpf;           // binned triangles over all views
  unsigned int nrec, nbig, bin_need, rec_need, big_need, error, nclip, clip_need, max_bin, items;
  unsigned int novl, ovl_need;
};
static_assert(sizeof(DevResult) % sizeof(unsigned) == 0, "DevResult is copied word by word");

// Everything a frame's kernels need, passed by value.
struct FrameArgs {
  const DevView* views;
  int num_views;
  uint32_t total_tiles;             // sum of the views' tiles
  uint32_t flags_any;               // OR of the views' flags
  int tile_shift;                   // raster tile = (1 << tile_shift)^2 pixels (4 or 5)
  int num_items;
  int total_blocks;
  int project_g;                    // k_cull faces a thread (project_faces_per_lane); k_light and
                                    // k_vertex take as many normals / vertices a thread
  uint32_t bin_cap;
  uint32_t rec_cap;
  uint32_t big_cap;
  const DevItem* items;
  const DevTex* texs;
  int num_tex;
  TriPacked* rast;
  TriShade* shade;
  TriUV* suv;                       // read only for textured triangles (TriShade::tex >= 0)
  TriWide* wide;
  TriColor* tcol;
  uint32_t* rec_of_face;            // per global face: its record (a face kept whole) or kClipFace |
                                    // the first record of its fans (a clipped face: fan k at first + k)
  uint32_t face_cap;
  uint32_t* bins;                   // tiles x bin_cap record indices
  uint32_t* bin_count;              // per tile: entries
  uint32_t* tile_cost;              // per tile: tile-clipped box pixels of entries larger than kSmallBox
  uint2* big;                       // multi-tile queue: (record, view)
  uint2* clip;                      // (item, face) pairs for the general clipper
  uint32_t clip_cap;
  uint2* kept;                      // (item, face) of the faces k_cull kept whole; k_setup writes
                                    // the record of entry k as record k
  uint32_t kept_cap;                // >= the frame's faces: never overflows
  int setup_blocks;                 // k_setup grid
  float* vlight;                    // per-normal Gouraud intensities (k_light)
  int light_blocks;                 // k_light grid (0: no Gouraud item)
  float4* vclip;                    // per item vertex: clip-space position (k_vertex)
  float4* vscr;                     // per item vertex: screen x, y before int() and clip W (k_vertex)
  int vert_blocks;                  // k_vertex grid
  unsigned long long* gkey;         // tiles x 1024 merged visibility keys of split tiles (zero when idle)
  uint32_t* tile_done;              // per tile: slices finished (zero when idle)
  uint32_t slice_cost;              // raster cost per slice (k_plan splits costlier tiles)
  DevWork* work;
  DevResult* result;
  DevResult* result_host;           // device address of page-locked host memory that the last raster
                                    // CTA copies the result into (null: the host copies it), followed
                                    // by a word it sets to 1 once the frame's writes are visible to the
                                    // host (every CTA fences at system scope before it retires)
  unsigned long long* view_tpf;     // per view: binned triangles (zeroed by k_plan)
  unsigned long long* view_tpf_out; // per view: published by k_plan
  uint2* plan;                      // raster work items (tile, slice | view << 5), plan_cap entries
  uint2* empty_tiles;               // (tile, view) of tiles without bin entries, cleared by k_raster
  uint32_t empty_cap;
  int clear_empty;                  // nonzero: tiles without bin entries go to that list (batches
                                    // shaded in place), not to the raster queue
  uint32_t plan_cap;
  int raster_ctas;                  // persistent raster grid
  Overlay* ovl;                     // overlay records (views with ShowEdges / ShowVertices)
  uint32_t ovl_cap;
  uint32_t* ovl_key;                // per pixel of every view: max (order key * 2 + vertex mark), 0 = none
  unsigned long long* pkey;         // per pixel of every view: final visibility keys, shaded by k_resolve
                                    // (null: k_raster shades each tile itself)
  uint4* tile_info;                 // per tile, from k_plan: x bin entries, y raster slices, z first key
                                    // slot of a split tile of a one-view frame (kNoSlot: merged in gkey)
  unsigned long long* slot_keys;    // one-view frames: slot_cap slots of TS x TS keys, one per slice of a
                                    // split tile; k_resolve takes the max over a tile's slots
  uint32_t slot_cap;
  unsigned long long total_pixels;  // sum of the views' pixels
};

// View flag (internal, never set by callers): the raster resolve writes the
// winning face's global index (or kNoFace) into out_rgba instead of a colour,
// computed from the visibility key alone, and writes no depth.
constexpr uint32_t kViewFaceIds = 0x80000000u;
constexpr uint32_t kNoSlot = 0xFFFFFFFFu;  // TileInfo: a split tile merged through gkey
constexpr uint32_t kNoFace = 0xFFFFFFFFu;

// ---- differentiable shading (an extension with no counterpart in the reference) ----
// One view of the differentiable object.
struct DiffView {
  double Q[12];                     // rows 0 and 1 of S * MVP, then row 3 of MVP (clip W)
  float Qf[24];                     // Q as float pairs: hi = float(Q), lo = float(Q - hi)
  int W, H;
  uint32_t pix_base;                // first pixel of this view in the per-pixel buffers
  uint32_t face_base;               // first global face index of this view's item
  uint32_t col_base, row_base;      // first entry of this view in col_tab / row_tab
};

// Per-pixel forward record: the visible face (or kNoFace), the texel it
// sampled (or kNoFace without a texture) and two perspective-correct
// barycentrics (the third is 1 - l0 - l1).
struct DiffRecord {
  uint32_t face;
  uint32_t texel;
  float l0, l1;
};

struct DiffArgs {
  const DiffView* views;
  int num_views;
  int max_pixels;                   // largest view (grid x extent)
  int nv, nf, nn;
  const float* pos;                 // nv x 4 (parameter)
  const float* vcol;                // nv x 3 (parameter)
  const float* tex;                 // th x tw x 4 RGBA (parameter; may be null)
  int tw, th;
  float L[4];                       // light direction (parameter)
  const int* vidx;                  // nf x 3
  const int* nidx;                  // nf x 3
  const float* uv;                  // nf x 6 (may be null)
  const float* nhat;                // nn x 4: normalised world-space vertex normals
  float* vh;                        // views x nv x 6: homogeneous screen x, y and clip W, each a
                                    // float-float pair (hi, lo) rounded from double
  float4* col_tab;                  // per view and column x: Q_0 - x Q_3 (xyz)
  float4* row_tab;                  // per view and row y: Q_1 - y Q_3 (xyz)
  const uint32_t* ids;              // per pixel: global face index or kNoFace (raster output)
  DiffRecord* rec;                  // per pixel
  const float* target;              // per pixel RGBA
  float* image;                     // per pixel RGBA (may be null)
  double* loss;                     // one value (page-locked host memory, its device address)
  float* g_pos;                     // nv x 4 (w left 0)
  float* g_vcol;                    // nv x 3
  float* g_tex;                     // th x tw x 4
  double* g_light;                  // 3 (page-locked host memory, its device address)
  double* partials;                 // kDiffSlots x {loss, light x, y, z}: per-warp sums, zero when idle
  float* g_face;                    // nf x 3 corners x {colour r, g, b, position x, y, z, 0, 0}: the
                                    // backward's per-face sums before k_diff_scatter (zero when idle),
                                    // two float4 a corner
};
constexpr int kDiffSlots = 1024;     // slots of DiffArgs::partials

// FrameBuffer.Fog on one framebuffer (gr_kernels.cu).
int launch_fog(uint32_t* rgba, const float* z, long long pixels, float fog_start, float fog_end, uint32_t color,
               void* stream);

// Kernel launchers (gr_kernels.cu).
// events (optional): 4 cudaEvent_t recorded before k_vertex, after k_setup,
// after k_bin_big (and k_clip) and after k_raster.
// A second stream and its fork / join events (created with timing off) for
// the frame's two pairs of independent kernels.
struct AuxStream {
  void* stream;
  void* fork[3];
  void* join[3];
};
int launch_frame(const FrameArgs& a, int big_blocks, void* stream, int* launches, void* const* events,
                 const AuxStream* aux = nullptr);

// Copies bytes from a page-locked staging slot (its device address) to
// device memory with one small kernel (16-byte aligned buffers).
int launch_stage(void* dst, const void* src, size_t bytes, void* stream);

// Persistent raster grid: SMs x resident CTAs of k_raster<TS> x waves.
int raster_grid(int tile_shift, int waves);

// Differentiable path (gr_diff.cu).
// Writes the bounding box (Mesh.BoundingBox layout) of pos into each item's
// bbox; partial holds 6 * kBBoxBlocks floats, *done is zero between calls.
constexpr int kBBoxBlocks = 152;
int launch_diff_bbox(const float* pos, int nv, DevItem* items, int num_items, float* partial, unsigned* done,
                     void* stream);
// nhat[n] = xyz of Vec4.Normalize(world * vnrm[n]) (renderer.go:328-331), w = 0.
int launch_diff_normals(const float* world, const float* vnrm, int nn, float* nhat, void* stream);
// Per (view, vertex) and per (view, column / row) tables, then per pixel
// shading; max_side = the largest view width or height.
int launch_diff_forward(const DiffArgs& a, int max_side, void* stream);
int launch_diff_backward(const DiffArgs& a, void* stream);

// Records a message for gr_last_error() on this thread and returns code (gr_api.cpp).
int32_t set_error(int32_t code, const char* fmt, ...);

}  // namespace gr
