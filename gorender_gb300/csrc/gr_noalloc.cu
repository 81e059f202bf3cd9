// gr_noalloc.cu -- gr_draw_noalloc: one frame with no device allocation.
//
// Who needs this: callers that must not call cudaMalloc/cudaFree, such as a
// render thread inside an engine or framework whose allocator owns all device
// memory, or a frame loop with a fixed memory budget where an allocation (and
// the device synchronisation cudaFree implies) would stall the frame.  They
// pass device pointers for every input and output; this entry point renders
// the frame with the same kernels as gr_draw, but all of the frame's working
// memory (triangle records, tile bins, queues, split-tile keys, counters,
// the item and texture tables) is carved from one file-scope device array of
// kScratchBytes (8 MiB).  Every GPU that loads the library holds that array
// until the process exits.
//
// Limits (larger frames are rejected with GR_ERR_UNSUPPORTED): at most
// kMaxFaces faces per frame, kMaxObjects objects, kMaxTextures textures,
// kMaxNormals vertex normals across Gouraud-lit objects, kMaxVertices vertex
// positions across objects with faces, and a framebuffer of at most
// kMaxSide x kMaxSide pixels.  Bins and record buffers cannot grow here: a
// frame that would overflow them returns GR_ERR_BIN_OVERFLOW.
//
// The caller's device-side indices (vertex, normal and face texture indices)
// are checked on the GPU by k_noalloc_check before the frame's kernels run;
// an index out of range returns GR_ERR_BAD_INDEX and nothing is drawn.
//
// The array is shared by every call in the process and keeps the previous
// call's contents: each call clears the parts that must start at zero.  Two
// calls whose GPU work overlapped would race on it; a per-device lock held
// until the call's stream has drained keeps calls on one device from
// overlapping (calls on different devices use different copies of the array
// and do not wait on each other).  The first call on each device looks up the
// array's device address with cudaGetSymbolAddress while that device is
// current; make that first call before any stream capture.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/gorender_cuda.h"
#include "gr_host_math.h"
#include "gr_internal.h"

namespace gr {
namespace {

constexpr int kMaxFaces = 4096;
constexpr int kMaxObjects = 16;
constexpr int kMaxTextures = 16;
constexpr int kMaxNormals = 16384;
constexpr int kMaxVertices = 32768;
constexpr int kMaxSide = 512;
constexpr int kTiles = (kMaxSide / 32) * (kMaxSide / 32);
constexpr uint32_t kRecCap = 3u * kMaxFaces;
constexpr uint32_t kBinCap = 1024;
constexpr uint32_t kQueueCap = kMaxFaces + 1024;
constexpr size_t kScratchBytes = 8u << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr size_t up256(size_t v) { return (v + 255) & ~(size_t)255; }

// Byte offsets of the sub-buffers inside g_scratch.
struct Layout {
  size_t items, texs, views, view_tpf, view_tpf_out, plan, empty, rast, shade, suv, wide, tcol, keys, bins, bin_count, tile_cost, big, clip, kept,
      vlight, vclip, vscr, gkey, tile_done, tile_info, work, result, check, end;
};

constexpr Layout make_layout() {
  Layout l{};
  size_t o = 0;
  l.items = o; o += up256(sizeof(DevItem) * kMaxObjects);
  l.texs = o; o += up256(sizeof(DevTex) * kMaxTextures);
  l.views = o; o += up256(sizeof(DevView));
  l.view_tpf = o; o += up256(sizeof(unsigned long long));
  l.view_tpf_out = o; o += up256(sizeof(unsigned long long));
  l.plan = o; o += up256(sizeof(uint2) * kTiles * kRasterMaxSlices);
  l.empty = o; o += up256(sizeof(uint2) * kTiles);
  l.rast = o; o += up256(sizeof(TriPacked) * kRecCap);
  l.shade = o; o += up256(sizeof(TriShade) * kRecCap);
  l.suv = o; o += up256(sizeof(TriUV) * kRecCap);
  l.wide = o; o += up256(sizeof(TriWide) * kRecCap);
  l.tcol = o; o += up256(sizeof(TriColor) * kRecCap);
  l.keys = o; o += up256(sizeof(uint32_t) * kMaxFaces);
  l.bins = o; o += up256(sizeof(uint32_t) * kTiles * kBinCap);
  l.bin_count = o; o += up256(sizeof(uint32_t) * kTiles);
  l.tile_cost = o; o += up256(sizeof(uint32_t) * kTiles);
  l.big = o; o += up256(sizeof(uint2) * kQueueCap);
  l.clip = o; o += up256(sizeof(uint2) * kQueueCap);
  l.kept = o; o += up256(sizeof(uint2) * kMaxFaces);
  l.vlight = o; o += up256(sizeof(float) * kMaxNormals);
  l.vclip = o; o += up256(sizeof(float4) * kMaxVertices);
  l.vscr = o; o += up256(sizeof(float4) * kMaxVertices);
  l.gkey = o; o += up256(sizeof(unsigned long long) * kTiles * 1024);
  l.tile_done = o; o += up256(sizeof(uint32_t) * kTiles);
  l.tile_info = o; o += up256(sizeof(uint4) * kTiles);
  l.work = o; o += up256(sizeof(DevWork));
  l.result = o; o += up256(sizeof(DevResult));
  l.check = o; o += up256(sizeof(uint32_t));
  l.end = o;
  return l;
}
constexpr Layout kLayout = make_layout();
static_assert(kLayout.end <= kScratchBytes, "scratch layout exceeds the static array");

std::mutex g_mu[kMaxDevices];             // one lock per device: calls on a device never overlap
unsigned char* g_ptr[kMaxDevices] = {};   // device address of g_scratch per device

// Bits of the index check's result word.
constexpr uint32_t kBadVertex = 1u, kBadNormal = 2u, kBadTexture = 4u;

// Checks every face's indices against its object's sizes: vertex indices in
// [0, nv), normal indices in [0, nn) where the frame lights the object per
// vertex (nn > 0), face texture indices below num_tex (negative = nil).  The
// frame's kernels gather through these indices without bounds checks, so an
// out-of-range one must stop the call before they run.  Faces are numbered
// over all items (item i's faces start at items[i].face_base); one thread a
// face, grid-stride.
__global__ void k_noalloc_check(const DevItem* __restrict__ items, int n_items, uint32_t faces, int num_tex,
                                int gouraud_frame, uint32_t* __restrict__ bad) {
  uint32_t acc = 0;
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < faces; g += gridDim.x * blockDim.x) {
    int i = 0;
    while (i + 1 < n_items && items[i + 1].face_base <= g) ++i;
    const DevItem& it = items[i];
    const uint32_t f = g - it.face_base;
    if (f >= (uint32_t)it.nf) continue;
    for (int k = 0; k < 3; ++k) {
      const int v = it.vidx[3 * (size_t)f + k];
      if (v < 0 || v >= it.nv) acc |= kBadVertex;
      if (gouraud_frame && it.nn > 0) {
        const int n = it.nidx[3 * (size_t)f + k];
        if (n < 0 || n >= it.nn) acc |= kBadNormal;
      }
    }
    if (it.tex && it.tex[f] >= num_tex) acc |= kBadTexture;
  }
  if (acc) atomicOr(bad, acc);
}

}  // namespace
}  // namespace gr

using namespace gr;

extern "C" int32_t gr_draw_noalloc(int32_t device, const gr_noalloc_object* objects, int32_t num_objects,
                                   const gr_noalloc_texture* textures, int32_t num_textures,
                                   const gr_frame_params* p, uint8_t* rgba_dev, float* z_dev, void* stream,
                                   int64_t* tpf_out) {
  if (!p || !rgba_dev || !z_dev || num_objects < 0 || (num_objects > 0 && !objects) || num_textures < 0 ||
      (num_textures > 0 && !textures))
    return set_error(GR_ERR_INVALID_ARGUMENT, "gr_draw_noalloc: missing argument");
  if (device < 0 || device >= kMaxDevices) return set_error(GR_ERR_INVALID_ARGUMENT, "gr_draw_noalloc: bad device %d", device);
  if (p->width <= 0 || p->height <= 0 || p->width > kMaxSide || p->height > kMaxSide)
    return set_error(GR_ERR_UNSUPPORTED, "gr_draw_noalloc: framebuffer %dx%d exceeds the %dx%d limit", p->width,
                     p->height, kMaxSide, kMaxSide);
  if (num_objects > kMaxObjects)
    return set_error(GR_ERR_UNSUPPORTED, "gr_draw_noalloc: %d objects exceed the limit of %d", num_objects, kMaxObjects);
  if (num_textures > kMaxTextures)
    return set_error(GR_ERR_UNSUPPORTED, "gr_draw_noalloc: %d textures exceed the limit of %d", num_textures,
                     kMaxTextures);
  if (p->flags & ~0x1FFu)
    return set_error(GR_ERR_INVALID_ARGUMENT, "gr_draw_noalloc: unknown flag bits 0x%x", p->flags & ~0x1FFu);
  if (p->flags & (GR_SHOW_EDGES | GR_SHOW_VERTICES))
    return set_error(GR_ERR_UNSUPPORTED, "edge and vertex overlays are not implemented");
  const bool gouraud_frame = (p->flags & GR_LIGHTING) && !(p->flags & GR_FLAT_SHADING);
  long faces = 0, normals = 0, vertices = 0;
  for (int i = 0; i < num_objects; ++i) {
    const gr_mesh_desc& m = objects[i].mesh;
    if (m.num_faces < 0 || m.num_vertices <= 0 || !m.positions || (m.num_faces > 0 && (!m.vertex_indices || !m.face_normals)))
      return set_error(GR_ERR_INVALID_ARGUMENT, "gr_draw_noalloc: object %d needs positions, vertex indices and face normals", i);
    if (gouraud_frame && m.num_normals > 0 && (!m.vertex_normals || !m.normal_indices))
      return set_error(GR_ERR_BAD_INDEX, "gr_draw_noalloc: object %d has vertex normals without normal indices", i);
    faces += m.num_faces;
    if (m.num_faces > 0) vertices += m.num_vertices;
    if (gouraud_frame) normals += m.num_normals;
  }
  if (faces > kMaxFaces)
    return set_error(GR_ERR_UNSUPPORTED, "gr_draw_noalloc: %ld faces exceed the limit of %d", faces, kMaxFaces);
  if (vertices > kMaxVertices)
    return set_error(GR_ERR_UNSUPPORTED, "gr_draw_noalloc: %ld vertices exceed the limit of %d", vertices, kMaxVertices);
  if (normals > kMaxNormals)
    return set_error(GR_ERR_UNSUPPORTED, "gr_draw_noalloc: %ld vertex normals exceed the limit of %d", normals,
                     kMaxNormals);

  std::lock_guard<std::mutex> lk(g_mu[device]);
  int prev = -1;
  cudaGetDevice(&prev);
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return set_error(GR_ERR_NO_DEVICE, "gr_draw_noalloc: cudaSetDevice(%d): %s", device, cudaGetErrorString(e));
  if (!g_ptr[device]) {
    // once per device, with that device current
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_scratch);
    if (e != cudaSuccess) {
      if (prev >= 0) cudaSetDevice(prev);
      return set_error(GR_ERR_CUDA, "gr_draw_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    }
    g_ptr[device] = (unsigned char*)ptr;
  }
  unsigned char* base = g_ptr[device];
  cudaStream_t s = (cudaStream_t)stream;

  // host staging of the item and texture tables (plain stack arrays)
  DevItem items[kMaxObjects];
  DevTex texs[kMaxTextures];
  std::memset(items, 0, sizeof(items));
  std::memset(texs, 0, sizeof(texs));
  int live = 0, blocks = 0, light_blocks = 0, light_total = 0, vert_blocks = 0;
  uint32_t vert_total = 0;
  uint32_t face_base = 0;
  for (int i = 0; i < num_objects; ++i) {
    const gr_mesh_desc& m = objects[i].mesh;
    const uint32_t fb = face_base;
    face_base += (uint32_t)m.num_faces;
    if (m.num_faces == 0) continue;
    DevItem& d = items[live++];
    std::memcpy(d.mvp, objects[i].mvp, sizeof(d.mvp));
    std::memcpy(d.world, objects[i].world, sizeof(d.world));
    std::memcpy(d.bbox, objects[i].bbox, sizeof(d.bbox));
    d.vis = box_visibility(d.mvp, d.bbox);
    d.pos = m.positions; d.vnrm = m.vertex_normals; d.fnrm = m.face_normals; d.vidx = m.vertex_indices;
    d.nidx = m.normal_indices; d.uv = m.uvs; d.tex = m.face_textures; d.vcol = m.vertex_colors;
    d.nv = m.num_vertices; d.nn = m.vertex_normals ? m.num_normals : 0; d.nf = m.num_faces;
    d.face_base = fb;
    d.block_base = blocks;
    d.view = 0;
    blocks += (m.num_faces + kProjectThreads - 1) / kProjectThreads;  // one face a thread (kMaxFaces is small)
    d.vert_base = vert_total;
    d.vert_block_base = vert_blocks;
    vert_total += (uint32_t)m.num_vertices;
    vert_blocks += (m.num_vertices + 255) / 256;
    d.light_base = light_total;
    d.light_block_base = light_blocks;
    if (gouraud_frame && d.nn > 0) {
      light_total += d.nn;
      light_blocks += (d.nn + 255) / 256;
    }
  }
  for (int i = 0; i < num_textures; ++i) {
    const gr_noalloc_texture& t = textures[i];
    DevTex& d = texs[i];
    d.kind = t.kind;
    d.scale = t.scale;
    d.color = (uint32_t)t.color[0] | ((uint32_t)t.color[1] << 8) | ((uint32_t)t.color[2] << 16) |
              ((uint32_t)t.color[3] << 24);
    if (t.kind != GR_TEXTURE_SOLID) {
      const bool pow2 = t.width > 0 && t.height > 0 && (t.width & (t.width - 1)) == 0 && (t.height & (t.height - 1)) == 0;
      if (!t.rgba || t.width <= 0 || t.height <= 0 || (t.kind == GR_TEXTURE_IMAGE_FAST && !pow2) ||
          (t.kind != GR_TEXTURE_IMAGE && t.kind != GR_TEXTURE_IMAGE_FAST)) {
        if (prev >= 0) cudaSetDevice(prev);
        return set_error(GR_ERR_INVALID_ARGUMENT, "gr_draw_noalloc: bad texture %d", i);
      }
      d.width = t.width;
      d.height = t.height;
      d.widthF = (float)t.width;
      d.heightF = (float)t.height;
      d.px = (const uint32_t*)t.rgba;
    }
  }

  DevView view;
  std::memset(&view, 0, sizeof(view));
  view.W = p->width;
  view.H = p->height;
  view.flags = p->flags;
  view.tiles_x = (p->width + 31) / 32;
  view.tiles_y = (p->height + 31) / 32;
  view.tile_base = 0;
  for (int k = 0; k < 8; ++k) view.S[k] = p->screen[k];
  for (int k = 0; k < 3; ++k) view.L[k] = p->light[k];
  view.out_rgba = (uint32_t*)rgba_dev;
  view.out_z = z_dev;
  view.vec_ok = (p->width % 4 == 0) && ((uintptr_t)rgba_dev % 16 == 0) && ((uintptr_t)z_dev % 16 == 0);
  const int tiles = view.tiles_x * view.tiles_y;

  FrameArgs a;
  std::memset(&a, 0, sizeof(a));
  a.views = (const DevView*)(base + kLayout.views);
  a.num_views = 1;
  a.total_tiles = (uint32_t)tiles;
  a.flags_any = p->flags;
  a.tile_shift = 5;
  a.num_items = live;
  a.total_blocks = blocks;
  a.project_g = 1;
  a.bin_cap = kBinCap;
  a.rec_cap = kRecCap;
  a.big_cap = kQueueCap;
  a.clip_cap = kQueueCap;
  a.slice_cost = kDefaultSliceCost;
  a.light_blocks = light_blocks;
  a.items = (const DevItem*)(base + kLayout.items);
  a.texs = (const DevTex*)(base + kLayout.texs);
  a.num_tex = num_textures;
  a.rast = (TriPacked*)(base + kLayout.rast);
  a.shade = (TriShade*)(base + kLayout.shade);
  a.suv = (TriUV*)(base + kLayout.suv);
  a.wide = (TriWide*)(base + kLayout.wide);
  a.tcol = (TriColor*)(base + kLayout.tcol);
  a.rec_of_face = (uint32_t*)(base + kLayout.keys);
  a.face_cap = kMaxFaces;
  a.bins = (uint32_t*)(base + kLayout.bins);
  a.bin_count = (uint32_t*)(base + kLayout.bin_count);
  a.tile_cost = (uint32_t*)(base + kLayout.tile_cost);
  a.big = (uint2*)(base + kLayout.big);
  a.clip = (uint2*)(base + kLayout.clip);
  a.kept = (uint2*)(base + kLayout.kept);
  a.kept_cap = kMaxFaces;
  a.setup_blocks = (int)std::min<long>(setup_blocks_max(a.project_g), (faces + kProjectThreads - 1) / kProjectThreads);
  a.vlight = (float*)(base + kLayout.vlight);
  a.vclip = (float4*)(base + kLayout.vclip);
  a.vscr = (float4*)(base + kLayout.vscr);
  a.vert_blocks = vert_blocks;
  a.gkey = (unsigned long long*)(base + kLayout.gkey);
  a.tile_done = (uint32_t*)(base + kLayout.tile_done);
  a.tile_info = (uint4*)(base + kLayout.tile_info);
  a.work = (DevWork*)(base + kLayout.work);
  a.result = (DevResult*)(base + kLayout.result);
  a.view_tpf = (unsigned long long*)(base + kLayout.view_tpf);
  a.view_tpf_out = (unsigned long long*)(base + kLayout.view_tpf_out);
  a.plan = (uint2*)(base + kLayout.plan);
  a.plan_cap = (uint32_t)(kTiles * kRasterMaxSlices);
  a.empty_tiles = (uint2*)(base + kLayout.empty);
  a.empty_cap = (uint32_t)kTiles;
  a.raster_ctas = raster_grid(5, 1);

  // The array keeps the previous call's contents: zero what the kernels
  // expect to find zeroed (counters, bin counts, split-tile keys).
  e = cudaMemsetAsync(base + kLayout.bin_count, 0, sizeof(uint32_t) * tiles, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(base + kLayout.tile_cost, 0, sizeof(uint32_t) * tiles, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(base + kLayout.gkey, 0, sizeof(unsigned long long) * tiles * 1024, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(base + kLayout.tile_done, 0, sizeof(uint32_t) * tiles, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(base + kLayout.work, 0, sizeof(DevWork), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(base + kLayout.view_tpf, 0, sizeof(unsigned long long), s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(base + kLayout.views, &view, sizeof(view), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && live) e = cudaMemcpyAsync(base + kLayout.items, items, sizeof(DevItem) * live, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && num_textures)
    e = cudaMemcpyAsync(base + kLayout.texs, texs, sizeof(DevTex) * num_textures, cudaMemcpyHostToDevice, s);
  // The caller's indices, checked on the GPU before any kernel gathers
  // through them (one small launch and one wait; faces <= kMaxFaces).
  uint32_t bad = 0;
  if (e == cudaSuccess) e = cudaMemsetAsync(base + kLayout.check, 0, sizeof(uint32_t), s);
  if (e == cudaSuccess && live) {
    k_noalloc_check<<<(unsigned)((faces + 255) / 256), 256, 0, s>>>(
        (const DevItem*)(base + kLayout.items), live, (uint32_t)faces, num_textures, gouraud_frame ? 1 : 0,
        (uint32_t*)(base + kLayout.check));
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, base + kLayout.check, sizeof(bad), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  }
  if (e == cudaSuccess && bad) {
    if (prev >= 0) cudaSetDevice(prev);
    return set_error(GR_ERR_BAD_INDEX, "gr_draw_noalloc: %s index out of range",
                     (bad & kBadVertex) ? "a vertex" : (bad & kBadNormal) ? "a normal" : "a face texture");
  }
  int launches = 0;
  if (e == cudaSuccess) e = (cudaError_t)launch_frame(a, kBigBlocks, s, &launches, nullptr);
  DevResult r;
  std::memset(&r, 0, sizeof(r));
  if (e == cudaSuccess) e = cudaMemcpyAsync(&r, base + kLayout.result, sizeof(r), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (prev >= 0) cudaSetDevice(prev);
  if (e != cudaSuccess) return set_error(GR_ERR_CUDA, "gr_draw_noalloc: %s", cudaGetErrorString(e));
  if (r.error & 1u) return set_error(GR_ERR_CLIP_OVERFLOW, "a clipped polygon exceeded 9 vertices");
  if (r.bin_need > kBinCap || r.rec_need > kRecCap || r.big_need > kQueueCap || r.clip_need > kQueueCap)
    return set_error(GR_ERR_BIN_OVERFLOW, "gr_draw_noalloc: the frame needs more working memory than the %zu-byte "
                     "static array provides (bins %u/%u, records %u/%u)", kScratchBytes, r.bin_need, kBinCap,
                     r.rec_need, kRecCap);
  if (tpf_out) *tpf_out = (int64_t)r.tpf;
  return GR_OK;
}
