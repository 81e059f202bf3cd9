// gr_api.cpp -- C-ABI of libgorender_cuda.so: contexts, resident meshes and
// textures, frame buffers sized for the frame, the draw entry points and the
// host Renderer (NewRenderer / Draw) built on them.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/gorender_cuda.h"
#include "gr_host_math.h"
#include "gr_internal.h"

using namespace gr;

namespace {

thread_local std::string g_err;

int32_t fail(int32_t code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      return fail(e_ == cudaErrorMemoryAllocation ? GR_ERR_OUT_OF_MEMORY : GR_ERR_CUDA,    \
                  "%s failed: %s", #call, cudaGetErrorString(e_));                         \
  } while (0)

uint32_t next_pow2(uint64_t v) {
  uint64_t p = 1;
  while (p < v) p <<= 1;
  return (uint32_t)std::min<uint64_t>(p, 0x80000000ull);
}

struct MeshRec {
  bool alive = false;
  int nv = 0, nn = 0, nf = 0;
  bool has_nidx = false, nidx_ok = false;
  float bbox[32];
  float *pos = nullptr, *vnrm = nullptr, *fnrm = nullptr, *uv = nullptr, *vcol = nullptr;
  int *vidx = nullptr, *nidx = nullptr, *tex = nullptr;
};

struct TexRec {
  DevTex d;
  void* px = nullptr;
};

}  // namespace

namespace {
// An asynchronous draw's graph reads the tables from its staging slot, so a
// scene drawn repeatedly holds one graph per slot: 12 keep four such scenes
// (or a presenter's two buffers) replaying.
constexpr int kFrameGraphs = 12;
struct FrameGraph {
  cudaGraphExec_t exec = nullptr;
  FrameArgs args{};
  const void* copy_src = nullptr;   // the staging slot k_stage reads as the graph's first kernel (or none)
  size_t copy_bytes = 0;
  int launches = 0;
  uint64_t used = 0;
};
}  // namespace

struct gr_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t aux_stream = nullptr;  // second branch of a frame (AuxStream)
  cudaEvent_t aux_ev[6] = {};
  AuxStream aux{};
  std::mutex mu;
  std::vector<MeshRec> meshes;
  std::vector<TexRec> texs;
  DevTex* d_texs = nullptr;
  int d_texs_cap = 0;
  bool texs_dirty = true;

  // The draw tables: the view table and the item table side by side in one
  // device allocation (d_views / d_items point into it), staged in
  // kStageSlots page-locked slots of the same layout, so that a draw uploads
  // both with one copy.
  unsigned char* d_tables = nullptr;
  unsigned char* h_tables = nullptr;
  size_t tables_off = 0;            // byte offset of the item table in a slot
  size_t tables_stride = 0;         // bytes of one slot
  int tab_views_cap = 0;
  DevView* d_views = nullptr;
  DevItem* d_items = nullptr;
  int items_cap = 0;
  // Pinned staging ring: back-to-back asynchronous draws write the next slot;
  // a slot is rewritten only after the copies that read it have run.
  cudaEvent_t stage_ev[kStageSlots] = {};
  bool stage_used[kStageSlots] = {};
  int stage_slot = 0;

  TriPacked* rast = nullptr;
  TriShade* shade = nullptr;
  TriUV* suv = nullptr;
  TriWide* wide = nullptr;
  TriColor* tcol = nullptr;
  uint32_t rec_cap = 0;
  uint32_t* rec_of_face = nullptr;  // per face of the frame: its record, or its clip slot
  uint32_t face_cap = 0;
  uint32_t* bins = nullptr;
  uint32_t* bin_count = nullptr;
  uint32_t* tile_cost = nullptr;    // per tile: boxes of its large entries (k_plan's cost estimate)
  uint4* tile_info = nullptr;       // per tile: entries, slices, key slot (k_plan)
  uint32_t bin_cap = 0;
  uint32_t tiles_cap = 0;
  uint2* big = nullptr;             // multi-tile queue: (record, view)
  uint32_t big_cap = 0;
  unsigned long long* gkey = nullptr;  // merged keys of tiles split over several CTAs
  uint32_t* tile_done = nullptr;
  uint32_t gkey_tiles = 0;
  uint2* clip = nullptr;            // faces for the general clipper
  uint32_t clip_cap = 0;
  uint2* kept = nullptr;         // faces k_cull kept whole (one entry per face of the frame)
  uint32_t kept_cap = 0;
  float* vlight = nullptr;          // per-normal Gouraud intensities
  uint64_t vlight_cap = 0;
  float4* vclip = nullptr;          // per item vertex: clip position and screen x, y (k_vertex)
  float4* vscr = nullptr;
  uint64_t vert_cap = 0;
  unsigned long long* view_tpf = nullptr;
  unsigned long long* view_tpf_out = nullptr;
  unsigned long long* h_view_tpf = nullptr;
  int views_cap = 0;
  uint2* plan = nullptr;            // raster work queue
  uint2* empty_tiles = nullptr;     // tiles without bin entries (cleared by k_raster<TS, true>)
  uint32_t empty_cap = 0;
  uint32_t plan_cap = 0;
  bool fog_on = false;              // FrameBuffer.Fog fused into every frame
  float fog_start = 0.0f, fog_end = 0.0f;
  uint32_t fog_color = 0;
  Overlay* ovl = nullptr;           // ShowEdges / ShowVertices marks
  uint32_t ovl_cap = 0;
  uint32_t* ovl_key = nullptr;      // per pixel of all views (zero when idle)
  unsigned long long* pkey = nullptr;  // per pixel of all views: keys for k_resolve
  uint64_t pkey_pixels = 0;
  unsigned long long* slot_keys = nullptr;  // keys of split tiles' slices, 4 x pkey_pixels
  uint64_t ovl_pixels = 0;
  int raster_waves = 1;             // persistent raster CTAs = SMs x resident CTAs x waves
  int last_views = 0;               // views of the last batched draw
  float tuned_ms = 0.0f;            // best batch time seen by the autotuner
  uint32_t slice_cost = kDefaultSliceCost;
  DevWork* work = nullptr;
  DevResult* d_result = nullptr;
  DevResult* h_result = nullptr;  // pinned
  DevResult* h_result_dev = nullptr;  // its device address (the raster writes a synchronous frame's result there)

  uint32_t* fb_rgba = nullptr;
  float* fb_z = nullptr;
  size_t fb_pixels = 0;

  void* flush_buf = nullptr;
  size_t flush_bytes = 0;
  cudaEvent_t events[64] = {};
  int last_launches = 0;
  FrameGraph frame_graphs[kFrameGraphs];  // captured launch sequences, by argument block
  uint64_t frame_tick = 0;
  int32_t pending = GR_OK;
  int64_t h2d_bytes = 0, d2h_bytes = 0;  // host<->device bytes of the last draw
  uint32_t want_bin_cap = 0, want_rec_cap = 0, want_big_cap = 0, want_clip_cap = 0, want_ovl_cap = 0;
  int tile_shift = kDefaultTileShift;  // raster tile size (autotuned per workload)
};

struct gr_renderer {
  gr_context* ctx = nullptr;
  int width = 0, height = 0;
  uint32_t flags = GR_FLAGS_DEFAULT;
  float fov_y = 0.0f;
  float light[3];
  int64_t tpf = 0;
  uint32_t* rgba = nullptr;  // device framebuffer (FrameBuffer.Pixels)
  float* z = nullptr;        // FrameBuffer.ZBuffer
};

namespace {

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

// One query for an output pointer: device memory (*dev), page-locked host
// memory (returns its device address) or neither (pageable, or null).
void* classify_out_ptr(void* p, bool* dev) {
  *dev = false;
  if (!p) return nullptr;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  *dev = at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

template <class T>
int32_t dev_alloc(T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  CK(cudaMalloc((void**)p, count * sizeof(T)));
  return GR_OK;
}

template <class T>
void dev_free(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

template <class T>
int32_t upload(gr_context* c, T** dst, const T* src, size_t count) {
  *dst = nullptr;
  if (!src || count == 0) return GR_OK;
  int32_t st = dev_alloc(dst, count);
  if (st) return st;
  CK(cudaMemcpyAsync(*dst, src, count * sizeof(T), cudaMemcpyHostToDevice, c->stream));
  return GR_OK;
}

int32_t ensure_tables(gr_context* c, int nviews, int nitems) {
  if (nviews <= c->tab_views_cap && nitems <= c->items_cap) return GR_OK;
  const int vcap = nviews > c->tab_views_cap ? std::max(nviews, 2 * c->tab_views_cap) : c->tab_views_cap;
  const int icap = nitems > c->items_cap ? std::max(nitems, 2 * c->items_cap) : c->items_cap;
  CK(cudaStreamSynchronize(c->stream));
  dev_free(c->d_tables);
  if (c->h_tables) cudaFreeHost(c->h_tables);
  c->h_tables = nullptr;
  c->d_views = nullptr;
  c->d_items = nullptr;
  c->tab_views_cap = 0;
  c->items_cap = 0;
  const size_t off = (sizeof(DevView) * (size_t)vcap + 15) & ~(size_t)15;
  const size_t stride = (off + sizeof(DevItem) * (size_t)icap + 255) & ~(size_t)255;
  int32_t st = dev_alloc(&c->d_tables, stride);
  if (st) return st;
  CK(cudaMallocHost((void**)&c->h_tables, stride * (kStageSlots + 1)));  // + the synchronous draws' slot
  c->tables_off = off;
  c->tables_stride = stride;
  c->d_views = reinterpret_cast<DevView*>(c->d_tables);
  c->d_items = reinterpret_cast<DevItem*>(c->d_tables + off);
  c->tab_views_cap = vcap;
  c->items_cap = icap;
  return GR_OK;
}

// Sizes the per-frame buffers for `faces` submitted faces and `tiles` tiles.
int32_t ensure_frame_buffers(gr_context* c, uint64_t faces, uint32_t tiles) {
  bool synced = false;
  auto sync = [&]() -> int32_t {
    if (!synced) {
      CK(cudaStreamSynchronize(c->stream));
      synced = true;
    }
    return GR_OK;
  };
  int32_t st;
  uint64_t want_rec = std::max<uint64_t>(c->want_rec_cap, 2 * faces + 1024);
  want_rec = std::min<uint64_t>(want_rec, (uint64_t)kMaxFan * faces + 1024);
  if (want_rec > c->rec_cap) {
    if ((st = sync())) return st;
    dev_free(c->rast); dev_free(c->shade); dev_free(c->suv); dev_free(c->wide); dev_free(c->tcol);
    c->rec_cap = 0;
    if ((st = dev_alloc(&c->rast, want_rec)) || (st = dev_alloc(&c->shade, want_rec)) ||
        (st = dev_alloc(&c->suv, want_rec)) || (st = dev_alloc(&c->wide, want_rec)) ||
        (st = dev_alloc(&c->tcol, want_rec)))
      return st;
    c->rec_cap = (uint32_t)want_rec;
  }
  if (faces > c->face_cap) {
    if ((st = sync())) return st;
    dev_free(c->rec_of_face);
    c->face_cap = 0;
    const uint64_t cap = std::max<uint64_t>(faces, 1024);
    if ((st = dev_alloc(&c->rec_of_face, cap))) return st;
    c->face_cap = (uint32_t)cap;
  }
  uint32_t want_bin = c->want_bin_cap;
  if (want_bin == 0) want_bin = std::max<uint32_t>(1024, next_pow2(4 * (2 * faces) / std::max<uint32_t>(tiles, 1)));
  if (tiles > c->tiles_cap || want_bin > c->bin_cap) {
    if ((st = sync())) return st;
    uint32_t nt = std::max(tiles, c->tiles_cap);
    uint32_t nc = std::max(want_bin, c->bin_cap);
    dev_free(c->bins); dev_free(c->bin_count); dev_free(c->tile_cost); dev_free(c->tile_info);
    c->tiles_cap = 0; c->bin_cap = 0;
    if ((st = dev_alloc(&c->bins, (size_t)nt * nc)) || (st = dev_alloc(&c->bin_count, nt)) ||
        (st = dev_alloc(&c->tile_cost, nt)) || (st = dev_alloc(&c->tile_info, nt)))
      return st;
    CK(cudaMemsetAsync(c->bin_count, 0, sizeof(uint32_t) * nt, c->stream));
    CK(cudaMemsetAsync(c->tile_cost, 0, sizeof(uint32_t) * nt, c->stream));
    if (nt > c->gkey_tiles) {
      dev_free(c->gkey); dev_free(c->tile_done);
      c->gkey_tiles = 0;
      if ((st = dev_alloc(&c->gkey, (size_t)nt * 1024)) || (st = dev_alloc(&c->tile_done, nt))) return st;
      CK(cudaMemsetAsync(c->gkey, 0, sizeof(unsigned long long) * nt * 1024, c->stream));
      CK(cudaMemsetAsync(c->tile_done, 0, sizeof(uint32_t) * nt, c->stream));
      c->gkey_tiles = nt;
    }
    c->tiles_cap = nt;
    c->bin_cap = nc;
  }
  uint64_t want_clip = std::max<uint64_t>(c->want_clip_cap, faces / 16 + 1024);
  if (want_clip > c->clip_cap) {
    if ((st = sync())) return st;
    dev_free(c->clip);
    c->clip_cap = 0;
    if ((st = dev_alloc(&c->clip, want_clip))) return st;
    c->clip_cap = (uint32_t)want_clip;
  }
  if (faces > c->kept_cap) {  // every face may be kept: sized to the frame, never overflows
    if ((st = sync())) return st;
    dev_free(c->kept);
    c->kept_cap = 0;
    const uint64_t cap = std::max<uint64_t>(faces, 1024);
    if ((st = dev_alloc(&c->kept, cap))) return st;
    c->kept_cap = (uint32_t)cap;
  }
  uint64_t want_big = std::max<uint64_t>(c->want_big_cap, faces / 8 + 1024);
  if (want_big > c->big_cap) {
    if ((st = sync())) return st;
    dev_free(c->big);
    c->big_cap = 0;
    if ((st = dev_alloc(&c->big, want_big))) return st;
    c->big_cap = (uint32_t)want_big;
  }
  return GR_OK;
}

int32_t ensure_fb(gr_context* c, size_t pixels) {
  if (pixels <= c->fb_pixels) return GR_OK;
  CK(cudaStreamSynchronize(c->stream));
  dev_free(c->fb_rgba);
  dev_free(c->fb_z);
  c->fb_pixels = 0;
  int32_t st;
  if ((st = dev_alloc(&c->fb_rgba, pixels)) || (st = dev_alloc(&c->fb_z, pixels))) return st;
  c->fb_pixels = pixels;
  return GR_OK;
}

int32_t upload_textures(gr_context* c) {
  if (!c->texs_dirty) return GR_OK;
  int n = (int)c->texs.size();
  if (n > c->d_texs_cap) {
    CK(cudaStreamSynchronize(c->stream));
    dev_free(c->d_texs);
    c->d_texs_cap = 0;
    int32_t st = dev_alloc(&c->d_texs, std::max(n, 16));
    if (st) return st;
    c->d_texs_cap = std::max(n, 16);
  }
  if (n) {
    std::vector<DevTex> h(n);
    for (int i = 0; i < n; ++i) h[i] = c->texs[i].d;
    CK(cudaMemcpy(c->d_texs, h.data(), sizeof(DevTex) * n, cudaMemcpyHostToDevice));
  }
  c->texs_dirty = false;
  return GR_OK;
}

struct Prepared {
  FrameArgs a;
  const void* copy_src = nullptr;   // the tables' page-locked source, uploaded by the frame's graph
  size_t copy_bytes = 0;            // (Upload::kInGraph, Upload::kRingInGraph; no separate copy)
  int ring_slot = -1;               // kRingInGraph: the slot whose event the caller records after the launch
  uint64_t faces;
  int nitems;
};

// One view of a draw: its parameters and device outputs.
struct ViewIn {
  const gr_frame_params* p;
  uint32_t* rgba;
  float* z;
  bool internal = false;  // may carry library-internal view flags (kViewFaceIds)
  bool host_out = false;  // outputs in page-locked host memory (written through device addresses)
};

int32_t ensure_views(gr_context* c, int nviews, uint32_t tiles) {
  if (nviews > c->views_cap) {
    CK(cudaStreamSynchronize(c->stream));
    dev_free(c->view_tpf); dev_free(c->view_tpf_out);
    if (c->h_view_tpf) cudaFreeHost(c->h_view_tpf);
    c->h_view_tpf = nullptr;
    c->views_cap = 0;
    const int cap = std::max(nviews, 2 * c->views_cap);
    int32_t st;
    if ((st = dev_alloc(&c->view_tpf, cap)) || (st = dev_alloc(&c->view_tpf_out, cap))) return st;
    CK(cudaMemsetAsync(c->view_tpf, 0, sizeof(unsigned long long) * cap, c->stream));
    CK(cudaMallocHost((void**)&c->h_view_tpf, sizeof(unsigned long long) * cap));
    c->views_cap = cap;
  }
  const uint64_t want_plan = (uint64_t)tiles * kRasterMaxSlices;
  if (want_plan > c->plan_cap) {
    CK(cudaStreamSynchronize(c->stream));
    dev_free(c->plan);
    c->plan_cap = 0;
    int32_t st = dev_alloc(&c->plan, want_plan);
    if (st) return st;
    c->plan_cap = (uint32_t)want_plan;
  }
  return GR_OK;
}

// How a draw's tables reach the device: a k_stage queued by prepare before
// the frame (kCopy), the synchronous draws' own slot read by the frame's
// graph (kInGraph), or a slot of the ring read by the frame's graph
// (kRingInGraph: the caller records the slot's event after launching).
enum class Upload { kCopy, kInGraph, kRingInGraph };

// Validates views and items, stages the view and item tables and fills the
// kernel arguments.  items[i].reserved is the item's view when batched.
int32_t prepare(gr_context* c, const ViewIn* views, int nviews, const gr_draw_item* items, int32_t n, bool batched,
                Prepared& out, DevView* own_views = nullptr, DevItem* own_items = nullptr,
                Upload upload = Upload::kCopy) {
  if (nviews <= 0 || !views) return fail(GR_ERR_INVALID_ARGUMENT, "no views");
  if (n < 0 || (n > 0 && !items)) return fail(GR_ERR_INVALID_ARGUMENT, "bad item list");
  const int ts = 1 << c->tile_shift;
  uint32_t total_tiles = 0, flags_any = 0;
  for (int v = 0; v < nviews; ++v) {
    const gr_frame_params* p = views[v].p;
    if (!p) return fail(GR_ERR_INVALID_ARGUMENT, "view %d: params is NULL", v);
    if (p->width <= 0 || p->height <= 0)
      return fail(GR_ERR_INVALID_ARGUMENT, "view %d: bad framebuffer size %dx%d", v, p->width, p->height);
    if (p->width > kMaxDim || p->height > kMaxDim)
      return fail(GR_ERR_UNSUPPORTED, "view %d: framebuffer %dx%d exceeds %d", v, p->width, p->height, kMaxDim);
    if (!views[v].rgba || !views[v].z) return fail(GR_ERR_INVALID_ARGUMENT, "view %d: missing outputs", v);
    if (p->flags & ~(0x1FFu | (views[v].internal ? kViewFaceIds : 0u)))
      return fail(GR_ERR_INVALID_ARGUMENT, "view %d: unknown flag bits 0x%x", v, p->flags & ~0x1FFu);
    const uint64_t t = (uint64_t)((p->width + ts - 1) / ts) * (uint64_t)((p->height + ts - 1) / ts);
    if (total_tiles + t >= (1ull << 31)) return fail(GR_ERR_UNSUPPORTED, "too many raster tiles");
    total_tiles += (uint32_t)t;
    flags_any |= p->flags;
  }
  int32_t st = ensure_tables(c, nviews, std::max(n, 1));
  if (st) return st;
  if ((st = upload_textures(c))) return st;
  if ((st = ensure_views(c, nviews, total_tiles))) return st;
  uint64_t total_pixels = 0;
  for (int v = 0; v < nviews; ++v) total_pixels += (uint64_t)views[v].p->width * (uint64_t)views[v].p->height;
  if ((flags_any & (GR_SHOW_EDGES | GR_SHOW_VERTICES)) && total_pixels > c->ovl_pixels) {
    CK(cudaStreamSynchronize(c->stream));
    dev_free(c->ovl_key);
    c->ovl_pixels = 0;
    if ((st = dev_alloc(&c->ovl_key, (size_t)total_pixels))) return st;
    CK(cudaMemsetAsync(c->ovl_key, 0, sizeof(uint32_t) * total_pixels, c->stream));
    c->ovl_pixels = total_pixels;
  }
  // One view: k_raster stores the final keys and k_resolve shades every
  // pixel at full occupancy.  Many views: k_raster shades each tile (the
  // keys of a large batch would cost more memory traffic than they save).
  // Outputs in host memory: k_raster shades each tile too, so the frame's
  // stores cross to the host while later tiles are still rasterised instead
  // of all at the end (measured: 0.156 against 0.173 ms a 1280x720 frame).
  const bool separate = nviews == 1 && !views[0].host_out;
  if (separate && total_pixels > c->pkey_pixels) {
    CK(cudaStreamSynchronize(c->stream));
    dev_free(c->pkey);
    dev_free(c->slot_keys);
    c->pkey_pixels = 0;
    if ((st = dev_alloc(&c->pkey, (size_t)total_pixels)) || (st = dev_alloc(&c->slot_keys, 4 * (size_t)total_pixels)))
      return st;
    c->pkey_pixels = total_pixels;
  }
  // Synchronous draws stage in a slot of their own (the previous one has
  // finished), read by the frame's graph; the others rotate through the
  // ring, each slot reused once the k_stage (or the frame) that read it has run.
  const bool in_graph = upload != Upload::kCopy && !own_views && !own_items;
  const bool sync_slot = in_graph && upload == Upload::kInGraph;
  const int slot = sync_slot ? kStageSlots : (c->stage_slot + 1) % kStageSlots;
  if (!sync_slot && c->stage_used[slot]) CK(cudaEventSynchronize(c->stage_ev[slot]));
  unsigned char* hslot = c->h_tables + (size_t)slot * c->tables_stride;
  DevView* hviews = reinterpret_cast<DevView*>(hslot);
  DevItem* hitems = reinterpret_cast<DevItem*>(hslot + c->tables_off);
  uint32_t tile_base = 0;
  uint64_t pix_base = 0;
  for (int v = 0; v < nviews; ++v) {
    const gr_frame_params* p = views[v].p;
    DevView& d = hviews[v];
    std::memset(&d, 0, sizeof(d));
    d.W = p->width;
    d.H = p->height;
    d.flags = p->flags;
    d.tiles_x = (p->width + ts - 1) / ts;
    d.tiles_y = (p->height + ts - 1) / ts;
    d.tile_base = tile_base;
    tile_base += (uint32_t)(d.tiles_x * d.tiles_y);
    for (int k = 0; k < 8; ++k) d.S[k] = p->screen[k];
    for (int k = 0; k < 3; ++k) d.L[k] = p->light[k];
    d.out_rgba = views[v].rgba;
    d.out_z = views[v].z;
    d.pix_base = pix_base;
    pix_base += (uint64_t)p->width * (uint64_t)p->height;
    d.fog_on = c->fog_on && !(p->flags & kViewFaceIds);
    d.fog_start = c->fog_start;
    d.fog_end = c->fog_end;
    d.fog_color = c->fog_color;
    d.vec_ok = (p->width % 4 == 0) && ((uintptr_t)d.out_rgba % 16 == 0) && ((uintptr_t)d.out_z % 16 == 0);
  }
  uint64_t faces = 0;
  int blocks = 0;
  int light_blocks = 0;
  uint64_t light_total = 0;
  uint64_t vert_total = 0;
  int vert_blocks = 0;
  int live = 0;
  uint64_t all_faces = 0;
  for (int i = 0; i < n; ++i) {
    const int m = items[i].mesh;
    if (m >= 0 && m < (int)c->meshes.size() && c->meshes[m].alive) all_faces += (uint64_t)c->meshes[m].nf;
  }
  const int project_g = project_faces_per_lane(all_faces);
  const int project_faces = kProjectThreads * project_g;
  for (int i = 0; i < n; ++i) {
    const int m = items[i].mesh;
    if (m < 0 || m >= (int)c->meshes.size() || !c->meshes[m].alive)
      return fail(GR_ERR_INVALID_ARGUMENT, "item %d: unknown mesh %d", i, m);
    const int view = batched ? items[i].reserved : 0;
    if (view < 0 || view >= nviews) return fail(GR_ERR_INVALID_ARGUMENT, "item %d: view %d of %d", i, view, nviews);
    const uint32_t fl = views[view].p->flags;
    const bool gouraud = (fl & GR_LIGHTING) && !(fl & GR_FLAT_SHADING);
    const MeshRec& mr = c->meshes[m];
    if (gouraud && mr.nn > 0 && !mr.nidx_ok)
      return fail(GR_ERR_BAD_INDEX, "item %d: mesh %d has missing or out-of-range normal indices", i, m);
    const uint64_t fb = faces;
    faces += (uint64_t)mr.nf;
    if (mr.nf == 0) continue;  // an empty mesh draws nothing
    DevItem& d = hitems[live++];
    std::memcpy(d.mvp, items[i].mvp, sizeof(d.mvp));
    std::memcpy(d.world, items[i].world, sizeof(d.world));
    std::memcpy(d.bbox, mr.bbox, sizeof(d.bbox));
    d.vis = box_visibility(d.mvp, d.bbox);
    d.pos = mr.pos; d.vnrm = mr.vnrm; d.fnrm = mr.fnrm; d.vidx = mr.vidx; d.nidx = mr.nidx;
    d.uv = mr.uv; d.tex = mr.tex; d.vcol = mr.vcol;
    d.nv = mr.nv; d.nn = mr.nn; d.nf = mr.nf;
    d.face_base = (uint32_t)fb;
    d.block_base = blocks;
    d.view = view;
    d.vert_base = (uint32_t)vert_total;
    d.vert_block_base = vert_blocks;
    vert_total += (uint64_t)mr.nv;
    vert_blocks += (mr.nv + 256 * project_g - 1) / (256 * project_g);
    blocks += (mr.nf + project_faces - 1) / project_faces;
    // every item gets a k_light block range (empty for non-Gouraud items) so the
    // kernel's block -> item search sees non-decreasing bases
    d.light_base = (int)light_total;
    d.light_block_base = light_blocks;
    if (gouraud && mr.nn > 0) {
      light_total += (uint64_t)mr.nn;
      light_blocks += (mr.nn + 256 * project_g - 1) / (256 * project_g);
    }
  }
  if (faces >= (1ull << 28)) return fail(GR_ERR_UNSUPPORTED, "more than 2^28 faces in one frame");
  if ((st = ensure_frame_buffers(c, faces, total_tiles))) return st;
  if (flags_any & (GR_SHOW_EDGES | GR_SHOW_VERTICES)) {
    const uint64_t want_ovl = std::max<uint64_t>(c->want_ovl_cap, std::min<uint64_t>(faces + 1024, 1u << 30));
    if (want_ovl > c->ovl_cap) {
      CK(cudaStreamSynchronize(c->stream));
      dev_free(c->ovl);
      c->ovl_cap = 0;
      if ((st = dev_alloc(&c->ovl, want_ovl))) return st;
      c->ovl_cap = (uint32_t)want_ovl;
    }
  }
  if (vert_total >= (1ull << 31)) return fail(GR_ERR_UNSUPPORTED, "more than 2^31 vertices in one frame");
  if (vert_total > c->vert_cap) {
    CK(cudaStreamSynchronize(c->stream));
    dev_free(c->vclip);
    dev_free(c->vscr);
    c->vert_cap = 0;
    const uint64_t cap = std::max<uint64_t>(vert_total, 1024);
    if ((st = dev_alloc(&c->vclip, cap)) || (st = dev_alloc(&c->vscr, cap))) return st;
    c->vert_cap = cap;
  }
  if (light_total > c->vlight_cap) {
    CK(cudaStreamSynchronize(c->stream));
    dev_free(c->vlight);
    c->vlight_cap = 0;
    if ((st = dev_alloc(&c->vlight, light_total))) return st;
    c->vlight_cap = light_total;
  }
  // a graph batch keeps its own tables, so other draws cannot overwrite them
  DevView* dviews = own_views ? own_views : c->d_views;
  DevItem* ditems = own_items ? own_items : c->d_items;
  if (in_graph) {  // both tables copied by k_stage, the first kernel of the frame's graph
    const size_t bytes = live ? c->tables_off + sizeof(DevItem) * (size_t)live : sizeof(DevView) * (size_t)nviews;
    out.copy_src = hslot;
    out.copy_bytes = bytes;
    c->h2d_bytes = (int64_t)bytes;
  } else if (!own_views && !own_items) {  // both tables with one k_stage, before the frame's graph
    const size_t bytes = live ? c->tables_off + sizeof(DevItem) * (size_t)live : sizeof(DevView) * (size_t)nviews;
    CK((cudaError_t)launch_stage(c->d_tables, hslot, bytes, c->stream));
    c->h2d_bytes = (int64_t)bytes;
  } else {  // tables of their own (batches, the differentiable pass): one k_stage each
    CK((cudaError_t)launch_stage(dviews, hviews, sizeof(DevView) * nviews, c->stream));
    if (live) CK((cudaError_t)launch_stage(ditems, hitems, sizeof(DevItem) * live, c->stream));
    c->h2d_bytes = (int64_t)sizeof(DevItem) * live + (int64_t)sizeof(DevView) * nviews;
  }
  if (!in_graph) {
    CK(cudaEventRecord(c->stage_ev[slot], c->stream));
    c->stage_used[slot] = true;
    c->stage_slot = slot;
  } else if (!sync_slot) {
    out.ring_slot = slot;
    c->stage_slot = slot;
  }
  c->d2h_bytes = 0;

  FrameArgs& a = out.a;
  std::memset(&a, 0, sizeof(a));
  a.views = dviews;
  a.num_views = nviews;
  a.total_tiles = total_tiles;
  a.flags_any = flags_any;
  a.tile_shift = c->tile_shift;
  a.num_items = live;
  a.total_blocks = blocks;
  a.project_g = project_g;
  a.bin_cap = c->bin_cap;
  a.rec_cap = c->rec_cap;
  a.big_cap = c->big_cap;
  a.items = ditems;
  a.texs = c->d_texs;
  a.num_tex = (int)c->texs.size();
  a.rast = c->rast;
  a.shade = c->shade;
  a.suv = c->suv;
  a.wide = c->wide;
  a.tcol = c->tcol;
  a.rec_of_face = c->rec_of_face;
  a.face_cap = c->face_cap;
  a.bins = c->bins;
  a.bin_count = c->bin_count;
  a.tile_cost = c->tile_cost;
  a.big = c->big;
  a.gkey = c->gkey;
  a.tile_done = c->tile_done;
  a.slice_cost = c->slice_cost;
  a.clip = c->clip;
  a.clip_cap = c->clip_cap;
  a.kept = c->kept;
  a.kept_cap = c->kept_cap;
  a.setup_blocks = (int)std::min<uint64_t>(setup_blocks_max(project_g), (faces + kProjectThreads - 1) / kProjectThreads);
  a.vlight = c->vlight;
  a.light_blocks = light_blocks;
  a.vclip = c->vclip;
  a.vscr = c->vscr;
  a.vert_blocks = vert_blocks;
  a.work = c->work;
  a.result = c->d_result;
  a.view_tpf = c->view_tpf;
  a.view_tpf_out = c->view_tpf_out;
  a.plan = c->plan;
  a.plan_cap = c->plan_cap;
  a.raster_ctas = raster_grid(c->tile_shift, c->raster_waves);
  a.ovl = c->ovl;
  a.ovl_cap = c->ovl_cap;
  a.ovl_key = c->ovl_key;
  a.pkey = separate ? c->pkey : nullptr;
  a.tile_info = c->tile_info;
  a.slot_keys = separate ? c->slot_keys : nullptr;
  a.slot_cap = separate ? (uint32_t)std::min<uint64_t>((4 * c->pkey_pixels) >> (2 * c->tile_shift), 0xFFFFFFF0u) : 0u;
  // Many views shaded in place: tiles without bin entries (most of a batch
  // of small meshes) are cleared by the raster CTAs once their queue is
  // empty, without keys (a 256-view batch 1.81 -> 1.62 ms with a kernel of
  // their own, 1.335 -> 1.286 ms inside k_raster); one view keeps them in the
  // raster queue (0.153 against 0.166 ms a frame with the separate kernel).
  a.clear_empty = (!separate && nviews > 1) ? 1 : 0;
  if (a.clear_empty && total_tiles > c->empty_cap) {  // allocated only for such frames
    CK(cudaStreamSynchronize(c->stream));
    dev_free(c->empty_tiles);
    c->empty_cap = 0;
    if ((st = dev_alloc(&c->empty_tiles, (size_t)total_tiles))) return st;
    c->empty_cap = total_tiles;
  }
  a.empty_tiles = c->empty_tiles;
  a.empty_cap = c->empty_cap;
  a.total_pixels = total_pixels;
  out.faces = faces;
  out.nitems = live;
  return GR_OK;
}

// Launches a frame's kernels.  The arguments are the same from frame to frame
// while a scene's counts and the buffers stay (items and views are read from
// device tables), so each launch sequence is captured once into a CUDA graph
// and replayed; a few are kept (least recently used goes first), so a caller
// alternating between scenes replays too.
int32_t launch(gr_context* c, const FrameArgs& a, void* const* events = nullptr, const void* copy_src = nullptr,
               size_t copy_bytes = 0) {
  int big_blocks = kBigBlocks;
  if (!events) {
    ++c->frame_tick;
    int victim = 0;
    for (int k = 0; k < kFrameGraphs; ++k) {
      FrameGraph& fg = c->frame_graphs[k];
      if (fg.exec && fg.copy_src == copy_src && fg.copy_bytes == copy_bytes &&
          std::memcmp(&a, &fg.args, sizeof(a)) == 0) {
        CK(cudaGraphLaunch(fg.exec, c->stream));
        fg.used = c->frame_tick;
        c->last_launches = fg.launches;
        return GR_OK;
      }
      if (fg.used < c->frame_graphs[victim].used) victim = k;
    }
    FrameGraph& fg = c->frame_graphs[victim];
    if (fg.exec) cudaGraphExecDestroy(fg.exec);
    fg.exec = nullptr;
    cudaGraph_t g = nullptr;
    int n = 0;
    if (cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      int err = 0;
      if (copy_bytes) err = launch_stage(c->d_tables, copy_src, copy_bytes, c->stream);
      if (!err) err = launch_frame(a, big_blocks, c->stream, &n, nullptr, &c->aux);
      if (copy_bytes) ++n;  // k_stage
      const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
      if (!err && e == cudaSuccess && g && cudaGraphInstantiate(&fg.exec, g, 0) == cudaSuccess) {
        cudaGraphDestroy(g);
        std::memcpy(&fg.args, &a, sizeof(a));
        fg.copy_src = copy_src;
        fg.copy_bytes = copy_bytes;
        fg.launches = n;
        fg.used = c->frame_tick;
        CK(cudaGraphLaunch(fg.exec, c->stream));
        c->last_launches = n;
        return GR_OK;
      }
      if (g) cudaGraphDestroy(g);
      fg.exec = nullptr;
      cudaGetLastError();  // capture failed: fall back to plain launches
    }
  }
  if (copy_bytes) CK((cudaError_t)launch_stage(c->d_tables, copy_src, copy_bytes, c->stream));
  int err = launch_frame(a, big_blocks, c->stream, &c->last_launches, events, &c->aux);
  if (err) return fail(GR_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString((cudaError_t)err));
  if (copy_bytes) ++c->last_launches;  // k_stage
  return GR_OK;
}

// Identity of every context buffer a captured graph refers to: a graph whose
// signature no longer matches must be captured again before it runs.
uint64_t buffers_signature(const gr_context* c) {
  const uintptr_t ps[] = {(uintptr_t)c->rast, (uintptr_t)c->shade, (uintptr_t)c->suv, (uintptr_t)c->wide, (uintptr_t)c->tcol,
                          (uintptr_t)c->rec_of_face, (uintptr_t)c->bins, (uintptr_t)c->bin_count, (uintptr_t)c->tile_cost, (uintptr_t)c->tile_info, (uintptr_t)c->gkey,
                          (uintptr_t)c->tile_done, (uintptr_t)c->clip, (uintptr_t)c->kept, c->kept_cap, (uintptr_t)c->big, (uintptr_t)c->vlight,
                          (uintptr_t)c->vclip, (uintptr_t)c->vscr,
                          (uintptr_t)c->d_texs, (uintptr_t)c->view_tpf, (uintptr_t)c->view_tpf_out,
                          (uintptr_t)c->h_view_tpf, (uintptr_t)c->plan, (uintptr_t)c->empty_tiles, c->empty_cap, c->rec_cap, c->face_cap, c->bin_cap,
                          c->big_cap, c->clip_cap, c->plan_cap, (uintptr_t)c->tile_shift, c->slice_cost,
                          (uintptr_t)c->raster_waves, c->texs.size(), (uintptr_t)c->ovl, (uintptr_t)c->ovl_key, (uintptr_t)c->pkey, (uintptr_t)c->slot_keys,
                          c->ovl_cap};
  uint64_t h = 1469598103934665603ull;  // FNV-1a over the words
  for (uintptr_t v : ps) {
    h ^= (uint64_t)v;
    h *= 1099511628211ull;
  }
  return h;
}

// Reads a frame's result; grows buffers that overflowed.  Returns 1 when the
// frame must be re-run.  The kernels record a *_need value only when an
// append did not fit, so any non-zero one means the frame is incomplete,
// even if the buffers have grown since it was queued (asynchronous frames).
int check_result(gr_context* c, const DevResult& r, int32_t* err) {
  *err = GR_OK;
  int rerun = 0;
  auto grow = [&](uint32_t need, uint32_t cap, uint32_t& want, uint64_t size) {
    if (!need) return;
    rerun = 1;
    if (need > cap) want = (uint32_t)std::min<uint64_t>(size, 0xFFFFFFFFull);
  };
  grow(r.bin_need, c->bin_cap, c->want_bin_cap, next_pow2((uint64_t)r.bin_need + r.bin_need / 4));
  grow(r.rec_need, c->rec_cap, c->want_rec_cap, (uint64_t)r.rec_need + r.rec_need / 8);
  grow(r.big_need, c->big_cap, c->want_big_cap, next_pow2((uint64_t)r.big_need + r.big_need / 4));
  grow(r.clip_need, c->clip_cap, c->want_clip_cap, next_pow2((uint64_t)r.clip_need + r.clip_need / 4));
  grow(r.ovl_need, c->ovl_cap, c->want_ovl_cap, next_pow2((uint64_t)r.ovl_need + r.ovl_need / 4));
  if (r.error & 1u) *err = fail(GR_ERR_CLIP_OVERFLOW, "a clipped polygon exceeded 9 vertices");
  if (r.error & 4u)
    *err = fail(GR_ERR_UNSUPPORTED, "an edge overlay line has more than %lld steps (a corner far off screen)",
                (long long)kMaxLineSteps);
  return rerun;
}

// After a kRingInGraph launch: the slot may be rewritten once this frame has run.
int32_t record_ring_slot(gr_context* c, const Prepared& pr) {
  if (pr.ring_slot < 0) return GR_OK;
  CK(cudaEventRecord(c->stage_ev[pr.ring_slot], c->stream));
  c->stage_used[pr.ring_slot] = true;
  return GR_OK;
}

int32_t draw_sync(gr_context* c, const gr_draw_item* items, int32_t n, const gr_frame_params* p,
                  uint8_t* rgba_out, float* z_out, int64_t* tpf_out) {
  if (!p) return fail(GR_ERR_INVALID_ARGUMENT, "params is NULL");
  const size_t px = (size_t)p->width * (size_t)p->height;
  // page-locked host outputs are written by the kernels through their device
  // addresses; pageable ones are copied from the context's framebuffer
  bool rgba_dev, z_dev;
  uint32_t* rgba_map = (uint32_t*)classify_out_ptr(rgba_out, &rgba_dev);
  float* z_map = (float*)classify_out_ptr(z_out, &z_dev);
  int32_t st;
  for (int attempt = 0; attempt < 4; ++attempt) {
    uint32_t* rgba = rgba_dev ? (uint32_t*)rgba_out : rgba_map;
    float* z = z_dev ? z_out : z_map;
    if (!rgba || !z) {
      if (p->width <= 0 || p->height <= 0) return fail(GR_ERR_INVALID_ARGUMENT, "bad framebuffer size");
      if ((st = ensure_fb(c, px))) return st;
      if (!rgba) rgba = c->fb_rgba;
      if (!z) z = c->fb_z;
    }
    ViewIn v{p, rgba, z};
    v.host_out = rgba_map || z_map;
    Prepared pr;
    if ((st = prepare(c, &v, 1, items, n, false, pr, nullptr, nullptr, Upload::kInGraph))) return st;
    // the counters and the outputs in one go: one host wait per frame (a frame
    // whose buffers overflowed is drawn again and its outputs copied again);
    // the last raster CTA writes the counters into page-locked memory itself,
    // then sets the done word after them
    pr.a.result_host = c->h_result_dev;
    volatile uint32_t* done = reinterpret_cast<volatile uint32_t*>(c->h_result + 1);
    *done = 0u;
    if ((st = launch(c, pr.a, nullptr, pr.copy_src, pr.copy_bytes))) return st;
    c->d2h_bytes = (int64_t)sizeof(DevResult);
    if (rgba_out && !rgba_dev) {
      if (!rgba_map) CK(cudaMemcpyAsync(rgba_out, rgba, px * 4, cudaMemcpyDeviceToHost, c->stream));
      c->d2h_bytes += (int64_t)px * 4;
    }
    if (z_out && !z_dev) {
      if (!z_map) CK(cudaMemcpyAsync(z_out, z, px * 4, cudaMemcpyDeviceToHost, c->stream));
      c->d2h_bytes += (int64_t)px * 4;
    }
    if (!v.host_out || (rgba_out && !rgba_dev && !rgba_map) || (z_out && !z_dev && !z_map)) {
      // device outputs (k_resolve runs after the raster) or copies after the frame
      CK(cudaStreamSynchronize(c->stream));
    } else {
      // Wait for the done word (counters and outputs are in host memory by
      // then) rather than for the whole stream; past a second (a fault, or a
      // device taken by other work) the stream wait decides and reports.
      bool seen = false;
      const auto t0 = std::chrono::steady_clock::now();
      for (uint32_t spins = 0;; ++spins) {
        if (__atomic_load_n(reinterpret_cast<const uint32_t*>(c->h_result + 1), __ATOMIC_ACQUIRE)) {
          seen = true;
          break;
        }
        if ((spins & 1023u) == 1023u && std::chrono::steady_clock::now() - t0 > std::chrono::seconds(1)) break;
      }
      if (!seen) CK(cudaStreamSynchronize(c->stream));
    }
    int32_t err;
    const int rerun = check_result(c, *c->h_result, &err);
    if (err) return err;
    if (rerun) {
      CK(cudaStreamSynchronize(c->stream));  // before buffers are resized
      continue;
    }
    if (tpf_out) *tpf_out = (int64_t)c->h_result->tpf;
    return GR_OK;
  }
  return fail(GR_ERR_OUT_OF_MEMORY, "frame buffers kept overflowing after resizing");
}

}  // namespace

namespace gr {
int32_t set_error(int32_t code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}
}  // namespace gr

extern "C" {

const char* gr_last_error(void) { return g_err.c_str(); }
const char* gr_version(void) { return "gorender-gb300 0.1 (sm_103a)"; }

int32_t gr_context_create(int32_t device, gr_context** out) {
  if (!out) return fail(GR_ERR_INVALID_ARGUMENT, "out is NULL");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return fail(GR_ERR_NO_DEVICE, "no CUDA device");
  }
  if (device < 0 || device >= ndev) return fail(GR_ERR_INVALID_ARGUMENT, "device %d of %d", device, ndev);
  CK(cudaSetDevice(device));
  gr_context* c = new (std::nothrow) gr_context();
  if (!c) return fail(GR_ERR_OUT_OF_MEMORY, "context allocation");
  c->device = device;
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc((void**)&c->work, sizeof(DevWork));
  if (e == cudaSuccess) e = cudaMemset(c->work, 0, sizeof(DevWork));
  if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_result, sizeof(DevResult));
  if (e == cudaSuccess) e = cudaMemset(c->d_result, 0, sizeof(DevResult));
  if (e == cudaSuccess) e = cudaMallocHost((void**)&c->h_result, 2 * sizeof(DevResult));  // + the done word
  if (e == cudaSuccess) e = cudaHostGetDevicePointer((void**)&c->h_result_dev, c->h_result, 0);
  for (int i = 0; i < 64 && e == cudaSuccess; ++i) e = cudaEventCreate(&c->events[i]);
  for (int i = 0; i < kStageSlots && e == cudaSuccess; ++i)
    e = cudaEventCreateWithFlags(&c->stage_ev[i], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->aux_stream, cudaStreamNonBlocking);
  for (int i = 0; i < 6 && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&c->aux_ev[i], cudaEventDisableTiming);
  if (e == cudaSuccess) {
    c->aux.stream = c->aux_stream;
    c->aux.fork[0] = c->aux_ev[0]; c->aux.join[0] = c->aux_ev[1];
    c->aux.fork[1] = c->aux_ev[2]; c->aux.join[1] = c->aux_ev[3];
    c->aux.fork[2] = c->aux_ev[4]; c->aux.join[2] = c->aux_ev[5];
  }
  if (e != cudaSuccess) {
    gr_context_destroy(c);
    return fail(GR_ERR_CUDA, "context setup: %s", cudaGetErrorString(e));
  }
  *out = c;
  return GR_OK;
}

int32_t gr_context_destroy(gr_context* c) {
  if (!c) return GR_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (auto& m : c->meshes) {
    dev_free(m.pos); dev_free(m.vnrm); dev_free(m.fnrm); dev_free(m.uv); dev_free(m.vcol);
    dev_free(m.vidx); dev_free(m.nidx); dev_free(m.tex);
  }
  for (auto& t : c->texs) if (t.px) cudaFree(t.px);
  dev_free(c->d_texs); dev_free(c->d_tables);
  if (c->h_tables) cudaFreeHost(c->h_tables);
  dev_free(c->rast); dev_free(c->shade); dev_free(c->suv); dev_free(c->wide); dev_free(c->tcol);
  dev_free(c->rec_of_face); dev_free(c->bins); dev_free(c->bin_count); dev_free(c->tile_cost); dev_free(c->tile_info);
  dev_free(c->big);
  dev_free(c->gkey); dev_free(c->tile_done); dev_free(c->clip); dev_free(c->kept); dev_free(c->vlight);
  dev_free(c->vclip); dev_free(c->vscr);
  dev_free(c->view_tpf); dev_free(c->view_tpf_out); dev_free(c->plan); dev_free(c->empty_tiles);
  dev_free(c->ovl); dev_free(c->ovl_key); dev_free(c->pkey); dev_free(c->slot_keys);
  if (c->h_view_tpf) cudaFreeHost(c->h_view_tpf);
  dev_free(c->work); dev_free(c->d_result);
  if (c->h_result) cudaFreeHost(c->h_result);
  dev_free(c->fb_rgba); dev_free(c->fb_z);
  if (c->flush_buf) cudaFree(c->flush_buf);
  for (auto& ev : c->events) if (ev) cudaEventDestroy(ev);
  for (auto& ev : c->stage_ev) if (ev) cudaEventDestroy(ev);
  for (auto& fg : c->frame_graphs)
    if (fg.exec) cudaGraphExecDestroy(fg.exec);
  for (auto& ev : c->aux_ev) if (ev) cudaEventDestroy(ev);
  if (c->aux_stream) cudaStreamDestroy(c->aux_stream);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return GR_OK;
}

int32_t gr_context_sync(gr_context* c) {
  if (!c) return fail(GR_ERR_INVALID_ARGUMENT, "ctx is NULL");
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  CK(cudaMemcpyAsync(c->h_result, c->d_result, sizeof(DevResult), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  int32_t st = c->pending;
  c->pending = GR_OK;
  int32_t err;
  if (check_result(c, *c->h_result, &err) && !st)
    st = fail(GR_ERR_BIN_OVERFLOW, "a frame overflowed its buffers; they have been grown, re-issue it");
  if (err && !st) st = err;
  return st;
}

int32_t gr_mesh_create(gr_context* c, const gr_mesh_desc* d, int32_t* mesh_out) {
  if (!c || !d || !mesh_out) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  if (d->num_vertices <= 0 || d->num_faces < 0 || !d->positions || (d->num_faces > 0 && !d->vertex_indices))
    return fail(GR_ERR_INVALID_ARGUMENT, "mesh needs positions and vertex indices");
  if (d->num_normals < 0 || (d->num_normals > 0 && !d->vertex_normals))
    return fail(GR_ERR_INVALID_ARGUMENT, "bad vertex normals");
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  const int nv = d->num_vertices, nf = d->num_faces, nn = d->num_normals;
  for (long i = 0; i < 3L * nf; ++i)
    if (d->vertex_indices[i] < 0 || d->vertex_indices[i] >= nv)
      return fail(GR_ERR_BAD_INDEX, "face %ld: vertex index %d out of range [0,%d)", i / 3, d->vertex_indices[i], nv);
  if (d->face_textures)
    for (int i = 0; i < nf; ++i)
      if (d->face_textures[i] >= (int)c->texs.size())
        return fail(GR_ERR_BAD_INDEX, "face %d: unknown texture %d", i, d->face_textures[i]);
  MeshRec m;
  m.nv = nv; m.nn = nn; m.nf = nf;
  m.has_nidx = d->normal_indices != nullptr;
  m.nidx_ok = m.has_nidx;
  if (m.has_nidx)
    for (long i = 0; i < 3L * nf && m.nidx_ok; ++i)
      if (d->normal_indices[i] < 0 || d->normal_indices[i] >= nn) m.nidx_ok = false;
  bounding_box(d->positions, nv, m.bbox);
  std::vector<float> fn;
  const float* fnp = d->face_normals;
  if (!fnp && nf > 0) {
    fn.resize((size_t)nf * 4);
    face_normals(d->positions, d->vertex_indices, nf, fn.data());
    fnp = fn.data();
  }
  int32_t st;
  if ((st = upload(c, &m.pos, d->positions, (size_t)nv * 4)) || (st = upload(c, &m.vnrm, d->vertex_normals, (size_t)nn * 4)) ||
      (st = upload(c, &m.fnrm, fnp, (size_t)nf * 4)) || (st = upload(c, &m.vidx, d->vertex_indices, (size_t)nf * 3)) ||
      (st = upload(c, &m.nidx, m.nidx_ok ? d->normal_indices : nullptr, (size_t)nf * 3)) ||
      (st = upload(c, &m.uv, d->uvs, (size_t)nf * 6)) || (st = upload(c, &m.tex, d->face_textures, (size_t)nf)) ||
      (st = upload(c, &m.vcol, d->vertex_colors, (size_t)nv * 3))) {
    dev_free(m.pos); dev_free(m.vnrm); dev_free(m.fnrm); dev_free(m.vidx); dev_free(m.nidx);
    dev_free(m.uv); dev_free(m.tex); dev_free(m.vcol);
    return st;
  }
  CK(cudaStreamSynchronize(c->stream));  // host arrays may be released after return
  m.alive = true;
  c->meshes.push_back(m);
  *mesh_out = (int32_t)c->meshes.size() - 1;
  return GR_OK;
}

int32_t gr_mesh_destroy(gr_context* c, int32_t mesh) {
  if (!c) return fail(GR_ERR_INVALID_ARGUMENT, "ctx is NULL");
  std::lock_guard<std::mutex> lk(c->mu);
  if (mesh < 0 || mesh >= (int)c->meshes.size() || !c->meshes[mesh].alive)
    return fail(GR_ERR_INVALID_ARGUMENT, "unknown mesh %d", mesh);
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));
  MeshRec& m = c->meshes[mesh];
  dev_free(m.pos); dev_free(m.vnrm); dev_free(m.fnrm); dev_free(m.vidx); dev_free(m.nidx);
  dev_free(m.uv); dev_free(m.tex); dev_free(m.vcol);
  m.alive = false;
  return GR_OK;
}

int32_t gr_mesh_bounding_box(gr_context* c, int32_t mesh, float* out32) {
  if (!c || !out32) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  std::lock_guard<std::mutex> lk(c->mu);
  if (mesh < 0 || mesh >= (int)c->meshes.size() || !c->meshes[mesh].alive)
    return fail(GR_ERR_INVALID_ARGUMENT, "unknown mesh %d", mesh);
  std::memcpy(out32, c->meshes[mesh].bbox, sizeof(float) * 32);
  return GR_OK;
}

int32_t gr_texture_create(gr_context* c, int32_t kind, int32_t width, int32_t height, const uint8_t* rgba,
                          float scale, const uint8_t* color, int32_t* tex_out) {
  if (!c || !tex_out) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  TexRec t;
  std::memset(&t.d, 0, sizeof(t.d));
  t.d.kind = kind;
  t.d.scale = scale;
  if (kind == GR_TEXTURE_SOLID) {
    if (!color) return fail(GR_ERR_INVALID_ARGUMENT, "solid texture needs a colour");
    t.d.color = (uint32_t)color[0] | ((uint32_t)color[1] << 8) | ((uint32_t)color[2] << 16) | ((uint32_t)color[3] << 24);
  } else if (kind == GR_TEXTURE_IMAGE || kind == GR_TEXTURE_IMAGE_FAST) {
    if (width <= 0 || height <= 0 || !rgba) return fail(GR_ERR_INVALID_ARGUMENT, "image texture needs pixels");
    bool pow2 = (width & (width - 1)) == 0 && (height & (height - 1)) == 0;
    if (kind == GR_TEXTURE_IMAGE_FAST && !pow2)
      return fail(GR_ERR_INVALID_ARGUMENT, "IMAGE_FAST needs power-of-two sizes");
    t.d.width = width;
    t.d.height = height;
    t.d.widthF = (float)width;
    t.d.heightF = (float)height;
    CK(cudaMalloc(&t.px, (size_t)width * height * 4));
    CK(cudaMemcpy(t.px, rgba, (size_t)width * height * 4, cudaMemcpyHostToDevice));
    t.d.px = (const uint32_t*)t.px;
  } else {
    return fail(GR_ERR_INVALID_ARGUMENT, "unknown texture kind %d", kind);
  }
  c->texs.push_back(t);
  c->texs_dirty = true;
  *tex_out = (int32_t)c->texs.size() - 1;
  return GR_OK;
}

int32_t gr_draw(gr_context* c, const gr_draw_item* items, int32_t n, const gr_frame_params* p,
                uint8_t* rgba_out, float* z_out, int64_t* tpf_out) {
  if (!c) return fail(GR_ERR_INVALID_ARGUMENT, "ctx is NULL");
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  return draw_sync(c, items, n, p, rgba_out, z_out, tpf_out);
}

int32_t gr_draw_async(gr_context* c, const gr_draw_item* items, int32_t n, const gr_frame_params* p,
                      uint8_t* rgba_dev, float* z_dev) {
  if (!c || !p) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  if ((rgba_dev && !is_device_ptr(rgba_dev)) || (z_dev && !is_device_ptr(z_dev)))
    return fail(GR_ERR_INVALID_ARGUMENT, "gr_draw_async needs device output pointers");
  int32_t st;
  const size_t px = (size_t)p->width * (size_t)p->height;
  if (!rgba_dev || !z_dev) {
    if (p->width <= 0 || p->height <= 0) return fail(GR_ERR_INVALID_ARGUMENT, "bad framebuffer size");
    if ((st = ensure_fb(c, px))) return st;
  }
  ViewIn v{p, rgba_dev ? (uint32_t*)rgba_dev : c->fb_rgba, z_dev ? z_dev : c->fb_z};
  Prepared pr;
  if ((st = prepare(c, &v, 1, items, n, false, pr, nullptr, nullptr, Upload::kRingInGraph))) return st;
  if ((st = launch(c, pr.a, nullptr, pr.copy_src, pr.copy_bytes))) return st;
  return record_ring_slot(c, pr);
}

int32_t gr_draw_profiled(gr_context* c, const gr_draw_item* items, int32_t n, const gr_frame_params* p,
                         uint8_t* rgba_dev, float* z_dev, float* kernel_ms3) {
  if (!c || !kernel_ms3 || !p) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  if ((rgba_dev && !is_device_ptr(rgba_dev)) || (z_dev && !is_device_ptr(z_dev)))
    return fail(GR_ERR_INVALID_ARGUMENT, "gr_draw_profiled needs device output pointers");
  const size_t px = (size_t)p->width * (size_t)p->height;
  int32_t st;
  for (int attempt = 0; attempt < 4; ++attempt) {
    if (!rgba_dev || !z_dev) {
      if (p->width <= 0 || p->height <= 0) return fail(GR_ERR_INVALID_ARGUMENT, "bad framebuffer size");
      if ((st = ensure_fb(c, px))) return st;
    }
    ViewIn v{p, rgba_dev ? (uint32_t*)rgba_dev : c->fb_rgba, z_dev ? z_dev : c->fb_z};
    Prepared pr;
    if ((st = prepare(c, &v, 1, items, n, false, pr))) return st;
    void* ev[4] = {c->events[60], c->events[61], c->events[62], c->events[63]};
    if ((st = launch(c, pr.a, ev))) return st;
    CK(cudaMemcpyAsync(c->h_result, c->d_result, sizeof(DevResult), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    int32_t err;
    int rerun = check_result(c, *c->h_result, &err);
    if (err) return err;
    if (rerun) continue;
    for (int k = 0; k < 3; ++k) CK(cudaEventElapsedTime(&kernel_ms3[k], c->events[60 + k], c->events[61 + k]));
    return GR_OK;
  }
  return fail(GR_ERR_OUT_OF_MEMORY, "frame buffers kept overflowing after resizing");
}

// ---- batched views ----

static int32_t views_in(gr_context* c, const gr_view* views, int32_t nv, std::vector<ViewIn>& out) {
  if (nv <= 0 || !views) return fail(GR_ERR_INVALID_ARGUMENT, "no views");
  out.resize((size_t)nv);
  for (int v = 0; v < nv; ++v) {
    if (!views[v].rgba_dev || !views[v].z_dev || !is_device_ptr(views[v].rgba_dev) || !is_device_ptr(views[v].z_dev))
      return fail(GR_ERR_INVALID_ARGUMENT, "view %d: outputs must be device pointers", v);
    out[v] = ViewIn{&views[v].params, (uint32_t*)views[v].rgba_dev, views[v].z_dev};
  }
  (void)c;
  return GR_OK;
}

int32_t gr_draw_views(gr_context* c, const gr_view* views, int32_t nviews, const gr_draw_item* items, int32_t n) {
  if (!c) return fail(GR_ERR_INVALID_ARGUMENT, "ctx is NULL");
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  std::vector<ViewIn> vin;
  int32_t st = views_in(c, views, nviews, vin);
  if (st) return st;
  Prepared pr;
  if ((st = prepare(c, vin.data(), nviews, items, n, true, pr))) return st;
  if ((st = launch(c, pr.a))) return st;
  CK(cudaMemcpyAsync(c->h_view_tpf, c->view_tpf_out, sizeof(unsigned long long) * nviews, cudaMemcpyDeviceToHost,
                     c->stream));
  c->last_views = nviews;
  return GR_OK;
}

int32_t gr_context_view_tpf(gr_context* c, int64_t* tpf, int32_t nviews) {
  if (!c || !tpf || nviews < 0) return fail(GR_ERR_INVALID_ARGUMENT, "bad argument");
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));
  if (nviews > c->last_views) return fail(GR_ERR_INVALID_ARGUMENT, "last batch had %d views", c->last_views);
  for (int v = 0; v < nviews; ++v) tpf[v] = (int64_t)c->h_view_tpf[v];
  return GR_OK;
}

}  // extern "C"

struct gr_batch {
  gr_context* ctx = nullptr;
  std::vector<gr_view> views;
  std::vector<ViewIn> vin;
  std::vector<gr_draw_item> items;
  DevView* d_views = nullptr;  // the batch's own view and item tables
  DevItem* d_items = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  uint64_t signature = 0;      // buffers_signature() at capture
  int launches = 0;
};

namespace {

void batch_drop_graph(gr_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}

// Stages the batch's tables (outside any capture) and captures its frame
// kernels as a CUDA graph.
int32_t batch_capture(gr_batch* b) {
  gr_context* c = b->ctx;
  batch_drop_graph(b);
  const int nv = (int)b->views.size();
  for (int v = 0; v < nv; ++v) b->vin[v].p = &b->views[v].params;
  if (!b->d_views) {
    int32_t st = dev_alloc(&b->d_views, (size_t)nv);
    if (!st) st = dev_alloc(&b->d_items, std::max<size_t>(1, b->items.size()));
    if (st) return st;
  }
  Prepared pr;
  int32_t st = prepare(c, b->vin.data(), nv, b->items.data(), (int)b->items.size(), true, pr, b->d_views, b->d_items);
  if (st) return st;
  // the last raster CTA writes the counters and the per-view TPF into
  // page-locked host memory itself: the graph ends with its kernels, no copy
  unsigned long long* tpf_dev = nullptr;
  CK(cudaHostGetDevicePointer((void**)&tpf_dev, c->h_view_tpf, 0));
  pr.a.result_host = c->h_result_dev;
  pr.a.view_tpf_out = tpf_dev;
  CK(cudaStreamSynchronize(c->stream));
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  int err = launch_frame(pr.a, kBigBlocks, c->stream, &b->launches, nullptr, &c->aux);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(c->stream, &g);
  if (err || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return fail(GR_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e != cudaSuccess ? e : (cudaError_t)err));
  }
  b->graph = g;
  CK(cudaGraphInstantiate(&b->exec, g, 0));
  b->signature = buffers_signature(c);
  c->last_launches = b->launches;
  c->last_views = nv;
  return GR_OK;
}

// Runs the batch once without a graph, growing buffers until it fits; returns
// the device time in ms of the final run.
// Writes 256 MiB (twice the L2) on the context stream so that what follows
// starts from a cold L2.
int32_t cold_l2(gr_context* c, int seed) {
  const size_t flush = 256u << 20;
  if (flush > c->flush_bytes) {
    CK(cudaStreamSynchronize(c->stream));
    if (c->flush_buf) cudaFree(c->flush_buf);
    c->flush_buf = nullptr;
    c->flush_bytes = 0;
    CK(cudaMalloc(&c->flush_buf, flush));
    c->flush_bytes = flush;
  }
  CK(cudaMemsetAsync(c->flush_buf, seed & 0xFF, flush, c->stream));
  return GR_OK;
}

// Raster candidates of the autotuners: tile size (and with it the raster CTA:
// TS*TS/4 threads) x raster cost per slice.
struct TuneCfg {
  int shift, slice, waves;
};
constexpr TuneCfg kTuneCands[] = {{5, 8192, 1}, {5, 16384, 1}, {5, 32768, 1}, {5, 65536, 1}, {5, 131072, 1},
                                  {4, 2048, 1}, {4, 4096, 1}, {4, 8192, 1}, {4, 16384, 1}};

// Runs `run(ms)` (one timed draw that also sizes the buffers) for every
// candidate, keeps the one with the lowest median of five and sizes the tile
// bins to the largest bin seen plus a quarter.
template <class Run>
int32_t autotune_with(gr_context* c, Run run) {
  TuneCfg best = kTuneCands[0];
  float best_ms = 1e30f;
  for (const TuneCfg& k : kTuneCands) {
    c->tile_shift = k.shift;
    c->slice_cost = (uint32_t)k.slice;
    c->raster_waves = k.waves;
    int32_t st = run(nullptr);  // warm up and size the buffers
    if (st) return st;
    float runs[5];
    for (int r = 0; r < 5; ++r) {
      runs[r] = 0.0f;
      if ((st = run(&runs[r]))) return st;
    }
    std::sort(runs, runs + 5);
    if (runs[2] < best_ms) {
      best_ms = runs[2];
      best = k;
    }
  }
  c->tile_shift = best.shift;
  c->slice_cost = (uint32_t)best.slice;
  c->raster_waves = best.waves;
  int32_t st = run(nullptr);
  if (st) return st;
  const uint32_t want = std::max<uint32_t>(256, next_pow2((uint64_t)c->h_result->max_bin + c->h_result->max_bin / 4));
  if (want != c->bin_cap) {
    CK(cudaStreamSynchronize(c->stream));
    dev_free(c->bins);
    dev_free(c->bin_count);
    c->tiles_cap = 0;
    c->bin_cap = 0;
    c->want_bin_cap = want;
  }
  c->tuned_ms = best_ms;
  return run(nullptr);
}

int32_t batch_run_plain(gr_batch* b, float* ms) {
  gr_context* c = b->ctx;
  const int nv = (int)b->views.size();
  for (int attempt = 0; attempt < 5; ++attempt) {
    Prepared pr;
    int32_t st = prepare(c, b->vin.data(), nv, b->items.data(), (int)b->items.size(), true, pr);
    if (st) return st;
    if (ms && (st = cold_l2(c, attempt))) return st;  // time as a frame after other work finds it
    CK(cudaEventRecord(c->events[58], c->stream));
    if ((st = launch(c, pr.a))) return st;
    CK(cudaEventRecord(c->events[59], c->stream));
    CK(cudaMemcpyAsync(c->h_result, c->d_result, sizeof(DevResult), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    int32_t err;
    const int rerun = check_result(c, *c->h_result, &err);
    if (err) return err;
    if (rerun) continue;
    if (ms) CK(cudaEventElapsedTime(ms, c->events[58], c->events[59]));
    return GR_OK;
  }
  return fail(GR_ERR_OUT_OF_MEMORY, "batch buffers kept overflowing after resizing");
}

// Autotuner: raster tile size and slice cost, each candidate timed on the
// batch itself from a cold L2 (median of five runs); then the tile bins are
// sized to the largest bin seen plus a quarter.
int32_t batch_autotune(gr_batch* b) {
  return autotune_with(b->ctx, [b](float* ms) { return batch_run_plain(b, ms); });
}

}  // namespace

extern "C" {

int32_t gr_batch_create(gr_context* c, const gr_view* views, int32_t nviews, const gr_draw_item* items,
                        int32_t nitems, int32_t autotune, gr_batch** out) {
  if (!c || !out || nitems < 0 || (nitems > 0 && !items)) return fail(GR_ERR_INVALID_ARGUMENT, "bad argument");
  *out = nullptr;
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  gr_batch* b = new (std::nothrow) gr_batch();
  if (!b) return fail(GR_ERR_OUT_OF_MEMORY, "batch allocation");
  b->ctx = c;
  b->views.assign(views, views + std::max(nviews, 0));
  b->items.assign(items, items + nitems);
  int32_t st = views_in(c, b->views.data(), nviews, b->vin);
  if (!st) st = autotune ? batch_autotune(b) : batch_run_plain(b, nullptr);
  if (!st) st = batch_capture(b);
  if (st) {
    batch_drop_graph(b);
    delete b;
    return st;
  }
  *out = b;
  return GR_OK;
}

int32_t gr_batch_run(gr_batch* b) {
  if (!b) return fail(GR_ERR_INVALID_ARGUMENT, "batch is NULL");
  gr_context* c = b->ctx;
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  if (b->signature != buffers_signature(c)) {
    // another draw on the context grew or moved a buffer the graph refers to
    int32_t st = batch_capture(b);
    if (st) return st;
  }
  CK(cudaGraphLaunch(b->exec, c->stream));
  c->last_launches = b->launches;
  return GR_OK;
}

int32_t gr_batch_sync(gr_batch* b) {
  if (!b) return fail(GR_ERR_INVALID_ARGUMENT, "batch is NULL");
  gr_context* c = b->ctx;
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));
  int32_t err;
  for (int attempt = 0; attempt < 4; ++attempt) {
    if (!check_result(c, *c->h_result, &err)) return err;
    if (err) return err;
    // overflowed: buffers grow in prepare(); capture again and re-run
    int32_t st = batch_capture(b);
    if (st) return st;
    CK(cudaGraphLaunch(b->exec, c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  return fail(GR_ERR_OUT_OF_MEMORY, "batch buffers kept overflowing after resizing");
}

int32_t gr_batch_profile(gr_batch* b, float* stage_ms3) {
  if (!b || !stage_ms3) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  gr_context* c = b->ctx;
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  const int nv = (int)b->views.size();
  for (int attempt = 0; attempt < 4; ++attempt) {
    Prepared pr;
    int32_t st = prepare(c, b->vin.data(), nv, b->items.data(), (int)b->items.size(), true, pr);
    if (st) return st;
    void* ev[4] = {c->events[60], c->events[61], c->events[62], c->events[63]};
    if ((st = launch(c, pr.a, ev))) return st;
    CK(cudaMemcpyAsync(c->h_result, c->d_result, sizeof(DevResult), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    int32_t err;
    const int rerun = check_result(c, *c->h_result, &err);
    if (err) return err;
    if (rerun) continue;
    for (int k = 0; k < 3; ++k) CK(cudaEventElapsedTime(&stage_ms3[k], c->events[60 + k], c->events[61 + k]));
    return GR_OK;
  }
  return fail(GR_ERR_OUT_OF_MEMORY, "batch buffers kept overflowing after resizing");
}

int32_t gr_batch_tuning(gr_batch* b, int32_t* tile_size, int32_t* slice_cost, int32_t* raster_waves,
                        int32_t* bin_capacity, float* tuned_ms) {
  if (!b) return fail(GR_ERR_INVALID_ARGUMENT, "batch is NULL");
  gr_context* c = b->ctx;
  if (tile_size) *tile_size = 1 << c->tile_shift;
  if (slice_cost) *slice_cost = (int32_t)c->slice_cost;
  if (raster_waves) *raster_waves = c->raster_waves;
  if (bin_capacity) *bin_capacity = (int32_t)c->bin_cap;
  if (tuned_ms) *tuned_ms = c->tuned_ms;
  return GR_OK;
}

int32_t gr_batch_destroy(gr_batch* b) {
  if (!b) return GR_OK;
  {
    std::lock_guard<std::mutex> lk(b->ctx->mu);
    cudaSetDevice(b->ctx->device);
    cudaStreamSynchronize(b->ctx->stream);
    batch_drop_graph(b);
    dev_free(b->d_views);
    dev_free(b->d_items);
  }
  delete b;
  return GR_OK;
}

int32_t gr_host_alloc(int64_t bytes, void** out) {
  if (!out || bytes <= 0) return fail(GR_ERR_INVALID_ARGUMENT, "bad argument");
  CK(cudaMallocHost(out, (size_t)bytes));
  return GR_OK;
}

int32_t gr_host_free(void* p) {
  if (p) CK(cudaFreeHost(p));
  return GR_OK;
}

int32_t gr_device_alloc(gr_context* c, int64_t bytes, void** out) {
  if (!c || !out || bytes <= 0) return fail(GR_ERR_INVALID_ARGUMENT, "bad argument");
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  CK(cudaMalloc(out, (size_t)bytes));
  return GR_OK;
}

int32_t gr_device_free(gr_context* c, void* p) {
  if (!c) return fail(GR_ERR_INVALID_ARGUMENT, "NULL context");
  if (!p) return GR_OK;
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  CK(cudaStreamSynchronize(c->stream));
  CK(cudaFree(p));
  return GR_OK;
}

int32_t gr_copy(gr_context* c, void* dst, const void* src, int64_t bytes) {
  if (!c || (bytes > 0 && (!dst || !src)) || bytes < 0) return fail(GR_ERR_INVALID_ARGUMENT, "bad argument");
  if (bytes == 0) return GR_OK;
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  CK(cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyDefault, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return GR_OK;
}

int32_t gr_context_last_transfer_bytes(gr_context* c, int64_t* h2d, int64_t* d2h) {
  if (!c || !h2d || !d2h) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  *h2d = c->h2d_bytes;
  *d2h = c->d2h_bytes;
  return GR_OK;
}

int32_t gr_object_matrices(const gr_object* o, const gr_camera* cam, int32_t width, int32_t height, float fov_y,
                           float* mvp, float* world) {
  if (!o || !cam || !mvp || !world || width <= 0 || height <= 0) return fail(GR_ERR_INVALID_ARGUMENT, "bad argument");
  object_matrices(o->scale, o->rotation, o->translation, cam->position, cam->direction, cam->up, width, height, fov_y,
                  mvp, world);
  return GR_OK;
}

int32_t gr_screen_matrix(int32_t width, int32_t height, float* out16) {
  if (!out16) return fail(GR_ERR_INVALID_ARGUMENT, "out is NULL");
  screen_matrix(width, height, out16);
  return GR_OK;
}

int32_t gr_normalize3(const float* v, float* out) {
  if (!v || !out) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  normalize3(v, out);
  return GR_OK;
}

int32_t gr_box_visibility(const float* mvp, const float* bbox, int32_t* out) {
  if (!mvp || !bbox || !out) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  *out = box_visibility(mvp, bbox);
  return GR_OK;
}

int32_t gr_mesh_face_normals(const float* pos, int32_t nv, const int32_t* vidx, int32_t nf, float* out) {
  if (!pos || !vidx || !out || nv <= 0 || nf < 0) return fail(GR_ERR_INVALID_ARGUMENT, "bad argument");
  for (long i = 0; i < 3L * nf; ++i)
    if (vidx[i] < 0 || vidx[i] >= nv) return fail(GR_ERR_BAD_INDEX, "vertex index out of range");
  face_normals(pos, vidx, nf, out);
  return GR_OK;
}

// ---- Renderer ----

int32_t gr_renderer_create(gr_context* c, int32_t width, int32_t height, gr_renderer** out) {
  if (!c || !out) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  if (width <= 0 || height <= 0) return fail(GR_ERR_INVALID_ARGUMENT, "bad size");
  if (width > kMaxDim || height > kMaxDim) return fail(GR_ERR_UNSUPPORTED, "framebuffer too large");
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  gr_renderer* r = new (std::nothrow) gr_renderer();
  if (!r) return fail(GR_ERR_OUT_OF_MEMORY, "renderer allocation");
  r->ctx = c;
  r->width = width;
  r->height = height;
  r->fov_y = 0.785398185f;  // float32(45 * (math.Pi / 180)), renderer.go:118
  const float l[3] = {-1.0f, 1.0f, 1.0f};
  normalize3(l, r->light);  // renderer.go:265
  size_t px = (size_t)width * height;
  if (cudaMalloc((void**)&r->rgba, px * 4) != cudaSuccess || cudaMalloc((void**)&r->z, px * 4) != cudaSuccess) {
    if (r->rgba) cudaFree(r->rgba);
    delete r;
    return fail(GR_ERR_OUT_OF_MEMORY, "framebuffer allocation");
  }
  *out = r;
  return GR_OK;
}

int32_t gr_renderer_destroy(gr_renderer* r) {
  if (!r) return GR_OK;
  cudaSetDevice(r->ctx->device);
  cudaStreamSynchronize(r->ctx->stream);
  cudaFree(r->rgba);
  cudaFree(r->z);
  delete r;
  return GR_OK;
}

int32_t gr_renderer_set_flags(gr_renderer* r, uint32_t flags) {
  if (!r) return fail(GR_ERR_INVALID_ARGUMENT, "renderer is NULL");
  r->flags = flags;
  return GR_OK;
}

int32_t gr_renderer_get_flags(gr_renderer* r, uint32_t* flags) {
  if (!r || !flags) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  *flags = r->flags;
  return GR_OK;
}

int32_t gr_renderer_set_fov(gr_renderer* r, float fov_y) {
  if (!r) return fail(GR_ERR_INVALID_ARGUMENT, "renderer is NULL");
  r->fov_y = fov_y;
  return GR_OK;
}

int32_t gr_renderer_set_light(gr_renderer* r, const float* d) {
  if (!r || !d) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  std::memcpy(r->light, d, sizeof(r->light));
  return GR_OK;
}

int32_t gr_renderer_draw(gr_renderer* r, const gr_object* objs, int32_t n, const gr_camera* cam) {
  if (!r || !cam || n < 0 || (n > 0 && !objs)) return fail(GR_ERR_INVALID_ARGUMENT, "bad argument");
  std::vector<gr_draw_item> items((size_t)n);
  for (int i = 0; i < n; ++i) {
    items[i].mesh = objs[i].mesh;
    items[i].reserved = 0;
    object_matrices(objs[i].scale, objs[i].rotation, objs[i].translation, cam->position, cam->direction, cam->up,
                    r->width, r->height, r->fov_y, items[i].mvp, items[i].world);
  }
  gr_frame_params p;
  std::memset(&p, 0, sizeof(p));
  p.width = r->width;
  p.height = r->height;
  p.flags = r->flags;
  screen_matrix(r->width, r->height, p.screen);
  std::memcpy(p.light, r->light, sizeof(p.light));
  return gr_draw(r->ctx, items.data(), n, &p, (uint8_t*)r->rgba, r->z, &r->tpf);
}

int32_t gr_renderer_read(gr_renderer* r, uint8_t* rgba_out, float* z_out) {
  if (!r) return fail(GR_ERR_INVALID_ARGUMENT, "renderer is NULL");
  gr_context* c = r->ctx;
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  size_t bytes = (size_t)r->width * r->height * 4;
  if (rgba_out) CK(cudaMemcpyAsync(rgba_out, r->rgba, bytes, cudaMemcpyDefault, c->stream));
  if (z_out) CK(cudaMemcpyAsync(z_out, r->z, bytes, cudaMemcpyDefault, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return GR_OK;
}

int32_t gr_renderer_tpf(gr_renderer* r, int64_t* tpf) {
  if (!r || !tpf) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  *tpf = r->tpf;
  return GR_OK;
}

int32_t gr_renderer_fog(gr_renderer* r, float fog_start, float fog_end, const uint8_t* color4) {
  if (!r || !color4) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  return gr_fog(r->ctx, (uint8_t*)r->rgba, r->z, r->width, r->height, fog_start, fog_end, color4);
}

// ---- timing helpers ----

int32_t gr_context_event_record(gr_context* c, int32_t slot) {
  if (!c || slot < 0 || slot >= 64) return fail(GR_ERR_INVALID_ARGUMENT, "bad event slot");
  CK(cudaEventRecord(c->events[slot], c->stream));
  return GR_OK;
}

int32_t gr_context_event_elapsed(gr_context* c, int32_t a, int32_t b, float* ms) {
  if (!c || !ms || a < 0 || a >= 64 || b < 0 || b >= 64) return fail(GR_ERR_INVALID_ARGUMENT, "bad event slot");
  CK(cudaEventSynchronize(c->events[b]));
  CK(cudaEventElapsedTime(ms, c->events[a], c->events[b]));
  return GR_OK;
}

int32_t gr_context_flush_l2(gr_context* c, int64_t bytes) {
  if (!c || bytes <= 0) return fail(GR_ERR_INVALID_ARGUMENT, "bad argument");
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  if ((size_t)bytes > c->flush_bytes) {
    CK(cudaStreamSynchronize(c->stream));
    if (c->flush_buf) cudaFree(c->flush_buf);
    c->flush_buf = nullptr;
    c->flush_bytes = 0;
    CK(cudaMalloc(&c->flush_buf, (size_t)bytes));
    c->flush_bytes = (size_t)bytes;
  }
  CK(cudaMemsetAsync(c->flush_buf, c->last_launches & 0xFF, (size_t)bytes, c->stream));
  return GR_OK;
}

int32_t gr_context_set_tuning(gr_context* c, int32_t tile_size, int32_t bin_capacity) {
  if (!c) return fail(GR_ERR_INVALID_ARGUMENT, "ctx is NULL");
  if (tile_size != 0 && tile_size != 16 && tile_size != 32)
    return fail(GR_ERR_INVALID_ARGUMENT, "tile size must be 16 or 32 (0 keeps it)");
  if (bin_capacity < 0) return fail(GR_ERR_INVALID_ARGUMENT, "negative bin capacity");
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  if (tile_size) c->tile_shift = tile_size == 16 ? 4 : 5;
  if (bin_capacity) {
    // takes effect at the next draw; the buffers are re-sized to exactly this
    CK(cudaStreamSynchronize(c->stream));
    dev_free(c->bins);
    dev_free(c->bin_count);
    c->tiles_cap = 0;
    c->bin_cap = 0;
    c->want_bin_cap = (uint32_t)bin_capacity;
  }
  return GR_OK;
}

int32_t gr_context_set_raster(gr_context* c, int32_t slice_cost, int32_t raster_waves) {
  if (!c) return fail(GR_ERR_INVALID_ARGUMENT, "ctx is NULL");
  if (slice_cost < 0 || raster_waves < 0 || raster_waves > 16)
    return fail(GR_ERR_INVALID_ARGUMENT, "bad raster tuning");
  std::lock_guard<std::mutex> lk(c->mu);
  if (slice_cost) c->slice_cost = (uint32_t)slice_cost;
  if (raster_waves) c->raster_waves = raster_waves;
  return GR_OK;
}

int32_t gr_context_get_raster(gr_context* c, int32_t* slice_cost, int32_t* raster_waves) {
  if (!c || !slice_cost || !raster_waves) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  *slice_cost = (int32_t)c->slice_cost;
  *raster_waves = c->raster_waves;
  return GR_OK;
}

int32_t gr_context_autotune(gr_context* c, const gr_draw_item* items, int32_t n, const gr_frame_params* p) {
  if (!c || !p) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  int32_t st;
  const size_t px = (size_t)p->width * (size_t)p->height;
  if (p->width <= 0 || p->height <= 0) return fail(GR_ERR_INVALID_ARGUMENT, "bad framebuffer size");
  if ((st = ensure_fb(c, px))) return st;
  gr_batch b;
  b.ctx = c;
  gr_view v;
  v.params = *p;
  v.rgba_dev = (uint8_t*)c->fb_rgba;
  v.z_dev = c->fb_z;
  b.views.push_back(v);
  b.vin.push_back(ViewIn{&b.views[0].params, c->fb_rgba, c->fb_z});
  if (n > 0) b.items.assign(items, items + n);
  for (auto& it : b.items) it.reserved = 0;
  return batch_autotune(&b);
}

int32_t gr_context_get_tuning(gr_context* c, int32_t* tile_size, int32_t* bin_capacity) {
  if (!c || !tile_size || !bin_capacity) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  *tile_size = 1 << c->tile_shift;
  *bin_capacity = (int32_t)c->bin_cap;
  return GR_OK;
}

int32_t gr_context_last_launches(gr_context* c, int32_t* launches) {
  if (!c || !launches) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  *launches = c->last_launches;
  return GR_OK;
}


}  // extern "C"

// ---------------------------------------------------------------------------
// Differentiable forward/backward (an extension; see the header)
// ---------------------------------------------------------------------------
struct gr_diff {
  gr_context* ctx = nullptr;
  int mesh = -1;
  int nv = 0, nf = 0, nn = 0;
  int tw = 0, th = 0;
  std::vector<gr_frame_params> params;  // per view: visibility flags + screen matrix
  std::vector<ViewIn> vin;
  std::vector<gr_draw_item> items;      // one item per view
  std::vector<DiffView> hviews;
  uint64_t pixels = 0;
  int max_pixels = 0;
  DiffView* d_views = nullptr;
  DevView* d_frame_views = nullptr;     // the visibility pass's own tables
  DevItem* d_items = nullptr;
  uint32_t* ids = nullptr;              // per pixel: visible face
  float* z = nullptr;                   // per pixel: zRec of the visible face
  DiffRecord* rec = nullptr;
  float* vh = nullptr;                  // views x vertices x 6 (three float-float pairs)
  float4* col_tab = nullptr;
  float4* row_tab = nullptr;
  uint32_t cols = 0, rows = 0;
  int max_side = 0;
  float* nhat = nullptr;
  float* d_world = nullptr;
  float* bbox_partial = nullptr;        // kBBoxBlocks x 6
  unsigned* bbox_done = nullptr;
  double* d_partials = nullptr;         // per-warp sums (kDiffSlots x 4), zero when idle
  float* d_gface = nullptr;             // per-face corner gradient sums (nf x 3 x 8), zero when idle
  double* h_acc = nullptr;              // pinned: loss, light gradient x 3
  double* h_acc_dev = nullptr;          // its device address (k_diff_sum writes the sums there)
  gr_diff_params last{};                // parameters of the last forward
  const float* last_target = nullptr;
  bool have_forward = false;
};

namespace {

DiffArgs diff_args(const gr_diff* d, const gr_diff_params& p, const float* target) {
  DiffArgs a;
  std::memset(&a, 0, sizeof(a));
  const MeshRec& mr = d->ctx->meshes[d->mesh];
  a.views = d->d_views;
  a.num_views = (int)d->hviews.size();
  a.max_pixels = d->max_pixels;
  a.nv = d->nv; a.nf = d->nf; a.nn = d->nn;
  a.pos = p.positions;
  a.vcol = p.vertex_colors;
  a.tex = p.texture;
  a.tw = d->tw; a.th = d->th;
  for (int k = 0; k < 3; ++k) a.L[k] = p.light[k];
  a.vidx = mr.vidx;
  a.nidx = mr.nidx;
  a.uv = mr.uv;
  a.nhat = d->nhat;
  a.vh = d->vh;
  a.col_tab = d->col_tab;
  a.row_tab = d->row_tab;
  a.ids = d->ids;
  a.rec = d->rec;
  a.target = target;
  a.loss = d->h_acc_dev;
  a.g_light = d->h_acc_dev + 1;
  a.partials = d->d_partials;
  a.g_face = d->d_gface;
  return a;
}

void diff_free(gr_diff* d) {
  dev_free(d->d_views); dev_free(d->d_frame_views); dev_free(d->d_items);
  dev_free(d->ids); dev_free(d->z); dev_free(d->rec); dev_free(d->nhat); dev_free(d->d_world);
  dev_free(d->vh); dev_free(d->col_tab); dev_free(d->row_tab);
  dev_free(d->bbox_partial); dev_free(d->bbox_done);
  dev_free(d->d_partials);
  dev_free(d->d_gface);
  if (d->h_acc) cudaFreeHost(d->h_acc);
  d->h_acc = nullptr;
}

// Autotunes the raster for the visibility pass of the views (with the mesh's
// own positions), as gr_batch does for a batch.
int32_t diff_tune_visibility(gr_diff* d) {
  gr_context* c = d->ctx;
  const MeshRec& mr = c->meshes[d->mesh];
  const int nviews = (int)d->params.size();
  auto run = [&](float* ms) -> int32_t {
    for (int attempt = 0; attempt < 5; ++attempt) {
      Prepared pr;
      int32_t st = prepare(c, d->vin.data(), nviews, d->items.data(), nviews, true, pr, d->d_frame_views,
                           d->d_items);
      if (st) return st;
      int e = launch_diff_bbox(mr.pos, d->nv, d->d_items, nviews, d->bbox_partial, d->bbox_done, c->stream);
      if (e) return fail(GR_ERR_CUDA, "diff bbox: %s", cudaGetErrorString((cudaError_t)e));
      if (ms && (st = cold_l2(c, attempt))) return st;
      CK(cudaEventRecord(c->events[58], c->stream));
      if ((st = launch(c, pr.a))) return st;
      CK(cudaEventRecord(c->events[59], c->stream));
      CK(cudaMemcpyAsync(c->h_result, c->d_result, sizeof(DevResult), cudaMemcpyDeviceToHost, c->stream));
      CK(cudaStreamSynchronize(c->stream));
      int32_t err;
      const int rerun = check_result(c, *c->h_result, &err);
      if (err) return err;
      if (rerun) continue;
      if (ms) CK(cudaEventElapsedTime(ms, c->events[58], c->events[59]));
      return GR_OK;
    }
    return fail(GR_ERR_OUT_OF_MEMORY, "frame buffers kept overflowing after resizing");
  };
  return autotune_with(c, run);
}

}  // namespace

extern "C" {

int32_t gr_diff_create(gr_context* c, int32_t mesh, const float* world, int32_t texture_width,
                       int32_t texture_height, const gr_diff_view* views, int32_t num_views, gr_diff** out) {
  if (!c || !world || !views || !out || num_views <= 0) return fail(GR_ERR_INVALID_ARGUMENT, "bad argument");
  *out = nullptr;
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  if (mesh < 0 || mesh >= (int)c->meshes.size() || !c->meshes[mesh].alive)
    return fail(GR_ERR_INVALID_ARGUMENT, "unknown mesh %d", mesh);
  const MeshRec& mr = c->meshes[mesh];
  if (mr.nn <= 0 || !mr.has_nidx || !mr.nidx_ok)
    return fail(GR_ERR_INVALID_ARGUMENT, "the differentiable mesh needs vertex normals with valid normal indices");
  if (mr.nf <= 0 || mr.nv <= 0) return fail(GR_ERR_INVALID_ARGUMENT, "empty mesh");
  if (texture_width < 0 || texture_height < 0 || (texture_width == 0) != (texture_height == 0))
    return fail(GR_ERR_INVALID_ARGUMENT, "bad texture size %dx%d", texture_width, texture_height);
  if ((uint64_t)mr.nf * (uint64_t)num_views >= (1ull << 28))
    return fail(GR_ERR_UNSUPPORTED, "more than 2^28 faces over all views");
  gr_diff* d = new (std::nothrow) gr_diff();
  if (!d) return fail(GR_ERR_OUT_OF_MEMORY, "diff allocation");
  d->ctx = c;
  d->mesh = mesh;
  d->nv = mr.nv; d->nf = mr.nf; d->nn = mr.nn;
  d->tw = texture_width; d->th = texture_height;
  d->params.resize(num_views);
  d->items.resize(num_views);
  d->hviews.resize(num_views);
  uint64_t pix = 0;
  int32_t st = GR_OK;
  for (int v = 0; v < num_views && !st; ++v) {
    const gr_diff_view& dv = views[v];
    if (dv.width <= 0 || dv.height <= 0 || dv.width > kMaxDim || dv.height > kMaxDim) {
      st = fail(GR_ERR_INVALID_ARGUMENT, "view %d: bad size %dx%d", v, dv.width, dv.height);
      break;
    }
    gr_frame_params& p = d->params[v];
    std::memset(&p, 0, sizeof(p));
    p.width = dv.width;
    p.height = dv.height;
    p.flags = (dv.flags & (GR_FRUSTUM_CLIPPING | GR_BACKFACE_CULLING)) | GR_SHOW_FACES | kViewFaceIds;
    std::memcpy(p.screen, dv.screen, sizeof(p.screen));
    gr_draw_item& it = d->items[v];
    it.mesh = mesh;
    it.reserved = v;
    std::memcpy(it.mvp, dv.mvp, sizeof(it.mvp));
    std::memcpy(it.world, world, sizeof(it.world));
    DiffView& hv = d->hviews[v];
    hv.W = dv.width;
    hv.H = dv.height;
    hv.pix_base = (uint32_t)pix;
    hv.face_base = (uint32_t)((uint64_t)v * (uint64_t)mr.nf);
    hv.col_base = d->cols;
    hv.row_base = d->rows;
    d->cols += (uint32_t)dv.width;
    d->rows += (uint32_t)dv.height;
    d->max_side = std::max(d->max_side, std::max(dv.width, dv.height));
    // Q = rows 0 and 1 of S * MVP (homogeneous screen x and y) and row 3 of
    // MVP (clip W), in double: products of two floats are exact there
    for (int j = 0; j < 4; ++j) {
      double q0 = 0.0, q1 = 0.0;
      for (int i = 0; i < 4; ++i) {
        q0 += (double)dv.screen[i] * (double)dv.mvp[4 * i + j];
        q1 += (double)dv.screen[4 + i] * (double)dv.mvp[4 * i + j];
      }
      hv.Q[j] = q0;
      hv.Q[4 + j] = q1;
      hv.Q[8 + j] = (double)dv.mvp[12 + j];
    }
    for (int j = 0; j < 12; ++j) {  // the same as float pairs for the float-float kernels
      const float hi = (float)hv.Q[j];
      hv.Qf[2 * j] = hi;
      hv.Qf[2 * j + 1] = (float)(hv.Q[j] - (double)hi);
    }
    pix += (uint64_t)dv.width * (uint64_t)dv.height;
    d->max_pixels = std::max(d->max_pixels, dv.width * dv.height);
    if (pix >= (1ull << 32)) st = fail(GR_ERR_UNSUPPORTED, "more than 2^32 pixels over all views");
  }
  d->pixels = pix;
  if (!st) st = dev_alloc(&d->d_views, (size_t)num_views);
  if (!st) st = dev_alloc(&d->d_frame_views, (size_t)num_views);
  if (!st) st = dev_alloc(&d->d_items, (size_t)num_views);
  if (!st) st = dev_alloc(&d->ids, (size_t)pix);
  if (!st) st = dev_alloc(&d->z, (size_t)pix);
  if (!st) st = dev_alloc(&d->rec, (size_t)pix);
  if (!st) st = dev_alloc(&d->nhat, (size_t)mr.nn * 4);
  if (!st) st = dev_alloc(&d->vh, (size_t)num_views * (size_t)mr.nv * 6);
  if (!st) st = dev_alloc(&d->col_tab, (size_t)d->cols);
  if (!st) st = dev_alloc(&d->row_tab, (size_t)d->rows);
  if (!st) st = dev_alloc(&d->d_world, (size_t)16);
  if (!st) st = dev_alloc(&d->bbox_partial, (size_t)kBBoxBlocks * 6);
  if (!st) st = dev_alloc(&d->bbox_done, (size_t)1);
  if (!st && cudaMemsetAsync(d->bbox_done, 0, sizeof(unsigned), c->stream) != cudaSuccess)
    st = fail(GR_ERR_CUDA, "diff counters");
  if (!st) st = dev_alloc(&d->d_partials, (size_t)kDiffSlots * 4);
  if (!st && cudaMemsetAsync(d->d_partials, 0, sizeof(double) * kDiffSlots * 4, c->stream) != cudaSuccess)
    st = fail(GR_ERR_CUDA, "diff partials");
  if (!st) st = dev_alloc(&d->d_gface, (size_t)d->nf * 24);
  if (!st && cudaMemsetAsync(d->d_gface, 0, sizeof(float) * 24 * (size_t)d->nf, c->stream) != cudaSuccess)
    st = fail(GR_ERR_CUDA, "diff face sums");
  if (!st && cudaMallocHost((void**)&d->h_acc, 4 * sizeof(double)) != cudaSuccess) {
    d->h_acc = nullptr;
    st = fail(GR_ERR_OUT_OF_MEMORY, "pinned accumulator");
  }
  if (!st && cudaHostGetDevicePointer((void**)&d->h_acc_dev, d->h_acc, 0) != cudaSuccess)
    st = fail(GR_ERR_CUDA, "pinned accumulator address");
  if (!st) {
    d->vin.resize(num_views);
    for (int v = 0; v < num_views; ++v)
      d->vin[v] = ViewIn{&d->params[v], d->ids + d->hviews[v].pix_base, d->z + d->hviews[v].pix_base, true};
    cudaError_t e = cudaMemcpyAsync(d->d_views, d->hviews.data(), sizeof(DiffView) * num_views,
                                    cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d->d_world, world, 16 * sizeof(float), cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) st = fail(GR_ERR_CUDA, "diff tables: %s", cudaGetErrorString(e));
  }
  if (!st) {
    int e = launch_diff_normals(d->d_world, mr.vnrm, mr.nn, d->nhat, c->stream);
    if (!e) e = (int)cudaStreamSynchronize(c->stream);
    if (e) st = fail(GR_ERR_CUDA, "diff normals: %s", cudaGetErrorString((cudaError_t)e));
  }
  // the visibility pass's raster tuning (the context's default slice cost
  // left a 64-view forward 12 % slower than the best)
  if (!st) st = diff_tune_visibility(d);
  if (st) {
    cudaStreamSynchronize(c->stream);
    diff_free(d);
    delete d;
    return st;
  }
  *out = d;
  return GR_OK;
}

int32_t gr_diff_forward(gr_diff* d, const gr_diff_params* p, const float* target_dev, float* image_dev,
                        double* loss) {
  if (!d || !p || !target_dev) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  if (!p->positions || !p->vertex_colors) return fail(GR_ERR_INVALID_ARGUMENT, "positions and colours are required");
  if (!is_device_ptr(p->positions) || !is_device_ptr(p->vertex_colors) || !is_device_ptr(target_dev) ||
      (p->texture && !is_device_ptr(p->texture)) || (image_dev && !is_device_ptr(image_dev)))
    return fail(GR_ERR_INVALID_ARGUMENT, "parameters, target and image must be device pointers");
  if ((uintptr_t)p->positions % 16 || (uintptr_t)target_dev % 16 || (p->texture && (uintptr_t)p->texture % 16) ||
      (image_dev && (uintptr_t)image_dev % 16))
    return fail(GR_ERR_INVALID_ARGUMENT, "positions, texture, target and image need 16-byte alignment");
  if (p->texture && d->tw == 0) return fail(GR_ERR_INVALID_ARGUMENT, "created without a texture size");
  gr_context* c = d->ctx;
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  MeshRec& mr = c->meshes[d->mesh];
  if (!mr.alive) return fail(GR_ERR_INVALID_ARGUMENT, "the mesh was destroyed");
  const int nviews = (int)d->params.size();
  DiffArgs a = diff_args(d, *p, target_dev);
  a.image = image_dev;
  for (int attempt = 0; attempt < 5; ++attempt) {
    // visibility with the parameter positions: the item tables take the
    // mesh's pointers, so the mesh briefly points at them
    float* keep = mr.pos;
    mr.pos = const_cast<float*>(p->positions);
    Prepared pr;
    int32_t st = prepare(c, d->vin.data(), nviews, d->items.data(), nviews, true, pr, d->d_frame_views,
                         d->d_items);
    mr.pos = keep;
    if (st) return st;
    int e = launch_diff_bbox(p->positions, d->nv, d->d_items, nviews, d->bbox_partial, d->bbox_done, c->stream);
    if (e) return fail(GR_ERR_CUDA, "diff bbox: %s", cudaGetErrorString((cudaError_t)e));
    // the visibility pass's counters and the loss reach page-locked host
    // memory from the kernels themselves: no copy between or after them
    pr.a.result_host = c->h_result_dev;
    if ((st = launch(c, pr.a))) return st;
    e = launch_diff_forward(a, d->max_side, c->stream);
    if (e) return fail(GR_ERR_CUDA, "diff forward: %s", cudaGetErrorString((cudaError_t)e));
    CK(cudaStreamSynchronize(c->stream));
    int32_t err;
    const int rerun = check_result(c, *c->h_result, &err);
    if (err) return err;
    if (rerun) continue;
    d->last = *p;
    d->last_target = target_dev;
    d->have_forward = true;
    if (loss) *loss = d->h_acc[0];
    return GR_OK;
  }
  return fail(GR_ERR_OUT_OF_MEMORY, "frame buffers kept overflowing after resizing");
}

int32_t gr_diff_backward(gr_diff* d, gr_diff_grads* g) {
  if (!d || !g) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  if (!d->have_forward) return fail(GR_ERR_INVALID_ARGUMENT, "gr_diff_backward before gr_diff_forward");
  if (!g->positions || !g->vertex_colors || !is_device_ptr(g->positions) || !is_device_ptr(g->vertex_colors) ||
      (g->texture && !is_device_ptr(g->texture)))
    return fail(GR_ERR_INVALID_ARGUMENT, "gradient buffers must be device pointers");
  if (d->last.texture && !g->texture) return fail(GR_ERR_INVALID_ARGUMENT, "texture gradient buffer is NULL");
  if (g->texture && ((uintptr_t)g->texture & 15u))
    return fail(GR_ERR_INVALID_ARGUMENT, "texture gradient buffer must be 16-byte aligned");
  gr_context* c = d->ctx;
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  DiffArgs a = diff_args(d, d->last, d->last_target);
  a.g_pos = g->positions;
  a.g_vcol = g->vertex_colors;
  a.g_tex = d->last.texture ? g->texture : nullptr;
  CK(cudaMemsetAsync(g->positions, 0, sizeof(float) * 4 * (size_t)d->nv, c->stream));
  CK(cudaMemsetAsync(g->vertex_colors, 0, sizeof(float) * 3 * (size_t)d->nv, c->stream));
  if (a.g_tex) CK(cudaMemsetAsync(a.g_tex, 0, sizeof(float) * 4 * (size_t)d->tw * (size_t)d->th, c->stream));
  int e = launch_diff_backward(a, c->stream);
  if (e) return fail(GR_ERR_CUDA, "diff backward: %s", cudaGetErrorString((cudaError_t)e));
  CK(cudaStreamSynchronize(c->stream));
  for (int k = 0; k < 3; ++k) g->light[k] = d->h_acc[1 + k];
  return GR_OK;
}

int32_t gr_diff_buffers(gr_diff* d, const uint32_t** face_ids, const void** records, int64_t* pixels) {
  if (!d) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  if (face_ids) *face_ids = d->ids;
  if (records) *records = d->rec;
  if (pixels) *pixels = (int64_t)d->pixels;
  return GR_OK;
}

int32_t gr_diff_destroy(gr_diff* d) {
  if (!d) return GR_OK;
  {
    std::lock_guard<std::mutex> lk(d->ctx->mu);
    cudaSetDevice(d->ctx->device);
    cudaStreamSynchronize(d->ctx->stream);
    diff_free(d);
  }
  delete d;
  return GR_OK;
}


int32_t gr_fog(gr_context* c, uint8_t* rgba_dev, const float* z_dev, int32_t width, int32_t height,
               float fog_start, float fog_end, const uint8_t* color4) {
  if (!c || !rgba_dev || !z_dev || !color4) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  if (width <= 0 || height <= 0) return fail(GR_ERR_INVALID_ARGUMENT, "bad framebuffer size");
  if (!is_device_ptr(rgba_dev) || !is_device_ptr(z_dev))
    return fail(GR_ERR_INVALID_ARGUMENT, "gr_fog needs device buffers");
  if ((uintptr_t)rgba_dev % 4) return fail(GR_ERR_INVALID_ARGUMENT, "rgba needs 4-byte alignment");
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  uint32_t col;
  std::memcpy(&col, color4, 4);
  const int e = launch_fog((uint32_t*)rgba_dev, z_dev, (long long)width * height, fog_start, fog_end, col, c->stream);
  if (e) return fail(GR_ERR_CUDA, "fog: %s", cudaGetErrorString((cudaError_t)e));
  CK(cudaStreamSynchronize(c->stream));
  return GR_OK;
}

int32_t gr_context_set_fog(gr_context* c, int32_t enable, float fog_start, float fog_end, const uint8_t* color4) {
  if (!c || (enable && !color4)) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  std::lock_guard<std::mutex> lk(c->mu);
  c->fog_on = enable != 0;
  c->fog_start = fog_start;
  c->fog_end = fog_end;
  if (enable) std::memcpy(&c->fog_color, color4, 4);
  return GR_OK;
}


}  // extern "C"

// ---------------------------------------------------------------------------
// Headless present: two device framebuffers, copies on a second stream
// ---------------------------------------------------------------------------
struct gr_presenter {
  gr_renderer* r = nullptr;
  cudaStream_t copy = nullptr;
  uint32_t* dev[2] = {nullptr, nullptr};
  uint8_t* host[2] = {nullptr, nullptr};      // pinned
  DevResult* res[2] = {nullptr, nullptr};     // pinned: each frame's counters (and the raster's done word)
  DevResult* res_dev[2] = {nullptr, nullptr}; // their device addresses: the last raster CTA writes there
  cudaEvent_t rendered[2] = {}, copied[2] = {};
  std::vector<gr_draw_item> items[2];
  bool queued[2] = {false, false};            // rendered + copy queued, not yet returned
  int64_t frame = 0;
};

namespace {

void presenter_free(gr_presenter* p) {
  for (int b = 0; b < 2; ++b) {
    dev_free(p->dev[b]);
    if (p->host[b]) cudaFreeHost(p->host[b]);
    if (p->res[b]) cudaFreeHost(p->res[b]);
    if (p->rendered[b]) cudaEventDestroy(p->rendered[b]);
    if (p->copied[b]) cudaEventDestroy(p->copied[b]);
  }
  if (p->copy) cudaStreamDestroy(p->copy);
}

// Queues frame buffer b: render on the context stream (after the copy that
// last read buffer b), its counters, then the copy to host on the copy stream.
int32_t presenter_enqueue(gr_presenter* p, int b) {
  gr_renderer* r = p->r;
  gr_context* c = r->ctx;
  gr_frame_params fp;
  std::memset(&fp, 0, sizeof(fp));
  fp.width = r->width;
  fp.height = r->height;
  fp.flags = r->flags;
  screen_matrix(r->width, r->height, fp.screen);
  std::memcpy(fp.light, r->light, sizeof(fp.light));
  CK(cudaStreamWaitEvent(c->stream, p->copied[b], 0));
  ViewIn v{&fp, p->dev[b], r->z};
  Prepared pr;
  int32_t st = prepare(c, &v, 1, p->items[b].data(), (int32_t)p->items[b].size(), false, pr, nullptr, nullptr,
                       Upload::kRingInGraph);
  if (st) return st;
  pr.a.result_host = p->res_dev[b];  // the counters without a copy on the render stream
  if ((st = launch(c, pr.a, nullptr, pr.copy_src, pr.copy_bytes)) || (st = record_ring_slot(c, pr))) return st;
  CK(cudaEventRecord(p->rendered[b], c->stream));
  CK(cudaStreamWaitEvent(p->copy, p->rendered[b], 0));
  CK(cudaMemcpyAsync(p->host[b], p->dev[b], (size_t)r->width * r->height * 4, cudaMemcpyDeviceToHost, p->copy));
  CK(cudaEventRecord(p->copied[b], p->copy));
  p->queued[b] = true;
  return GR_OK;
}

// Waits for buffer b's copy; renders it again while its buffers overflowed.
int32_t presenter_collect(gr_presenter* p, int b, const uint8_t** rgba, int64_t* tpf) {
  gr_context* c = p->r->ctx;
  for (int attempt = 0; attempt < 5; ++attempt) {
    CK(cudaEventSynchronize(p->copied[b]));
    int32_t err;
    const int rerun = check_result(c, *p->res[b], &err);
    if (err) return err;
    if (!rerun) {
      p->queued[b] = false;
      if (rgba) *rgba = p->host[b];
      if (tpf) *tpf = (int64_t)p->res[b]->tpf;
      return GR_OK;
    }
    int32_t st = presenter_enqueue(p, b);  // the buffers grow in prepare()
    if (st) return st;
  }
  return fail(GR_ERR_OUT_OF_MEMORY, "frame buffers kept overflowing after resizing");
}

}  // namespace

extern "C" {

int32_t gr_presenter_create(gr_renderer* r, gr_presenter** out) {
  if (!r || !out) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  *out = nullptr;
  gr_context* c = r->ctx;
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  gr_presenter* p = new (std::nothrow) gr_presenter();
  if (!p) return fail(GR_ERR_OUT_OF_MEMORY, "presenter allocation");
  p->r = r;
  const size_t px = (size_t)r->width * r->height;
  cudaError_t e = cudaStreamCreateWithFlags(&p->copy, cudaStreamNonBlocking);
  int32_t st = e == cudaSuccess ? GR_OK : fail(GR_ERR_CUDA, "copy stream: %s", cudaGetErrorString(e));
  for (int b = 0; b < 2 && !st; ++b) {
    if ((st = dev_alloc(&p->dev[b], px))) break;
    e = cudaMallocHost((void**)&p->host[b], px * 4);
    if (e == cudaSuccess) e = cudaMallocHost((void**)&p->res[b], 2 * sizeof(DevResult));
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void**)&p->res_dev[b], p->res[b], 0);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->rendered[b], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->copied[b], cudaEventDisableTiming);
    if (e != cudaSuccess) st = fail(GR_ERR_CUDA, "presenter buffers: %s", cudaGetErrorString(e));
  }
  if (st) {
    presenter_free(p);
    delete p;
    return st;
  }
  *out = p;
  return GR_OK;
}

int32_t gr_presenter_frame(gr_presenter* p, const gr_object* objs, int32_t n, const gr_camera* cam,
                           const uint8_t** prev_rgba, int64_t* prev_tpf) {
  if (!p || !cam || n < 0 || (n > 0 && !objs)) return fail(GR_ERR_INVALID_ARGUMENT, "bad argument");
  gr_renderer* r = p->r;
  gr_context* c = r->ctx;
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  const int b = (int)(p->frame & 1), prev = b ^ 1;
  if (p->queued[b]) {  // never returned (a flush was skipped): collect it first
    int32_t st = presenter_collect(p, b, nullptr, nullptr);
    if (st) return st;
  }
  std::vector<gr_draw_item>& items = p->items[b];
  items.assign((size_t)n, gr_draw_item{});
  for (int i = 0; i < n; ++i) {
    items[i].mesh = objs[i].mesh;
    object_matrices(objs[i].scale, objs[i].rotation, objs[i].translation, cam->position, cam->direction, cam->up,
                    r->width, r->height, r->fov_y, items[i].mvp, items[i].world);
  }
  int32_t st = presenter_enqueue(p, b);
  if (st) return st;
  p->frame += 1;
  if (prev_rgba) *prev_rgba = nullptr;
  if (prev_tpf) *prev_tpf = -1;
  if (!p->queued[prev]) return GR_OK;
  return presenter_collect(p, prev, prev_rgba, prev_tpf);
}

int32_t gr_presenter_flush(gr_presenter* p, const uint8_t** rgba, int64_t* tpf) {
  if (!p) return fail(GR_ERR_INVALID_ARGUMENT, "presenter is NULL");
  gr_context* c = p->r->ctx;
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  if (rgba) *rgba = nullptr;
  if (tpf) *tpf = -1;
  const int last = (int)((p->frame + 1) & 1);  // the most recently queued buffer
  if (!p->queued[last]) return GR_OK;
  return presenter_collect(p, last, rgba, tpf);
}

int32_t gr_presenter_destroy(gr_presenter* p) {
  if (!p) return GR_OK;
  {
    std::lock_guard<std::mutex> lk(p->r->ctx->mu);
    cudaSetDevice(p->r->ctx->device);
    cudaStreamSynchronize(p->r->ctx->stream);
    if (p->copy) cudaStreamSynchronize(p->copy);
    presenter_free(p);
  }
  delete p;
  return GR_OK;
}
}  // extern "C"
