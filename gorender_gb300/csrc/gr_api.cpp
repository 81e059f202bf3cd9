// gr_api.cpp -- C-ABI of libgorender_cuda.so: contexts, resident meshes and
// textures, frame buffers sized for the frame, the draw entry points and the
// host Renderer (NewRenderer / Draw) built on them.
#include <cuda_runtime.h>

#include <algorithm>
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

struct gr_context {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::mutex mu;
  std::vector<MeshRec> meshes;
  std::vector<TexRec> texs;
  DevTex* d_texs = nullptr;
  int d_texs_cap = 0;
  bool texs_dirty = true;

  DevItem* d_items = nullptr;
  DevItem* h_items = nullptr;  // pinned staging
  int items_cap = 0;

  TriRaster* rast = nullptr;
  TriShade* shade = nullptr;
  TriWide* wide = nullptr;
  TriColor* tcol = nullptr;
  uint32_t rec_cap = 0;
  uint32_t* rec_of_key = nullptr;
  uint32_t key_cap = 0;
  uint32_t* bins = nullptr;
  uint32_t* bin_count = nullptr;
  uint32_t bin_cap = 0;
  uint32_t tiles_cap = 0;
  uint32_t* big = nullptr;
  uint32_t big_cap = 0;
  unsigned long long* gkey = nullptr;  // merged keys of tiles split over several CTAs
  uint32_t* tile_done = nullptr;
  uint32_t gkey_tiles = 0;
  uint2* clip = nullptr;            // faces for the general clipper
  uint32_t clip_cap = 0;
  float* vlight = nullptr;          // per-normal Gouraud intensities
  uint64_t vlight_cap = 0;
  uint32_t slice_entries = kDefaultSliceEntries;
  DevWork* work = nullptr;
  DevResult* d_result = nullptr;
  DevResult* h_result = nullptr;  // pinned

  uint32_t* fb_rgba = nullptr;
  float* fb_z = nullptr;
  size_t fb_pixels = 0;

  void* flush_buf = nullptr;
  size_t flush_bytes = 0;
  cudaEvent_t events[64] = {};
  int last_launches = 0;
  int32_t pending = GR_OK;
  int64_t h2d_bytes = 0, d2h_bytes = 0;  // host<->device bytes of the last draw
  uint32_t want_bin_cap = 0, want_rec_cap = 0, want_big_cap = 0, want_clip_cap = 0;
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

int32_t ensure_items(gr_context* c, int n) {
  if (n <= c->items_cap) return GR_OK;
  int cap = std::max(n, 2 * c->items_cap);
  CK(cudaStreamSynchronize(c->stream));
  dev_free(c->d_items);
  if (c->h_items) cudaFreeHost(c->h_items);
  c->h_items = nullptr;
  c->items_cap = 0;
  int32_t st = dev_alloc(&c->d_items, cap);
  if (st) return st;
  CK(cudaMallocHost((void**)&c->h_items, sizeof(DevItem) * cap));
  c->items_cap = cap;
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
    dev_free(c->rast); dev_free(c->shade); dev_free(c->wide); dev_free(c->tcol);
    c->rec_cap = 0;
    if ((st = dev_alloc(&c->rast, want_rec)) || (st = dev_alloc(&c->shade, want_rec)) ||
        (st = dev_alloc(&c->wide, want_rec)) || (st = dev_alloc(&c->tcol, want_rec)))
      return st;
    c->rec_cap = (uint32_t)want_rec;
  }
  uint64_t want_key = (uint64_t)kKeysPerFace * faces + kKeysPerFace;
  if (want_key > c->key_cap) {
    if ((st = sync())) return st;
    dev_free(c->rec_of_key);
    c->key_cap = 0;
    if ((st = dev_alloc(&c->rec_of_key, want_key))) return st;
    c->key_cap = (uint32_t)want_key;
  }
  uint32_t want_bin = c->want_bin_cap;
  if (want_bin == 0) want_bin = std::max<uint32_t>(1024, next_pow2(4 * (2 * faces) / std::max<uint32_t>(tiles, 1)));
  if (tiles > c->tiles_cap || want_bin > c->bin_cap) {
    if ((st = sync())) return st;
    uint32_t nt = std::max(tiles, c->tiles_cap);
    uint32_t nc = std::max(want_bin, c->bin_cap);
    dev_free(c->bins); dev_free(c->bin_count);
    c->tiles_cap = 0; c->bin_cap = 0;
    if ((st = dev_alloc(&c->bins, (size_t)nt * nc)) || (st = dev_alloc(&c->bin_count, nt))) return st;
    CK(cudaMemsetAsync(c->bin_count, 0, sizeof(uint32_t) * nt, c->stream));
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
  uint64_t faces;
  int nitems;
};

// Validates the items, stages DevItems and fills the kernel arguments.
int32_t prepare(gr_context* c, const gr_draw_item* items, int32_t n, const gr_frame_params* p, Prepared& out) {
  if (!p) return fail(GR_ERR_INVALID_ARGUMENT, "params is NULL");
  if (n < 0 || (n > 0 && !items)) return fail(GR_ERR_INVALID_ARGUMENT, "bad item list");
  if (p->width <= 0 || p->height <= 0) return fail(GR_ERR_INVALID_ARGUMENT, "bad framebuffer size %dx%d", p->width, p->height);
  if (p->width > kMaxDim || p->height > kMaxDim)
    return fail(GR_ERR_UNSUPPORTED, "framebuffer %dx%d exceeds %d", p->width, p->height, kMaxDim);
  if (p->flags & (GR_SHOW_EDGES | GR_SHOW_VERTICES))
    return fail(GR_ERR_UNSUPPORTED, "edge and vertex overlays are not implemented");
  int32_t st = ensure_items(c, std::max(n, 1));
  if (st) return st;
  if ((st = upload_textures(c))) return st;
  const bool gouraud = (p->flags & GR_LIGHTING) && !(p->flags & GR_FLAT_SHADING);
  uint64_t faces = 0;
  int blocks = 0;
  int light_blocks = 0;
  uint64_t light_total = 0;
  int live = 0;
  for (int i = 0; i < n; ++i) {
    int m = items[i].mesh;
    if (m < 0 || m >= (int)c->meshes.size() || !c->meshes[m].alive)
      return fail(GR_ERR_INVALID_ARGUMENT, "item %d: unknown mesh %d", i, m);
    const MeshRec& mr = c->meshes[m];
    if (gouraud && mr.nn > 0 && !mr.nidx_ok)
      return fail(GR_ERR_BAD_INDEX, "item %d: mesh %d has missing or out-of-range normal indices", i, m);
    uint64_t fb = faces;
    faces += (uint64_t)mr.nf;
    if (mr.nf == 0) continue;  // an empty mesh draws nothing
    DevItem& d = c->h_items[live++];
    std::memcpy(d.mvp, items[i].mvp, sizeof(d.mvp));
    std::memcpy(d.world, items[i].world, sizeof(d.world));
    std::memcpy(d.bbox, mr.bbox, sizeof(d.bbox));
    d.pos = mr.pos; d.vnrm = mr.vnrm; d.fnrm = mr.fnrm; d.vidx = mr.vidx; d.nidx = mr.nidx;
    d.uv = mr.uv; d.tex = mr.tex; d.vcol = mr.vcol;
    d.nv = mr.nv; d.nn = mr.nn; d.nf = mr.nf;
    d.face_base = (uint32_t)fb;
    d.block_base = blocks;
    blocks += (mr.nf + kProjectThreads - 1) / kProjectThreads;
    // every item gets a k_light block range (empty for non-Gouraud items) so the
    // kernel's block -> item search sees non-decreasing bases
    d.light_base = (int)light_total;
    d.light_block_base = light_blocks;
    if (gouraud && mr.nn > 0) {
      light_total += (uint64_t)mr.nn;
      light_blocks += (mr.nn + 255) / 256;
    }
  }
  if (faces >= (1ull << 28)) return fail(GR_ERR_UNSUPPORTED, "more than 2^28 faces in one frame");
  const int ts = 1 << c->tile_shift;
  const int tiles_x = (p->width + ts - 1) / ts;
  const int tiles_y = (p->height + ts - 1) / ts;
  if ((st = ensure_frame_buffers(c, faces, (uint32_t)(tiles_x * tiles_y)))) return st;
  if (light_total > c->vlight_cap) {
    CK(cudaStreamSynchronize(c->stream));
    dev_free(c->vlight);
    c->vlight_cap = 0;
    if ((st = dev_alloc(&c->vlight, light_total))) return st;
    c->vlight_cap = light_total;
  }
  if (live) CK(cudaMemcpyAsync(c->d_items, c->h_items, sizeof(DevItem) * live, cudaMemcpyHostToDevice, c->stream));
  c->h2d_bytes = (int64_t)sizeof(DevItem) * live;
  c->d2h_bytes = 0;

  FrameArgs& a = out.a;
  std::memset(&a, 0, sizeof(a));
  a.W = p->width;
  a.H = p->height;
  a.flags = p->flags;
  a.tiles_x = tiles_x;
  a.tiles_y = tiles_y;
  a.tile_shift = c->tile_shift;
  a.num_items = live;
  a.total_blocks = blocks;
  a.bin_cap = c->bin_cap;
  a.rec_cap = c->rec_cap;
  a.big_cap = c->big_cap;
  a.key_cap = c->key_cap;
  for (int k = 0; k < 8; ++k) a.S[k] = p->screen[k];
  for (int k = 0; k < 3; ++k) a.L[k] = p->light[k];
  a.items = c->d_items;
  a.texs = c->d_texs;
  a.num_tex = (int)c->texs.size();
  a.rast = c->rast;
  a.shade = c->shade;
  a.wide = c->wide;
  a.tcol = c->tcol;
  a.rec_of_key = c->rec_of_key;
  a.bins = c->bins;
  a.bin_count = c->bin_count;
  a.big = c->big;
  a.gkey = c->gkey;
  a.tile_done = c->tile_done;
  a.slice_entries = c->slice_entries;
  a.clip = c->clip;
  a.clip_cap = c->clip_cap;
  a.vlight = c->vlight;
  a.light_blocks = light_blocks;
  a.work = c->work;
  a.result = c->d_result;
  out.faces = faces;
  out.nitems = live;
  return GR_OK;
}

void set_outputs(FrameArgs& a, uint32_t* rgba, float* z) {
  a.out_rgba = rgba;
  a.out_z = z;
  a.vec_ok = (a.W % 4 == 0) && ((uintptr_t)rgba % 16 == 0) && ((uintptr_t)z % 16 == 0);
}

int32_t launch(gr_context* c, const FrameArgs& a, void* const* events = nullptr) {
  int big_blocks = 2 * 152;
  int err = launch_frame(a, big_blocks, c->stream, &c->last_launches, events);
  if (err) return fail(GR_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString((cudaError_t)err));
  return GR_OK;
}

// Reads the frame result; grows buffers that overflowed.  Returns 1 when the
// frame must be re-run.
int check_result(gr_context* c, const DevResult& r, int32_t* err) {
  *err = GR_OK;
  int rerun = 0;
  if (r.bin_need > c->bin_cap) { c->want_bin_cap = next_pow2((uint64_t)r.bin_need + r.bin_need / 4); rerun = 1; }
  if (r.rec_need > c->rec_cap) { c->want_rec_cap = r.rec_need + r.rec_need / 8; rerun = 1; }
  if (r.big_need > c->big_cap) { c->want_big_cap = next_pow2((uint64_t)r.big_need + r.big_need / 4); rerun = 1; }
  if (r.clip_need > c->clip_cap) { c->want_clip_cap = next_pow2((uint64_t)r.clip_need + r.clip_need / 4); rerun = 1; }
  if (r.error & 1u) *err = fail(GR_ERR_CLIP_OVERFLOW, "a clipped polygon exceeded 9 vertices");
  return rerun;
}

int32_t draw_sync(gr_context* c, const gr_draw_item* items, int32_t n, const gr_frame_params* p,
                  uint8_t* rgba_out, float* z_out, int64_t* tpf_out) {
  const size_t px = (size_t)p->width * (size_t)p->height;
  const bool rgba_dev = is_device_ptr(rgba_out), z_dev = is_device_ptr(z_out);
  int32_t st;
  for (int attempt = 0; attempt < 4; ++attempt) {
    Prepared pr;
    if ((st = prepare(c, items, n, p, pr))) return st;
    uint32_t* rgba = rgba_dev ? (uint32_t*)rgba_out : nullptr;
    float* z = z_dev ? z_out : nullptr;
    if (!rgba || !z) {
      if ((st = ensure_fb(c, px))) return st;
      if (!rgba) rgba = c->fb_rgba;
      if (!z) z = c->fb_z;
    }
    set_outputs(pr.a, rgba, z);
    if ((st = launch(c, pr.a))) return st;
    CK(cudaMemcpyAsync(c->h_result, c->d_result, sizeof(DevResult), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    int32_t err;
    int rerun = check_result(c, *c->h_result, &err);
    if (err) return err;
    if (rerun) continue;
    c->d2h_bytes = (int64_t)sizeof(DevResult);
    if (rgba_out && !rgba_dev) {
      CK(cudaMemcpyAsync(rgba_out, rgba, px * 4, cudaMemcpyDeviceToHost, c->stream));
      c->d2h_bytes += (int64_t)px * 4;
    }
    if (z_out && !z_dev) {
      CK(cudaMemcpyAsync(z_out, z, px * 4, cudaMemcpyDeviceToHost, c->stream));
      c->d2h_bytes += (int64_t)px * 4;
    }
    CK(cudaStreamSynchronize(c->stream));
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
  if (e == cudaSuccess) e = cudaMallocHost((void**)&c->h_result, sizeof(DevResult));
  for (int i = 0; i < 64 && e == cudaSuccess; ++i) e = cudaEventCreate(&c->events[i]);
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
  dev_free(c->d_texs); dev_free(c->d_items);
  if (c->h_items) cudaFreeHost(c->h_items);
  dev_free(c->rast); dev_free(c->shade); dev_free(c->wide); dev_free(c->tcol);
  dev_free(c->rec_of_key); dev_free(c->bins); dev_free(c->bin_count); dev_free(c->big);
  dev_free(c->gkey); dev_free(c->tile_done); dev_free(c->clip); dev_free(c->vlight);
  dev_free(c->work); dev_free(c->d_result);
  if (c->h_result) cudaFreeHost(c->h_result);
  dev_free(c->fb_rgba); dev_free(c->fb_z);
  if (c->flush_buf) cudaFree(c->flush_buf);
  for (auto& ev : c->events) if (ev) cudaEventDestroy(ev);
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
  if (!c) return fail(GR_ERR_INVALID_ARGUMENT, "ctx is NULL");
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  if ((rgba_dev && !is_device_ptr(rgba_dev)) || (z_dev && !is_device_ptr(z_dev)))
    return fail(GR_ERR_INVALID_ARGUMENT, "gr_draw_async needs device output pointers");
  Prepared pr;
  int32_t st = prepare(c, items, n, p, pr);
  if (st) return st;
  const size_t px = (size_t)p->width * (size_t)p->height;
  if (!rgba_dev || !z_dev)
    if ((st = ensure_fb(c, px))) return st;
  set_outputs(pr.a, rgba_dev ? (uint32_t*)rgba_dev : c->fb_rgba, z_dev ? z_dev : c->fb_z);
  return launch(c, pr.a);
}

int32_t gr_draw_profiled(gr_context* c, const gr_draw_item* items, int32_t n, const gr_frame_params* p,
                         uint8_t* rgba_dev, float* z_dev, float* kernel_ms3) {
  if (!c || !kernel_ms3) return fail(GR_ERR_INVALID_ARGUMENT, "NULL argument");
  std::lock_guard<std::mutex> lk(c->mu);
  CK(cudaSetDevice(c->device));
  if ((rgba_dev && !is_device_ptr(rgba_dev)) || (z_dev && !is_device_ptr(z_dev)))
    return fail(GR_ERR_INVALID_ARGUMENT, "gr_draw_profiled needs device output pointers");
  const size_t px = (size_t)p->width * (size_t)p->height;
  int32_t st;
  for (int attempt = 0; attempt < 4; ++attempt) {
    Prepared pr;
    if ((st = prepare(c, items, n, p, pr))) return st;
    if (!rgba_dev || !z_dev)
      if ((st = ensure_fb(c, px))) return st;
    set_outputs(pr.a, rgba_dev ? (uint32_t*)rgba_dev : c->fb_rgba, z_dev ? z_dev : c->fb_z);
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

int32_t gr_host_alloc(int64_t bytes, void** out) {
  if (!out || bytes <= 0) return fail(GR_ERR_INVALID_ARGUMENT, "bad argument");
  CK(cudaMallocHost(out, (size_t)bytes));
  return GR_OK;
}

int32_t gr_host_free(void* p) {
  if (p) CK(cudaFreeHost(p));
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
