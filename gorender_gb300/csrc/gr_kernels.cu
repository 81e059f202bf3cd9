// gr_kernels.cu -- sm_103a kernels of the frame pipeline.
//
// A frame runs as a short sequence of kernels on one stream (captured once
// into a CUDA graph and replayed):
//   k_light    Gouraud intensity once per vertex normal.
//   k_vertex   clip-space position and unsnapped screen x, y once per vertex.
//   k_cull     faces in groups of 32 x G per warp: backface and frustum
//              tests on every face; faces kept whole are compacted into one
//              list, straddling faces go to k_clip (the general clipper, one
//              warp per face, beside k_setup).
//   k_setup    full warps of kept faces: attributes, screen vertices, bin
//              test (TPF) and edge-function setup; records are appended with
//              one atomic per warp and binned with warp-aggregated atomics
//              (__match_any_sync) or, past four tiles, queued for k_bin_big.
//   k_bin_big  one warp per multi-tile triangle: appends it to every tile its
//              edge functions can reach.
//   k_plan     splits heavy tiles into slices by estimated cost and orders
//              the work queue heaviest first.
//   k_raster   persistent CTAs over the queue, one TS x TS tile slice each:
//              visibility in shared memory as a 64-bit max of (ordered zRec,
//              draw-order key); each row of a footprint is narrowed to its
//              exact covered span, so only covered pixels reach the depth
//              test; slices merge through global keys.  Many views: the
//              tile is shaded in place.  One view: the final keys are stored
//              and
//   k_resolve  shades every pixel once for its winner (deferred), with Clear,
//              DotGrid, overlays, crosshair and fog, one thread per pixel.
//
// Bit-exactness: every float operation is an explicit round-to-nearest
// intrinsic in the reference's source order (no contraction; the files are
// also built with --fmad=false), Go amd64 float->int conversions are
// emulated, and edge functions use Go's int64 wraparound semantics.  The
// visibility rule reproduces the sequential z-test of rasterizer.go:156:
// the final pixel belongs to the LAST triangle in (object, face, fan) order
// among those with the maximum zRec >= -1 (NaN never passes), and Z holds
// that triangle's own zRec bits.
#include <cuda_runtime.h>

#include <algorithm>

#include "gr_internal.h"

namespace gr {

#define FULL_MASK 0xffffffffu

// ---------------------------------------------------------------------------
// exact fp32 arithmetic and Go conversions
// ---------------------------------------------------------------------------
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fd(float a, float b) { return __fdiv_rn(a, b); }

// int(float32) on Go amd64 (CVTTSS2SQ): truncate; NaN / out of range -> INT64_MIN.
__device__ __forceinline__ long long go_int(float f) {
  return (f >= -9223372036854775808.0f && f < 9223372036854775808.0f)
             ? __float2ll_rz(f)
             : (long long)0x8000000000000000ULL;
}
// uint8(float32): through int32 (CVTTSS2SL, indefinite 0x80000000), low byte.
__device__ __forceinline__ uint32_t go_u8(float f) {
  return (f >= -2147483648.0f && f < 2147483648.0f) ? ((uint32_t)__float2int_rz(f) & 0xFFu) : 0u;
}

struct V4 {
  float x, y, z, w;
};

// matrixMultiplyVec4Inplace / the batch transform: ((m0*x + m1*y) + m2*z) + m3*w.
__device__ __forceinline__ V4 mat_vec(const float* m, V4 v) {
  V4 r;
  r.x = fa(fa(fa(fm(m[0], v.x), fm(m[1], v.y)), fm(m[2], v.z)), fm(m[3], v.w));
  r.y = fa(fa(fa(fm(m[4], v.x), fm(m[5], v.y)), fm(m[6], v.z)), fm(m[7], v.w));
  r.z = fa(fa(fa(fm(m[8], v.x), fm(m[9], v.y)), fm(m[10], v.z)), fm(m[11], v.w));
  r.w = fa(fa(fa(fm(m[12], v.x), fm(m[13], v.y)), fm(m[14], v.z)), fm(m[15], v.w));
  return r;
}
__device__ __forceinline__ float dot4(V4 a, V4 b) {
  return fa(fa(fa(fm(a.x, b.x), fm(a.y, b.y)), fm(a.z, b.z)), fm(a.w, b.w));
}
__device__ __forceinline__ V4 sub4(V4 a, V4 b) {
  return V4{fs(a.x, b.x), fs(a.y, b.y), fs(a.z, b.z), fs(a.w, b.w)};
}
__device__ __forceinline__ V4 ld4(const float* p) {
  float4 q = __ldg(reinterpret_cast<const float4*>(p));
  return V4{q.x, q.y, q.z, q.w};
}

// The same for data read once a frame (vertex positions and normals in
// k_vertex and k_light): evict-first, so the per-vertex results, indices and
// records that later kernels gather stay in L2 instead.
__device__ __forceinline__ V4 ld4_stream(const float* p) {
  float4 q = __ldcs(reinterpret_cast<const float4*>(p));
  return V4{q.x, q.y, q.z, q.w};
}

// Frustum planes (clipping.go:93-129) with zNear = 0, zFar = 50 (renderer.go:121).
__constant__ float c_plane_p[6][4] = {{-1, 0, 0, 1}, {1, 0, 0, 1}, {0, -1, 0, 1},
                                      {0, 1, 0, 1},  {0, 0, 0, 1}, {0, 0, 50, 1}};
__constant__ float c_plane_n[6][4] = {{1, 0, 0, 1},  {-1, 0, 0, 1}, {0, 1, 0, 1},
                                      {0, -1, 0, 1}, {0, 0, -1, 0}, {0, 0, 1, 0}};

__device__ __forceinline__ V4 plane_p(int i) {
  return V4{c_plane_p[i][0], c_plane_p[i][1], c_plane_p[i][2], c_plane_p[i][3]};
}
__device__ __forceinline__ V4 plane_n(int i) {
  return V4{c_plane_n[i][0], c_plane_n[i][1], c_plane_n[i][2], c_plane_n[i][3]};
}
// Plane.IsVertexInside (clipping.go:74-76): (q - P) . N <= 0.
__device__ __forceinline__ bool plane_inside(int i, V4 q) {
  return dot4(sub4(q, plane_p(i)), plane_n(i)) <= 0.0f;
}

// Polygon vertex during clipping: position, UV, intensity, RGB (extension).
struct PV {
  V4 p;
  float u, v, in, r, g, b;
};

__device__ __forceinline__ float lerp32(float a, float b, float f) { return fa(a, fm(fs(b, a), f)); }

// Plane.Intersect (clipping.go:79-86) + lerp32/lerpUV of the attributes.
__device__ __forceinline__ PV intersect(int i, const PV& A, const PV& B) {
  V4 P = plane_p(i), N = plane_n(i);
  V4 u = sub4(B.p, A.p);
  V4 w = sub4(A.p, P);
  float d = dot4(N, u);
  float n = -dot4(N, w);
  float f = fd(n, d);
  PV o;
  o.p = V4{fa(A.p.x, fm(u.x, f)), fa(A.p.y, fm(u.y, f)), fa(A.p.z, fm(u.z, f)), fa(A.p.w, fm(u.w, f))};
  o.in = lerp32(A.in, B.in, f);
  o.u = fa(A.u, fm(fs(B.u, A.u), f));
  o.v = fa(A.v, fm(fs(B.v, A.v), f));
  o.r = lerp32(A.r, B.r, f);
  o.g = lerp32(A.g, B.g, f);
  o.b = lerp32(A.b, B.b, f);
  return o;
}

// Frustum.ClipTriangle (clipping.go:167-236) in place on poly (count 3 on
// entry).  Returns the polygon vertex count (0: clipped away) or -1 when the
// polygon would exceed 9 vertices (the reference panics there).
__device__ int clip_polygon(PV* poly, PV* tmp) {
  int count = 3;
  PV* a = poly;
  PV* b = tmp;
  for (int pi = 0; pi < 6; ++pi) {
    int n2 = 0;
    for (int bi = 0; bi < count; ++bi) {
      int ai = (bi + 1 == count) ? 0 : bi + 1;
      const PV A = a[ai];
      const PV B = a[bi];
      bool inA = plane_inside(pi, A.p);
      if (inA) {
        if (!plane_inside(pi, B.p)) {
          if (n2 >= 9) return -1;
          b[n2++] = intersect(pi, A, B);
        }
        if (n2 >= 9) return -1;
        b[n2++] = A;
      } else if (plane_inside(pi, B.p)) {
        if (n2 >= 9) return -1;
        b[n2++] = intersect(pi, A, B);
      }
    }
    if (n2 == 0) return 0;
    count = n2;
    PV* t = a;
    a = b;
    b = t;
  }
  if (a != poly)
    for (int k = 0; k < count; ++k) poly[k] = a[k];
  return count;
}

// Screen-space vertex after divide + screen map (renderer.go:361-370) and
// the int() truncations of drawProjection (renderer.go:182-184).
struct SV {
  long long X, Y;
  float sx, sy, W, u, v, in, r, g, b;
};

// Divide + screen map of a clip-space position (renderer.go:361-370): the
// whole vector divided by W (so W/W = 1), then the screen matrix's rows 0, 1.
__device__ __forceinline__ float2 screen_of(V4 p, const float* S) {
  const float W = p.w;
  const float dx = fd(p.x, W), dy = fd(p.y, W), dz = fd(p.z, W), dw = fd(p.w, W);
  return make_float2(fa(fa(fa(fm(S[0], dx), fm(S[1], dy)), fm(S[2], dz)), fm(S[3], dw)),
                     fa(fa(fa(fm(S[4], dx), fm(S[5], dy)), fm(S[6], dz)), fm(S[7], dw)));
}

// Screen vertex from precomputed screen coordinates and the corner's attributes.
__device__ __forceinline__ SV sv_of(float2 scr, float W, const PV& q) {
  SV s;
  s.sx = scr.x;
  s.sy = scr.y;
  s.X = go_int(s.sx);
  s.Y = go_int(s.sy);
  s.W = W;
  s.u = q.u;
  s.v = q.v;
  s.in = q.in;
  s.r = q.r;
  s.g = q.g;
  s.b = q.b;
  return s;
}

__device__ __forceinline__ SV to_screen(const PV& q, const float* S) {
  const float2 scr = screen_of(q.p, S);
  SV s;
  s.sx = scr.x;
  s.sy = scr.y;
  s.X = go_int(s.sx);
  s.Y = go_int(s.sy);
  s.W = q.p.w;
  s.u = q.u;
  s.v = q.v;
  s.in = q.in;
  s.r = q.r;
  s.g = q.g;
  s.b = q.b;
  return s;
}

// identifyTriangleTiles with the single screen tile (renderer.go:226-244):
// Go's min/max propagate NaN, so a NaN coordinate drops the triangle.
__device__ __forceinline__ bool bin_test(const SV& a, const SV& b, const SV& c, float Wf, float Hf) {
  if (isnan(a.sx) || isnan(b.sx) || isnan(c.sx) || isnan(a.sy) || isnan(b.sy) || isnan(c.sy)) return false;
  float minX = fminf(fminf(a.sx, b.sx), c.sx), maxX = fmaxf(fmaxf(a.sx, b.sx), c.sx);
  float minY = fminf(fminf(a.sy, b.sy), c.sy), maxY = fmaxf(fmaxf(a.sy, b.sy), c.sy);
  return maxX >= 0.0f && minX <= Wf && maxY >= 0.0f && minY <= Hf;
}

// Overlay record of a binned triangle (ShowEdges / ShowVertices).  Called by
// every lane of a converged warp; one atomic per warp.
__device__ __forceinline__ void emit_overlay(const FrameArgs& a, bool on, const SV& s0, const SV& s1, const SV& s2,
                                             uint32_t key, int view) {
  const unsigned m = __ballot_sync(FULL_MASK, on);
  if (!m) return;
  const unsigned lane = threadIdx.x & 31u;
  const int ldr = __ffs(m) - 1;
  uint32_t b = 0;
  if ((int)lane == ldr) b = atomicAdd(&a.work->novl, (uint32_t)__popc(m));
  b = __shfl_sync(FULL_MASK, b, ldr);
  if (!on) return;
  const uint32_t q = b + __popc(m & ((1u << lane) - 1u));
  if (q >= a.ovl_cap) {
    atomicMax(&a.work->ovl_need, q + 1);
    return;
  }
  Overlay o;
  o.X[0] = s0.X; o.X[1] = s1.X; o.X[2] = s2.X;
  o.Y[0] = s0.Y; o.Y[1] = s1.Y; o.Y[2] = s2.Y;
  o.sx[0] = s0.sx; o.sx[1] = s1.sx; o.sx[2] = s2.sx;
  o.sy[0] = s0.sy; o.sy[1] = s1.sy; o.sy[2] = s2.sy;
  o.key = key;
  o.view = (uint32_t)view;
  a.ovl[q] = o;
}

__device__ __forceinline__ long long min3ll(long long a, long long b, long long c) { return min(min(a, b), c); }
__device__ __forceinline__ long long max3ll(long long a, long long b, long long c) { return max(max(a, b), c); }

// Top-left adjustment (rasterizer.go:120-129): keep f when dy > 0 or
// (dy == 0 and dx > 0), else f - 1.
__device__ __forceinline__ bool keeps_edge(long long dx, long long dy) { return dy > 0 || (dy == 0 && dx > 0); }

// Setup of one fan triangle.  Returns false when no pixel can pass the
// inside test (empty clamped bounding box, or, for narrow triangles, a
// non-negative sum of the adjusted edge functions).
struct Setup {
  TriRaster r;
  TriWide w;
  bool wide;
};

__device__ __forceinline__ bool setup_tri(const SV& p0, const SV& p1, const SV& p2, int W, int H, Setup& s) {
  long long bx0 = max(min3ll(p0.X, p1.X, p2.X), 0LL);
  long long bx1 = min(max3ll(p0.X, p1.X, p2.X), (long long)W - 1);
  long long by0 = max(min3ll(p0.Y, p1.Y, p2.Y), 0LL);
  long long by1 = min(max3ll(p0.Y, p1.Y, p2.Y), (long long)H - 1);
  if (bx0 > bx1 || by0 > by1) return false;
  const long long lim = kNarrowLimit;
  bool narrow = p0.X > -lim && p0.X < lim && p1.X > -lim && p1.X < lim && p2.X > -lim && p2.X < lim &&
                p0.Y > -lim && p0.Y < lim && p1.Y > -lim && p1.Y < lim && p2.Y > -lim && p2.Y < lim;
  s.r.bx0 = (int16_t)bx0;
  s.r.bx1 = (int16_t)bx1;
  s.r.by0 = (int16_t)by0;
  s.r.by1 = (int16_t)by1;
  s.r.w0 = p0.W;
  s.r.w1 = p1.W;
  s.r.w2 = p2.W;
  if (narrow) {
    int x0 = (int)p0.X, y0 = (int)p0.Y, x1 = (int)p1.X, y1 = (int)p1.Y, x2 = (int)p2.X, y2 = (int)p2.Y;
    int a01 = y0 - y1, b01 = x1 - x0, c01 = x0 * y1 - x1 * y0;
    int a12 = y1 - y2, b12 = x2 - x1, c12 = x1 * y2 - x2 * y1;
    int a20 = y2 - y0, b20 = x0 - x2, c20 = x2 * y0 - x0 * y2;
    if (!keeps_edge(a01, b01)) c01 -= 1;
    if (!keeps_edge(a12, b12)) c12 -= 1;
    if (!keeps_edge(a20, b20)) c20 -= 1;
    long long sum = (long long)c01 + (long long)c12 + (long long)c20;
    if (sum >= 0) return false;
    s.r.a01 = a01; s.r.b01 = b01; s.r.c01 = c01;
    s.r.a12 = a12; s.r.b12 = b12; s.r.c12 = c12;
    s.r.a20 = a20; s.r.b20 = b20; s.r.c20 = c20;
    s.r.sumf = __ll2float_rn(sum);
    s.wide = false;
  } else {
    typedef unsigned long long u64;
    u64 x0 = (u64)p0.X, y0 = (u64)p0.Y, x1 = (u64)p1.X, y1 = (u64)p1.Y, x2 = (u64)p2.X, y2 = (u64)p2.Y;
    u64 a01 = y0 - y1, b01 = x1 - x0, c01 = x0 * y1 - x1 * y0;
    u64 a12 = y1 - y2, b12 = x2 - x1, c12 = x1 * y2 - x2 * y1;
    u64 a20 = y2 - y0, b20 = x0 - x2, c20 = x2 * y0 - x0 * y2;
    if (!keeps_edge((long long)a01, (long long)b01)) c01 -= 1;
    if (!keeps_edge((long long)a12, (long long)b12)) c12 -= 1;
    if (!keeps_edge((long long)a20, (long long)b20)) c20 -= 1;
    u64 sum = c01 + c12 + c20;
    s.w.a01 = (long long)a01; s.w.b01 = (long long)b01; s.w.c01 = (long long)c01;
    s.w.a12 = (long long)a12; s.w.b12 = (long long)b12; s.w.c12 = (long long)c12;
    s.w.a20 = (long long)a20; s.w.b20 = (long long)b20; s.w.c20 = (long long)c20;
    s.w.bx0 = s.w.bx1 = s.w.by0 = s.w.by1 = 0;
    s.r.a01 = s.r.b01 = s.r.c01 = s.r.a12 = s.r.b12 = s.r.c12 = s.r.a20 = s.r.b20 = s.r.c20 = 0;
    s.r.sumf = __ll2float_rn((long long)sum);
    s.wide = true;
  }
  return true;
}

// The raster record r as the raster, binning and resolve use it, rebuilt from
// its stored TriPacked for a view of W x H pixels: for a narrow triangle the
// same integer arithmetic as setup_tri, from the same corners, so the same
// values.
__device__ __forceinline__ TriRaster unpack_tri(const FrameArgs& a, uint32_t r, int W, int H) {
  const int4* src = reinterpret_cast<const int4*>(a.rast + r);
  const int4 c = src[0];
  const float4 w = reinterpret_cast<const float4*>(src)[1];
  TriRaster t;
  t.key = (uint32_t)c.w;
  t.w0 = w.x; t.w1 = w.y; t.w2 = w.z;
  if (t.key & 0x80000000u) {
    const TriWide& wd = a.wide[r];
    t.a01 = t.b01 = t.c01 = t.a12 = t.b12 = t.c12 = t.a20 = t.b20 = t.c20 = 0;
    t.sumf = w.w;
    t.bx0 = wd.bx0; t.bx1 = wd.bx1; t.by0 = wd.by0; t.by1 = wd.by1;
    return t;
  }
  const int x0 = (int16_t)(c.x & 0xFFFF), y0 = (int16_t)((uint32_t)c.x >> 16);
  const int x1 = (int16_t)(c.y & 0xFFFF), y1 = (int16_t)((uint32_t)c.y >> 16);
  const int x2 = (int16_t)(c.z & 0xFFFF), y2 = (int16_t)((uint32_t)c.z >> 16);
  t.a01 = y0 - y1; t.b01 = x1 - x0; t.c01 = x0 * y1 - x1 * y0;
  t.a12 = y1 - y2; t.b12 = x2 - x1; t.c12 = x1 * y2 - x2 * y1;
  t.a20 = y2 - y0; t.b20 = x0 - x2; t.c20 = x2 * y0 - x0 * y2;
  if (!keeps_edge(t.a01, t.b01)) t.c01 -= 1;
  if (!keeps_edge(t.a12, t.b12)) t.c12 -= 1;
  if (!keeps_edge(t.a20, t.b20)) t.c20 -= 1;
  t.sumf = __ll2float_rn((long long)t.c01 + (long long)t.c12 + (long long)t.c20);
  t.bx0 = (int16_t)max(min(min(x0, x1), x2), 0);
  t.bx1 = (int16_t)min(max(max(x0, x1), x2), W - 1);
  t.by0 = (int16_t)max(min(min(y0, y1), y2), 0);
  t.by1 = (int16_t)min(max(max(y0, y1), y2), H - 1);
  return t;
}

// Ordered 64-bit visibility key: high word = zRec mapped to an unsigned
// order (-0 folded onto +0), low word = draw-order key (0 for background).
__device__ __forceinline__ unsigned long long depth_key(float z, uint32_t okey) {
  uint32_t u = __float_as_uint(z);
  if (u == 0x80000000u) u = 0u;
  uint32_t o = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
  return ((unsigned long long)o << 32) | (unsigned long long)(okey & 0x7FFFFFFFu);
}
#define BG_KEY 0x407fffff00000000ULL  // depth_key(-1.0f, 0): ~0xbf800000 = 0x407fffff

// The zRec bits of visibility key k (the inverse of depth_key's order map);
// +0 also stands for a zRec of -0, which depth_key folds onto it.
__device__ __forceinline__ float key_depth(unsigned long long k) {
  const uint32_t o = (uint32_t)(k >> 32);
  return __uint_as_float((o & 0x80000000u) ? (o & 0x7FFFFFFFu) : ~o);
}

// Barycentrics and zRec at a covered pixel (rasterizer.go:149-153).
__device__ __forceinline__ float zrec_of(float e12f, float e20f, float sumf, float w0, float w1, float w2,
                                         float& al, float& be, float& ga) {
  al = fd(e12f, sumf);
  be = fd(e20f, sumf);
  ga = fs(fs(1.0f, al), be);
  return -fa(fa(fd(al, w0), fd(be, w1)), fd(ga, w2));
}

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialization may be scheduled while its predecessor is still finishing;
// it waits here, before reading anything, for the predecessor grid to
// complete with its writes visible (a no-op after an ordinary launch).
__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Tile-clipped pixel box of a triangle with box [bx0,bx1] x [by0,by1] in
// tile (tx, ty).
__device__ __forceinline__ uint32_t tile_box(int bx0, int bx1, int by0, int by1, uint32_t tx, uint32_t ty, int sh) {
  const int ts = 1 << sh;
  const int x0 = max(bx0, (int)(tx << sh)), x1 = min(bx1, (int)(tx << sh) + ts - 1);
  const int y0 = max(by0, (int)(ty << sh)), y1 = min(by1, (int)(ty << sh) + ts - 1);
  return (uint32_t)(max(0, x1 - x0 + 1) * max(0, y1 - y0 + 1));
}

// Reserves one bin entry of tile `tile` for a triangle whose tile-clipped box
// holds `box` pixels; boxes beyond kSmallBox add their area to the tile's
// raster cost estimate (small ones count kEntryCost each, in k_plan).
__device__ __forceinline__ uint32_t bin_append(const FrameArgs& a, uint32_t tile, uint32_t box) {
  if (box > (uint32_t)kSmallBox) atomicAdd(&a.tile_cost[tile], box);
  return atomicAdd(&a.bin_count[tile], 1u);
}

// Appends record r to tile t's bin; over capacity the position is recorded
// so the host can grow the bins and re-run the frame.
__device__ __forceinline__ void bin_store(const FrameArgs& a, uint32_t tile, uint32_t pos, uint32_t r) {
  if (pos < a.bin_cap)
    a.bins[(size_t)tile * a.bin_cap + pos] = r;
  else
    atomicMax(&a.work->bin_need, pos + 1);
}

// Appends record r, pixel box [bx0,bx1] x [by0,by1], to each of the at most
// kBinDirectMax tiles [tx0,tx1] x [ty0,ty1] of view vw: every tile's
// bin-count atomic is issued before any store, so their round trips overlap.
__device__ __forceinline__ void bin_direct(const FrameArgs& a, uint32_t tile_base, uint32_t tiles_x, uint32_t tx0,
                                           uint32_t tx1, uint32_t ty0, uint32_t ty1, int bx0, int bx1, int by0,
                                           int by1, uint32_t r) {
  const uint32_t nx = tx1 - tx0 + 1, n = nx * (ty1 - ty0 + 1);
  uint32_t tile[kBinDirectMax], pos[kBinDirectMax];
#pragma unroll
  for (int k = 0; k < kBinDirectMax; ++k) {
    if ((uint32_t)k < n) {
      const uint32_t dy = (uint32_t)k / nx, tx = tx0 + ((uint32_t)k - dy * nx), ty = ty0 + dy;
      tile[k] = tile_base + ty * tiles_x + tx;
      pos[k] = bin_append(a, tile[k], tile_box(bx0, bx1, by0, by1, tx, ty, a.tile_shift));
    }
  }
#pragma unroll
  for (int k = 0; k < kBinDirectMax; ++k)
    if ((uint32_t)k < n) bin_store(a, tile[k], pos[k], r);
}

// Lighting of one normal (renderer.go:326-346): 0.5 + (normalize(W*n) . L) * 0.5
// with Vec4.Normalize, whose length includes w.
__device__ __forceinline__ float light_of(const float* world, V4 nrm, const float* L) {
  V4 n = mat_vec(world, nrm);
  float len = __fsqrt_rn(fa(fa(fa(fm(n.x, n.x), fm(n.y, n.y)), fm(n.z, n.z)), fm(n.w, n.w)));
  float x = fd(n.x, len), y = fd(n.y, len), z = fd(n.z, len);
  float d = fa(fa(fm(x, L[0]), fm(y, L[1])), fm(z, L[2]));
  return fa(0.5f, fm(d, 0.5f));
}

__device__ __forceinline__ bool gouraud(const FrameArgs& a, const DevItem& it) {
  const uint32_t fl = a.views[it.view].flags;
  return (fl & 0x08u) && !(fl & 0x10u) && it.nn != 0;
}

// facingCamera (renderer.go:246-250) on clip-space vertices.
__device__ __forceinline__ bool facing_camera(V4 v0, V4 v1, V4 v2) {
  float e1x = fs(v1.x, v0.x), e1y = fs(v1.y, v0.y), e1z = fs(v1.z, v0.z);
  float e2x = fs(v2.x, v0.x), e2y = fs(v2.y, v0.y), e2z = fs(v2.z, v0.z);
  float nx = fs(fm(e1y, e2z), fm(e1z, e2y));
  float ny = fs(fm(e1z, e2x), fm(e1x, e2z));
  float nz = fs(fm(e1x, e2y), fm(e1y, e2x));
  float d = fa(fa(fm(nx, fs(0.0f, v0.x)), fm(ny, fs(0.0f, v0.y))), fm(nz, fs(0.0f, v0.z)));
  return d > 0.0f;
}

// Per-vertex attributes of face f (intensity, UV, RGB) and its texture slot.
__device__ __forceinline__ void face_attributes(const FrameArgs& a, const DevItem& it, int f, int i0, int i1, int i2,
                                                const float* world, PV& p0, PV& p1, PV& p2, int& tex) {
  const DevView& vw = a.views[it.view];
  const uint32_t fl = vw.flags;
  float in0, in1, in2;
  if (fl & 0x08u) {
    if (gouraud(a, it)) {
      // per-normal intensities computed once per frame by k_light
      const float* vl = a.vlight + it.light_base;
      in0 = __ldg(vl + __ldg(it.nidx + 3 * f));
      in1 = __ldg(vl + __ldg(it.nidx + 3 * f + 1));
      in2 = __ldg(vl + __ldg(it.nidx + 3 * f + 2));
    } else {
      in0 = in1 = in2 = light_of(world, ld4(it.fnrm + 4 * (size_t)f), vw.L);
    }
  } else {
    in0 = in1 = in2 = 0.5f;
  }
  p0.in = in0; p1.in = in1; p2.in = in2;
  const int t = it.tex ? __ldg(it.tex + f) : -1;
  tex = ((fl & 0x20u) && t >= 0) ? t : (it.vcol ? -2 : -1);  // renderer.go:176-178
  // texture coordinates reach the shading only through a texture, vertex
  // colours only without one: the other is left at zero
  if (tex >= 0 && it.uv) {
    const float2* uv = reinterpret_cast<const float2*>(it.uv + 6 * (size_t)f);
    const float2 t0 = __ldg(uv), t1 = __ldg(uv + 1), t2 = __ldg(uv + 2);
    p0.u = t0.x; p0.v = t0.y; p1.u = t1.x; p1.v = t1.y; p2.u = t2.x; p2.v = t2.y;
  } else {
    p0.u = p0.v = p1.u = p1.v = p2.u = p2.v = 0.0f;
  }
  if (tex == -2) {
    const float* c0 = it.vcol + 3 * (size_t)i0;
    const float* c1 = it.vcol + 3 * (size_t)i1;
    const float* c2 = it.vcol + 3 * (size_t)i2;
    p0.r = __ldg(c0); p0.g = __ldg(c0 + 1); p0.b = __ldg(c0 + 2);
    p1.r = __ldg(c1); p1.g = __ldg(c1 + 1); p1.b = __ldg(c1 + 2);
    p2.r = __ldg(c2); p2.g = __ldg(c2 + 1); p2.b = __ldg(c2 + 2);
  } else {
    p0.r = p0.g = p0.b = p1.r = p1.g = p1.b = p2.r = p2.g = p2.b = 0.0f;
  }
}

// Writes record r of a set-up triangle (raster part, int64 edges, shading).
// The caller records where the resolve finds it (rec_of_face).
__device__ __forceinline__ void write_record(const FrameArgs& a, uint32_t r, Setup& s, const SV& q0, const SV& q1,
                                             const SV& q2, int tex, uint32_t okey, bool from_kept = false) {
  s.r.key = okey | (s.wide ? 0x80000000u : 0u);
  int4* dst = reinterpret_cast<int4*>(a.rast + r);
  if (s.wide) {
    dst[0] = make_int4(0, 0, 0, (int)s.r.key);
    s.w.bx0 = s.r.bx0; s.w.bx1 = s.r.bx1; s.w.by0 = s.r.by0; s.w.by1 = s.r.by1;
    const int4* ws = reinterpret_cast<const int4*>(&s.w);
    int4* wd = reinterpret_cast<int4*>(a.wide + r);
#pragma unroll
    for (int q = 0; q < 5; ++q) wd[q] = ws[q];
  } else {  // narrow: |X|, |Y| < 2^14 (setup_tri)
    dst[0] = make_int4((int)(((uint32_t)(uint16_t)(int16_t)q0.X) | ((uint32_t)(uint16_t)(int16_t)q0.Y << 16)),
                       (int)(((uint32_t)(uint16_t)(int16_t)q1.X) | ((uint32_t)(uint16_t)(int16_t)q1.Y << 16)),
                       (int)(((uint32_t)(uint16_t)(int16_t)q2.X) | ((uint32_t)(uint16_t)(int16_t)q2.Y << 16)),
                       (int)s.r.key);
  }
  reinterpret_cast<float4*>(dst)[1] = make_float4(s.r.w0, s.r.w1, s.r.w2, s.r.sumf);
  reinterpret_cast<float4*>(a.shade)[r] = make_float4(q0.in, q1.in, q2.in, __int_as_float(tex == -2 && from_kept ? -3 : tex));
  if (tex >= 0) {  // read by the shading only through a texture (rasterizer.go:132-137)
    float4* uv = reinterpret_cast<float4*>(a.suv + r);
    uv[0] = make_float4(fd(q0.u, q0.W), fd(q0.v, q0.W), fd(q1.u, q1.W), fd(q1.v, q1.W));
    uv[1] = make_float4(fd(q2.u, q2.W), fd(q2.v, q2.W), 0.0f, 0.0f);
  }
  if (tex == -2 && !from_kept) {
    TriColor* c = a.tcol + r;
    c->c[0] = q0.r; c->c[1] = q0.g; c->c[2] = q0.b;
    c->c[3] = q1.r; c->c[4] = q1.g; c->c[5] = q1.b;
    c->c[6] = q2.r; c->c[7] = q2.g; c->c[8] = q2.b;
  }
}

// Record index of the triangle with order key okey (face * 8 + fan + 1): a
// face kept whole maps to its record, a clipped face to the first record of
// its fans, which lie side by side in fan order.
__device__ __forceinline__ uint32_t record_of_key(const FrameArgs& a, uint32_t okey) {
  const uint32_t e = a.rec_of_face[okey / (uint32_t)kKeysPerFace];
  return (e & kClipFace) ? (e & ~kClipFace) + (okey % (uint32_t)kKeysPerFace - 1u) : e;
}

// Binning without warp aggregation (the rare clipped path): up to
// kBinDirectMax tiles directly; returns true for a triangle spanning more,
// which the calling warp bins together (bin_tiles_warp).
__device__ __forceinline__ bool bin_record_direct(const FrameArgs& a, uint32_t r, const TriRaster& t, int view) {
  const DevView& vw = a.views[view];
  const uint32_t tx0 = (uint32_t)t.bx0 >> a.tile_shift, tx1 = (uint32_t)t.bx1 >> a.tile_shift;
  const uint32_t ty0 = (uint32_t)t.by0 >> a.tile_shift, ty1 = (uint32_t)t.by1 >> a.tile_shift;
  const uint32_t ntiles = (tx1 - tx0 + 1) * (ty1 - ty0 + 1);
  if (ntiles > (uint32_t)kBinDirectMax) return true;
  bin_direct(a, vw.tile_base, (uint32_t)vw.tiles_x, tx0, tx1, ty0, ty1, t.bx0, t.bx1, t.by0, t.by1, r);
  return false;
}

// One warp appends record r (view `view`) to every tile its box overlaps,
// lanes over the tiles; a narrow triangle skips tiles that one of its edges
// excludes entirely (the exact int32 edge minimum over the tile-clipped box
// is >= 0).  All lanes of the warp must call it with the same r.
__device__ __forceinline__ void bin_tiles_warp(const FrameArgs& a, uint32_t r, int view) {
  const int sh = a.tile_shift;
  const int ts = 1 << sh;
  const uint32_t lane = threadIdx.x & 31u;
  const DevView& vw = a.views[view];
  const TriRaster t = unpack_tri(a, r, vw.W, vw.H);
  const uint32_t tx0 = (uint32_t)t.bx0 >> sh, tx1 = (uint32_t)t.bx1 >> sh;
  const uint32_t ty0 = (uint32_t)t.by0 >> sh, ty1 = (uint32_t)t.by1 >> sh;
  const uint32_t nx = tx1 - tx0 + 1, n = nx * (ty1 - ty0 + 1);
  const bool wide = (t.key & 0x80000000u) != 0;
  for (uint32_t j = lane; j < n; j += 32u) {
    const uint32_t tx = tx0 + j % nx, ty = ty0 + j / nx;
    if (!wide) {
      const int X0 = max((int)(tx << sh), (int)t.bx0);
      const int X1 = min((int)(tx << sh) + ts - 1, (int)t.bx1);
      const int Y0 = max((int)(ty << sh), (int)t.by0);
      const int Y1 = min((int)(ty << sh) + ts - 1, (int)t.by1);
      const int e01 = t.c01 + min(t.a01 * X0, t.a01 * X1) + min(t.b01 * Y0, t.b01 * Y1);
      const int e12 = t.c12 + min(t.a12 * X0, t.a12 * X1) + min(t.b12 * Y0, t.b12 * Y1);
      const int e20 = t.c20 + min(t.a20 * X0, t.a20 * X1) + min(t.b20 * Y0, t.b20 * Y1);
      if (e01 >= 0 || e12 >= 0 || e20 >= 0) continue;
    }
    const uint32_t tile = vw.tile_base + ty * (uint32_t)vw.tiles_x + tx;
    bin_store(a, tile, bin_append(a, tile, tile_box(t.bx0, t.bx1, t.by0, t.by1, tx, ty, sh)), r);
  }
}

// The item owning this block: kind 0 face blocks (k_cull), 1 normal blocks
// (k_light), 2 vertex blocks (k_vertex): the last item whose first block is
// at most blockIdx.x (the bases never decrease; item 0's is 0).  Called by a
// whole warp: each round probes 32 items spread over the remaining range at
// once, so a frame of up to 32 items takes one round trip and one of 1024
// two, where a binary search over the item table takes log2(items).
__device__ __forceinline__ int find_item(const FrameArgs& a, int kind) {
  const int lane = (int)lane_id();
  int lo = 0, hi = a.num_items - 1;  // the answer lies in [lo, hi]
  while (lo < hi) {
    const int step = (hi - lo + 31) >> 5;  // probes lo + 1, lo + 1 + step, ... cover (lo, hi]
    const int p = lo + 1 + lane * step;
    bool ok = false;
    if (p <= hi) {
      const DevItem& m = a.items[p];
      const int base = kind == 1 ? m.light_block_base : kind == 2 ? m.vert_block_base : m.block_base;
      ok = base <= (int)blockIdx.x;
    }
    const unsigned got = __ballot_sync(FULL_MASK, ok);  // a prefix of the lanes
    if (!got) break;                                     // no later item qualifies: lo
    const int last = 31 - __clz((int)got);
    lo += 1 + last * step;
    hi = min(hi, lo + step - 1);
  }
  return lo;
}

// ---------------------------------------------------------------------------
// k_vertex: every vertex of every item transformed once per frame
// (matrixMultiplyVec4Batch, renderer.go:303-304) and mapped to the screen
// (renderer.go:361-370).  Faces share vertices, and the result of a vertex
// does not depend on the face that uses it, so the face pass gathers these
// instead of transforming each corner again.
// ---------------------------------------------------------------------------
template <int G>
__global__ void __launch_bounds__(256) k_vertex(const FrameArgs a) {
  griddep_wait();  // after k_stage's tables (a no-op without a programmatic launch)
  __shared__ float s_mvp[16];
  __shared__ float s_S[8];
  __shared__ int s_item;
  if (threadIdx.x < 32) {
    const int item = find_item(a, 2);
    if (threadIdx.x == 0) s_item = item;
  }
  __syncthreads();
  const DevItem& it = a.items[s_item];
  if (threadIdx.x < 16) s_mvp[threadIdx.x] = it.mvp[threadIdx.x];
  if (threadIdx.x < 8) s_S[threadIdx.x] = a.views[it.view].S[threadIdx.x];
  __syncthreads();
  const int v0 = ((int)blockIdx.x - it.vert_block_base) * (256 * G) + (int)threadIdx.x;
#pragma unroll
  for (int k = 0; k < G; ++k) {
    const int v = v0 + k * 256;
    if (v < it.nv) {
      const V4 c = mat_vec(s_mvp, ld4_stream(it.pos + 4 * (size_t)v));
      a.vclip[it.vert_base + v] = make_float4(c.x, c.y, c.z, c.w);
      const float2 sc = screen_of(c, s_S);
      a.vscr[it.vert_base + v] = make_float4(sc.x, sc.y, c.w, 0.0f);  // W beside x, y: one gather in k_setup
    }
  }
}

// ---------------------------------------------------------------------------
// k_light: Gouraud intensity of every vertex normal of every item, once per
// frame.  The reference normalises WorldVertexNormals[NormalIndices[k]] per
// face corner (renderer.go:327-333); the value depends only on the normal
// index, so computing it once per normal gives the same bits.
// ---------------------------------------------------------------------------
template <int G>
__global__ void __launch_bounds__(256) k_light(const FrameArgs a) {
  __shared__ float s_world[16];
  __shared__ int s_item;
  if (threadIdx.x < 32) {
    const int item = find_item(a, 1);
    if (threadIdx.x == 0) s_item = item;
  }
  __syncthreads();
  const DevItem& it = a.items[s_item];
  if (threadIdx.x < 16) s_world[threadIdx.x] = it.world[threadIdx.x];
  __syncthreads();
  if (!gouraud(a, it)) return;
  const int n0 = ((int)blockIdx.x - it.light_block_base) * (256 * G) + (int)threadIdx.x;
#pragma unroll
  for (int k = 0; k < G; ++k) {
    const int n = n0 + k * 256;
    if (n < it.nn)
      a.vlight[it.light_base + n] = light_of(s_world, ld4_stream(it.vnrm + 4 * (size_t)n), a.views[it.view].L);
  }
}

// ---------------------------------------------------------------------------
// k_cull: G faces a thread, the backface and frustum tests of every face.
// Faces for the general clipper are queued for k_clip; faces kept whole are
// compacted over the CTA and appended to the kept list with one atomic per
// CTA, for k_setup.  Most faces of a closed mesh face away or miss the
// screen, so the setup runs on full warps of kept faces instead of on the
// few survivors of each warp, and k_clip can start as soon as this pass ends.
// ---------------------------------------------------------------------------
template <int G>
__global__ void __launch_bounds__(kProjectThreads) k_cull(const FrameArgs a) {
  griddep_wait();
  __shared__ int s_item;
  constexpr int kWarps = kProjectThreads / 32;
  __shared__ uint32_t s_wn[kWarps];
  __shared__ uint32_t s_base;
  __shared__ uint2 s_keep[kWarps][32 * G];  // (item, face) of the warp's kept faces

  const int tid = threadIdx.x;
  if (tid < 32) {
    const int item = find_item(a, 0);
    if (tid == 0) s_item = item;
  }
  __syncthreads();
  const int item = s_item;
  const DevItem& it = a.items[item];
  // Frustum.BoxVisibility of the transformed bounding box (renderer.go:268-275),
  // computed once per item where the box is known (box_visibility)
  const int vis = it.vis;
  if (vis == 0) return;  // whole block: object outside the frustum
  const DevView& vw = a.views[it.view];

  const uint32_t fl = vw.flags;
  const unsigned lane = lane_id();
  const int warp = tid >> 5;
  // The clip-space corners come from k_vertex: the same arithmetic, done
  // once per vertex.
  uint2* keep_list = s_keep[warp];
  int nkeep = 0;
  const int fgroup = ((int)blockIdx.x - it.block_base) * (kProjectThreads * G) + warp * (32 * G);
  const int nf = it.nf;
  const int* vidx = it.vidx;
  // A face's vertex indices are loaded one face ahead (G > 1), so that the
  // next load from memory overlaps this face's corner gathers and tests.
  int n0 = 0, n1 = 0, n2 = 0;
  if (fgroup + (int)lane < nf) {
    const int f = fgroup + (int)lane;
    n0 = __ldg(vidx + 3 * f);
    n1 = __ldg(vidx + 3 * f + 1);
    n2 = __ldg(vidx + 3 * f + 2);
  }
#pragma unroll
  for (int k = 0; k < G; ++k) {
    const int f = fgroup + k * 32 + (int)lane;
    const int i0 = n0, i1 = n1, i2 = n2;
    if (k + 1 < G && f + 32 < nf) {
      n0 = __ldg(vidx + 3 * (f + 32));
      n1 = __ldg(vidx + 3 * (f + 32) + 1);
      n2 = __ldg(vidx + 3 * (f + 32) + 2);
    }
    bool draw = false;
    bool general = false;  // this face needs the general clipper (k_clip)
    if (f < nf) {
      const float4 c0 = __ldg(a.vclip + it.vert_base + i0), c1 = __ldg(a.vclip + it.vert_base + i1),
                   c2 = __ldg(a.vclip + it.vert_base + i2);
      const V4 v0{c0.x, c0.y, c0.z, c0.w}, v1{c1.x, c1.y, c1.z, c1.w}, v2{c2.x, c2.y, c2.z, c2.w};
      draw = !(fl & 0x04u) || facing_camera(v0, v1, v2);  // BackfaceCulling
      // Frustum clipping (renderer.go:349-359).  At the first plane, in
      // clipping order, where not all three vertices are inside: all outside
      // means the polygon reaching that plane is still the face itself (every
      // earlier pass only rotated it), so ClipTriangle returns no triangle; a
      // mix needs the general clipper.  With no such plane the six passes
      // rotate the face back to itself and it passes through unchanged.
      if (draw && (fl & 0x01u) && vis != 2) {
        for (int i = 0; i < 6; ++i) {
          const int m = (int)plane_inside(i, v0) + (int)plane_inside(i, v1) + (int)plane_inside(i, v2);
          if (m == 3) continue;
          if (m == 0) draw = false;
          else general = true;
          break;
        }
      }
    }
    // Faces for the general clipper: one atomic per warp.
    const unsigned gm = __ballot_sync(FULL_MASK, general);
    if (gm) {
      uint32_t qb = 0;
      const int ldr = __ffs(gm) - 1;
      if ((int)lane == ldr) qb = atomicAdd(&a.work->nclip, (uint32_t)__popc(gm));
      qb = __shfl_sync(FULL_MASK, qb, ldr);
      if (general) {
        const uint32_t q = qb + __popc(gm & ((1u << lane) - 1u));
        if (q < a.clip_cap) a.clip[q] = make_uint2((uint32_t)item, (uint32_t)f);
        else atomicMax(&a.work->clip_need, q + 1);
      }
    }
    const bool keep = draw && !general;
    const unsigned km = __ballot_sync(FULL_MASK, keep);
    if (keep) keep_list[nkeep + __popc(km & ((1u << lane) - 1u))] = make_uint2((uint32_t)item, (uint32_t)f);
    nkeep += __popc(km);
  }
  // The CTA's kept faces: one atomic, each warp's run at its offset.
  if (lane == 0) s_wn[warp] = (uint32_t)nkeep;
  __syncthreads();
  if (tid == 0) {
    uint32_t t = 0;
    for (int w = 0; w < kWarps; ++w) {
      const uint32_t n = s_wn[w];
      s_wn[w] = t;
      t += n;
    }
    s_base = t ? atomicAdd(&a.work->nkept, t) : 0u;
  }
  __syncthreads();
  const uint32_t base = s_base + s_wn[warp];
  for (int k = (int)lane; k < nkeep; k += 32) {
    const uint32_t q = base + (uint32_t)k;
    if (q < a.kept_cap) a.kept[q] = keep_list[k];
  }
}

// ---------------------------------------------------------------------------
// k_setup: the faces k_cull kept, 32 a warp over the whole list: attributes,
// screen vertices, the bin test (TPF), setup, the record and its bins.  A
// warp's faces may belong to different items and views.
// ---------------------------------------------------------------------------
// CTAS resident CTAs an SM (setup_ctas_per_sm): 2 measured 3 us less than 4
// CTAs with spills on a 200k-face frame.  Registers are capped at 104 with 2
// CTAs (2 x 256 x 104 = 53,248: a 96-register k_clip CTA still fits beside
// them, as k_clip runs beside k_setup) and at 80 with 3 (3 x 256 x 80).
template <int CTAS>
__global__ void __maxnreg__(CTAS == 3 ? 80 : 104) k_setup(const FrameArgs a) {
  griddep_wait();
  const uint32_t nkept = min(*(volatile uint32_t*)&a.work->nkept, a.kept_cap);
  const unsigned lane = lane_id();
  // consecutive chunks of 32 go to different CTAs, so that the SMs share a short list evenly
  const uint32_t gwarp = (threadIdx.x >> 5) * gridDim.x + blockIdx.x;
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t k0 = gwarp * 32u; k0 < nkept; k0 += warps * 32u) {
    // the record of kept face k is record k: no atomic, no second setup
    const uint32_t r = k0 + lane;
    const bool valid = r < nkept;
    const uint2 e = a.kept[valid ? r : 0u];  // (item, face)
    const DevItem& it = a.items[e.x];
    const int f = (int)e.y;
    const int view = it.view;
    const uint32_t vbase = it.vert_base, okey = (it.face_base + e.y) * (uint32_t)kKeysPerFace + 1u;
    const DevView& vw = a.views[view];
    const uint32_t fl = vw.flags;
    const int W = vw.W, H = vw.H;
    const uint32_t tile_base = vw.tile_base, tiles_x = (uint32_t)vw.tiles_x;
    bool emit = false;   // this face yields one record
    int ntpf = 0;
    int tex = -1;
    SV s0, s1, s2;
    Setup s;
    if (valid) {
      PV p0, p1, p2;
      const int i0 = __ldg(it.vidx + 3 * f), i1 = __ldg(it.vidx + 3 * f + 1), i2 = __ldg(it.vidx + 3 * f + 2);
      const uint32_t v0 = vbase + i0, v1 = vbase + i1, v2 = vbase + i2;
      face_attributes(a, it, f, i0, i1, i2, it.world, p0, p1, p2, tex);
      const float4 q0 = __ldg(a.vscr + v0), q1 = __ldg(a.vscr + v1), q2 = __ldg(a.vscr + v2);
      s0 = sv_of(make_float2(q0.x, q0.y), q0.z, p0);
      s1 = sv_of(make_float2(q1.x, q1.y), q1.z, p1);
      s2 = sv_of(make_float2(q2.x, q2.y), q2.z, p2);
      if (bin_test(s0, s1, s2, (float)W, (float)H)) {
        ntpf = 1;
        // ShowFaces off: triangles still count in TPF but are not rasterised (renderer.go:180)
        emit = (fl & 0x02u) && setup_tri(s0, s1, s2, W, H, s);
      }
    }

    // TPF: one atomic per view present in the warp (nearly always one).
    unsigned pend = __ballot_sync(FULL_MASK, ntpf != 0);
    while (pend) {
      const int ldr = __ffs(pend) - 1;
      const int v = __shfl_sync(FULL_MASK, view, ldr);
      const unsigned mine = __ballot_sync(FULL_MASK, ntpf != 0 && view == v);
      if ((int)lane == ldr) atomicAdd(&a.view_tpf[v], (unsigned long long)__popc(mine));
      pend &= ~mine;
    }
    if (__any_sync(FULL_MASK, fl & 0xC0u))  // ShowEdges / ShowVertices: every binned triangle leaves marks
      emit_overlay(a, ntpf != 0 && (fl & 0xC0u), s0, s1, s2, okey, view);

    const bool ok = emit && r < a.rec_cap;
    if (emit && !ok) atomicMax(&a.work->rec_need, r + 1u);
    uint32_t tx0 = 0, tx1 = 0, ty0 = 0, ty1 = 0;
    int pbx0 = 0, pbx1 = -1, pby0 = 0, pby1 = -1;  // the record's pixel box
    if (ok) {
      write_record(a, r, s, s0, s1, s2, tex, okey, true);
      if (okey / (uint32_t)kKeysPerFace < a.face_cap) a.rec_of_face[okey / (uint32_t)kKeysPerFace] = r;
      pbx0 = s.r.bx0; pbx1 = s.r.bx1; pby0 = s.r.by0; pby1 = s.r.by1;
      tx0 = (uint32_t)s.r.bx0 >> a.tile_shift;
      tx1 = (uint32_t)s.r.bx1 >> a.tile_shift;
      ty0 = (uint32_t)s.r.by0 >> a.tile_shift;
      ty1 = (uint32_t)s.r.by1 >> a.tile_shift;
    }
    const uint32_t ntiles = ok ? (tx1 - tx0 + 1) * (ty1 - ty0 + 1) : 0u;
    // One to four tiles: the k-th tile of every lane's box in round k, one
    // bin-count atomic per distinct tile of the round (neighbouring faces
    // share tiles, and the hot tiles of a frame take hundreds of entries:
    // per-lane atomics on them serialise).  All rounds' atomics are issued
    // before any result is used, so their round trips overlap.
    const uint32_t nx = tx1 - tx0 + 1;
    uint32_t tile[kBinDirectMax], grp[kBinDirectMax], pos[kBinDirectMax];
#pragma unroll
    for (int k = 0; k < kBinDirectMax; ++k) {
      const bool act = (uint32_t)k < ntiles && ntiles <= (uint32_t)kBinDirectMax;
      const unsigned am = __ballot_sync(FULL_MASK, act);
      grp[k] = 0u;
      pos[k] = 0u;
      if (act) {
        const uint32_t dy = (uint32_t)k / nx, tx = tx0 + ((uint32_t)k - dy * nx), ty = ty0 + dy;
        tile[k] = tile_base + ty * tiles_x + tx;
        grp[k] = __match_any_sync(am, tile[k]);
        const uint32_t box = tile_box(pbx0, pbx1, pby0, pby1, tx, ty, a.tile_shift);
        const uint32_t cost = __reduce_add_sync(grp[k], box > (uint32_t)kSmallBox ? box : 0u);
        if ((int)lane == __ffs(grp[k]) - 1) {
          if (cost) atomicAdd(&a.tile_cost[tile[k]], cost);
          pos[k] = atomicAdd(&a.bin_count[tile[k]], (uint32_t)__popc(grp[k]));
        }
      }
    }
#pragma unroll
    for (int k = 0; k < kBinDirectMax; ++k) {
      if (grp[k]) {
        const uint32_t p = __shfl_sync(grp[k], pos[k], __ffs(grp[k]) - 1) + __popc(grp[k] & ((1u << lane) - 1u));
        bin_store(a, tile[k], p, r);
      }
    }
    // more: the multi-tile queue, one atomic per warp
    const bool many = ntiles > (uint32_t)kBinDirectMax;
    const unsigned mm = __ballot_sync(FULL_MASK, many);
    if (mm) {
      uint32_t qb = 0;
      const int l2 = __ffs(mm) - 1;
      if ((int)lane == l2) qb = atomicAdd(&a.work->nbig, (uint32_t)__popc(mm));
      qb = __shfl_sync(FULL_MASK, qb, l2);
      if (many) {
        const uint32_t q = qb + __popc(mm & ((1u << lane) - 1u));
        if (q < a.big_cap) a.big[q] = make_uint2(r, (uint32_t)view);
        else atomicMax(&a.work->big_need, q + 1);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// k_clip: faces that straddle a frustum plane, one warp per face.  The
// polygon lives in registers, vertex k on lane k.  Each plane pass of
// Frustum.ClipTriangle (clipping.go:199-232) visits edges b = 0..count-1 with
// A = vertex b+1, B = vertex b and emits (I, A), (A), (I) or nothing; here lane
// b computes its edge's outputs, a warp scan of the output counts gives their
// positions in the reference's order, and every output lane gathers its
// vertex with shuffles.  Fan triangles (clipping.go:42-62) go one per lane.
// ---------------------------------------------------------------------------
__device__ __forceinline__ PV shfl_pv(const PV& v, int src) {
  PV o;
  o.p.x = __shfl_sync(FULL_MASK, v.p.x, src);
  o.p.y = __shfl_sync(FULL_MASK, v.p.y, src);
  o.p.z = __shfl_sync(FULL_MASK, v.p.z, src);
  o.p.w = __shfl_sync(FULL_MASK, v.p.w, src);
  o.u = __shfl_sync(FULL_MASK, v.u, src);
  o.v = __shfl_sync(FULL_MASK, v.v, src);
  o.in = __shfl_sync(FULL_MASK, v.in, src);
  o.r = __shfl_sync(FULL_MASK, v.r, src);
  o.g = __shfl_sync(FULL_MASK, v.g, src);
  o.b = __shfl_sync(FULL_MASK, v.b, src);
  return o;
}

__device__ __forceinline__ SV shfl_sv(const SV& v, int src) {
  SV o;
  o.X = __shfl_sync(FULL_MASK, v.X, src);
  o.Y = __shfl_sync(FULL_MASK, v.Y, src);
  o.sx = __shfl_sync(FULL_MASK, v.sx, src);
  o.sy = __shfl_sync(FULL_MASK, v.sy, src);
  o.W = __shfl_sync(FULL_MASK, v.W, src);
  o.u = __shfl_sync(FULL_MASK, v.u, src);
  o.v = __shfl_sync(FULL_MASK, v.v, src);
  o.in = __shfl_sync(FULL_MASK, v.in, src);
  o.r = __shfl_sync(FULL_MASK, v.r, src);
  o.g = __shfl_sync(FULL_MASK, v.g, src);
  o.b = __shfl_sync(FULL_MASK, v.b, src);
  return o;
}

// Capped at 96 registers (128 threads a CTA): k_clip runs beside k_setup,
// and one of its CTAs (12,288 registers) then fits beside two k_setup<2> CTAs
// (2 x 26,624) on an SM; at 104+ registers it waited for k_setup's CTAs to
// leave, and k_plan waited for it (same-box A/B: heightfield +5 us).
__global__ void __maxnreg__(96) k_clip(const FrameArgs a) {
  griddep_wait();
  const uint32_t nclip = min(*(volatile uint32_t*)&a.work->nclip, a.clip_cap);
  const uint32_t nkept = *(volatile uint32_t*)&a.work->nkept;
  const int lane = (int)lane_id();
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); q < nclip; q += warps) {
    const uint2 e = a.clip[q];
    const DevItem& it = a.items[e.x];
    const int f = (int)e.y;
    // lanes 0..2: the face's vertices with their attributes
    PV v;
    int tex = -1;
    {
      const int i0 = __ldg(it.vidx + 3 * f), i1 = __ldg(it.vidx + 3 * f + 1), i2 = __ldg(it.vidx + 3 * f + 2);
      PV p0, p1, p2;
      face_attributes(a, it, f, i0, i1, i2, it.world, p0, p1, p2, tex);
      const int ik = lane == 0 ? i0 : (lane == 1 ? i1 : i2);
      v = lane == 0 ? p0 : (lane == 1 ? p1 : p2);
      v.p = mat_vec(it.mvp, ld4(it.pos + 4 * (size_t)ik));
    }
    int count = 3;
    bool overflow = false;
    // A pass whose plane has every vertex inside emits A for every edge b
    // (a = (b+1) % count): the polygon rotated by one.  Such passes only
    // advance `rot` (logical vertex i sits on lane (i + rot) % count); the
    // rotation is applied before the next pass that cuts, and at the end.
    int rot = 0;
    for (int pi = 0; pi < 6 && count > 0; ++pi) {
      const bool act = lane < count;
      if (__all_sync(FULL_MASK, !act || plane_inside(pi, v.p))) {
        rot = rot + 1 == count ? 0 : rot + 1;
        continue;
      }
      if (rot) {
        v = shfl_pv(v, (lane + rot) % count);
        rot = 0;
      }
      const PV A = shfl_pv(v, (lane + 1 < count) ? lane + 1 : 0);  // a = (b+1) % count
      const bool inA = act && plane_inside(pi, A.p);
      const bool inB = act && plane_inside(pi, v.p);
      const int nout = inA ? (inB ? 1 : 2) : (inB ? 1 : 0);
      PV X = A;
      if (inA != inB) X = intersect(pi, A, v);
      // exclusive scan of the output counts in edge order
      int incl = nout;
#pragma unroll
      for (int o = 1; o < 16; o <<= 1) {
        const int y = __shfl_up_sync(FULL_MASK, incl, o);
        if (lane >= o) incl += y;
      }
      const int total = __shfl_sync(FULL_MASK, incl, 15);
      const int pos = incl - nout;
      if (total > 9) {  // the reference would index past its 9-vertex arrays
        overflow = true;
        break;
      }
      // output j comes from the last edge lane whose range starts at or before j
      int src = 0;
      for (int l = 0; l < 9; ++l) {
        const int pl = __shfl_sync(FULL_MASK, pos, l);
        const int nl = __shfl_sync(FULL_MASK, nout, l);
        if (nl > 0 && pl <= lane) src = l;
      }
      const int spos = __shfl_sync(FULL_MASK, pos, src);
      const int sn = __shfl_sync(FULL_MASK, nout, src);
      const PV gX = shfl_pv(X, src);
      const PV gA = shfl_pv(A, src);
      // a two-output edge emits (I, A); a one-output edge emits A when A is
      // inside, else I
      const int src_in_a = __shfl_sync(FULL_MASK, (int)inA, src);  // every lane shuffles
      const bool takeX = (sn == 2) ? (lane == spos) : !src_in_a;
      if (lane < total) v = takeX ? gX : gA;
      count = total;
    }
    if (overflow) {
      if (lane == 0) atomicOr(&a.work->error, 1u);
      continue;
    }
    if (count < 3) continue;  // Polygon.Triangulate returns nothing
    if (rot) v = shfl_pv(v, (lane + rot) % count);
    const DevView& vw = a.views[it.view];
    const SV sv = to_screen(v, vw.S);  // lane k: polygon vertex k
    const SV s0 = shfl_sv(sv, 0), s1 = shfl_sv(sv, lane + 1 < 9 ? lane + 1 : 0),
             s2 = shfl_sv(sv, lane + 2 < 9 ? lane + 2 : 0);
    const bool fan = lane + 2 < count;
    int ntpf = 0;
    bool many = false;  // spans more than kBinDirectMax tiles: binned by the warp below
    uint32_t rr = 0;
    Setup s;
    bool emit = false;
    if (fan && bin_test(s0, s1, s2, (float)vw.W, (float)vw.H)) {
      ntpf = 1;
      emit = (vw.flags & 0x02u) && setup_tri(s0, s1, s2, vw.W, vw.H, s);
    }
    // The face's fan records are consecutive, after the kept faces' records:
    // one slot a fan (a fan that yields no record leaves its slot unused), so
    // the resolve finds fan k at the first record + k.
    const unsigned em = __ballot_sync(FULL_MASK, emit);
    if (em) {
      uint32_t first = 0;
      if (lane == 0) {
        first = nkept + atomicAdd(&a.work->nrec, (uint32_t)(count - 2));
        if (it.face_base + (uint32_t)f < a.face_cap) a.rec_of_face[it.face_base + (uint32_t)f] = kClipFace | first;
      }
      first = __shfl_sync(FULL_MASK, first, 0);
      const uint32_t r = first + (uint32_t)lane;
      if (emit && r < a.rec_cap) {
        write_record(a, r, s, s0, s1, s2, tex, (it.face_base + (uint32_t)f) * (uint32_t)kKeysPerFace + (uint32_t)lane + 1u);
        many = bin_record_direct(a, r, s.r, it.view);
        rr = r;
      } else if (emit) {
        atomicMax(&a.work->rec_need, r + 1);
      }
    }
    // Fan triangles over many tiles, one at a time by the whole warp, so that
    // k_clip needs nothing from k_bin_big and the two run side by side.
    unsigned mm = __ballot_sync(FULL_MASK, many);
    __syncwarp();  // the records just written are read by the other lanes
    while (mm) {
      const int l = __ffs(mm) - 1;
      mm &= mm - 1u;
      bin_tiles_warp(a, __shfl_sync(FULL_MASK, rr, l), it.view);
    }
    const int wt = __reduce_add_sync(FULL_MASK, ntpf);
    if (lane == 0 && wt) atomicAdd(&a.view_tpf[it.view], (unsigned long long)wt);
    if (vw.flags & 0xC0u)
      emit_overlay(a, ntpf != 0, s0, s1, s2,
                   (it.face_base + (uint32_t)f) * (uint32_t)kKeysPerFace + (uint32_t)lane + 1u, it.view);
  }
}

// ---------------------------------------------------------------------------
// k_bin_big: one warp per multi-tile triangle
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_bin_big(const FrameArgs a) {
  griddep_wait();
  const uint32_t nbig = min(*(volatile uint32_t*)&a.work->nbig, a.big_cap);
  // one warp per queued triangle: most span 5 to a few dozen tiles
  const uint32_t warps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t q = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); q < nbig; q += warps) {
    const uint2 be = a.big[q];
    bin_tiles_warp(a, be.x, (int)be.y);
  }
}

// ---------------------------------------------------------------------------
// k_raster / k_resolve: shading helpers, the per-tile raster, the resolve
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t tex_sample(const DevTex& t, float u, float v) {
  // Texture.Sample (texture.go:69-89)
  if (t.kind == 0) return t.color;
  if (t.kind == 2) {
    long long x = go_int(fm(fm(fs(1.0f, u), t.scale), t.widthF)) & (long long)(t.width - 1);
    long long y = go_int(fm(fm(v, t.scale), t.heightF)) & (long long)(t.height - 1);
    return __ldg(t.px + y * t.width + x);
  }
  if (t.kind == 1) {
    long long x = go_int(fm(fm(fs(1.0f, u), t.scale), t.widthF)) % (long long)t.width;
    long long y = go_int(fm(fm(v, t.scale), t.heightF)) % (long long)t.height;
    long long idx = y * t.width + x;
    if (idx < 0) idx = 0;
    return __ldg(t.px + idx);
  }
  return 0xFFFF00FFu;  // magenta (255, 0, 255, 255)
}

__device__ __forceinline__ uint32_t color_intensity(uint32_t c, float I) {
  // colorIntensity (rasterizer.go:81-88)
  uint32_t r = go_u8(fm((float)(c & 0xFFu), I));
  uint32_t g = go_u8(fm((float)((c >> 8) & 0xFFu), I));
  uint32_t b = go_u8(fm((float)((c >> 16) & 0xFFu), I));
  return r | (g << 8) | (b << 16) | (c & 0xFF000000u);
}

// FrameBuffer.CrossHair (rasterizer.go:209-217): four 3-pixel lines 3..5
// pixels from the centre, plotted through FrameBuffer.Pixel (linear index,
// index 0 skipped).  True when pixel (x, y) is one of them.
__device__ __forceinline__ bool crosshair_hit(int W, int H, int x, int y) {
  const long long cx = W / 2, cy = H / 2, i = (long long)y * W + x, n = (long long)W * H;
#pragma unroll
  for (int k = 3; k <= 5; ++k) {
    const long long p[4] = {cy * W + (cx - k), cy * W + (cx + k), (cy - k) * W + cx, (cy + k) * W + cx};
#pragma unroll
    for (int q = 0; q < 4; ++q)
      if (p[q] == i && p[q] > 0 && p[q] < n) return true;
  }
  return false;
}

// FrameBuffer.Fog for one pixel (rasterizer.go:193-207) with blendRGBA
// (185-191): uint8(float32(a)*(1-f) + float32(b)*f) per channel.
__device__ __forceinline__ uint32_t fog_pixel(uint32_t c, float depth, float fog_start, float fog_end,
                                              uint32_t fog_color) {
  if (depth >= fog_start) return c;
  if (depth <= fog_end) return fog_color;
  const float f = fs(1.0f, fd(fs(fog_end, depth), fs(fog_end, fog_start)));
  const float g = fs(1.0f, f);
  uint32_t r = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float a = (float)((c >> (8 * k)) & 0xFFu), b = (float)((fog_color >> (8 * k)) & 0xFFu);
    r |= go_u8(fa(fm(a, g), fm(b, f))) << (8 * k);
  }
  return r;
}

__global__ void __launch_bounds__(256) k_fog(uint32_t* rgba, const float* z, long long n, float fog_start,
                                             float fog_end, uint32_t color) {
  for (long long i = blockIdx.x * 256ll + threadIdx.x; i < n; i += (long long)gridDim.x * 256)
    rgba[i] = fog_pixel(rgba[i], z[i], fog_start, fog_end, color);
}

int launch_fog(uint32_t* rgba, const float* z, long long pixels, float fog_start, float fog_end, uint32_t color,
               void* stream) {
  if (pixels <= 0) return 0;
  const long long blocks = std::min<long long>((pixels + 255) / 256, 152ll * 16);
  k_fog<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(rgba, z, pixels, fog_start, fog_end, color);
  return (int)cudaGetLastError();
}

// Edge values of record t at pixel (x, y).
__device__ __forceinline__ void edges_at(const TriRaster& t, const TriWide* wide, uint32_t r, int x, int y,
                                         bool& inside, float& e12f, float& e20f) {
  if (!(t.key & 0x80000000u)) {
    int e01 = t.a01 * x + t.b01 * y + t.c01;
    int e12 = t.a12 * x + t.b12 * y + t.c12;
    int e20 = t.a20 * x + t.b20 * y + t.c20;
    inside = e01 < 0 && e12 < 0 && e20 < 0;
    e12f = __int2float_rn(e12);
    e20f = __int2float_rn(e20);
  } else {
    typedef unsigned long long u64;
    const TriWide& w = wide[r];
    u64 X = (u64)(long long)x, Y = (u64)(long long)y;
    long long e01 = (long long)((u64)w.a01 * X + (u64)w.b01 * Y + (u64)w.c01);
    long long e12 = (long long)((u64)w.a12 * X + (u64)w.b12 * Y + (u64)w.c12);
    long long e20 = (long long)((u64)w.a20 * X + (u64)w.b20 * Y + (u64)w.c20);
    inside = e01 < 0 && e12 < 0 && e20 < 0;
    e12f = __ll2float_rn(e12);
    e20f = __ll2float_rn(e20);
  }
}

template <int TS>
struct RasterShape {
  static constexpr int kThreads = TS * TS / 4;  // 4 pixels per thread in the resolve
  static constexpr int kStride = TS + 8;        // padded key row: 8x4 warp blocks hit disjoint banks
  static constexpr int kWarps = kThreads / 32;
  static constexpr int kMinBlocks = 2048 / kThreads / 2;  // 32 warps per SM: 64 registers a thread
};

// Exact depth test of one covered pixel: zRec in the reference's order,
// then a 64-bit max of (ordered zRec, draw-order key) into the tile's keys.
//
// Early out: at a covered pixel the barycentrics are e/sum of adjusted edge
// values that are all negative, so they lie in [0, 1] (to rounding) and
// zRec = -(al/w0 + be/w1 + ga/w2) <= (1 / min|w|) * (1 + ~1e-6) when every w
// is negative (in front of the camera).  A candidate whose bound stays below
// the depth the pixel already holds, with a 1e-5 margin for the roundings,
// loses strictly (ties, where draw order decides, are never skipped), so its
// five divisions are not needed.
// The depth test proper at pixel p with edge values e12, e20 (as floats).
__device__ __forceinline__ void depth_at(unsigned long long* p, const TriRaster& t, float e12f, float e20f) {
  float al, be, ga;
  const float z = zrec_of(e12f, e20f, t.sumf, t.w0, t.w1, t.w2, al, be, ga);
  if (!(z >= -1.0f)) return;  // rasterizer.go:156 against the cleared Z of -1
  const unsigned long long k = depth_key(z, t.key);
  if (k > *(volatile unsigned long long*)p) atomicMax(p, k);
}

// True when the pixel at p already holds a depth that a candidate with
// vertex depths w0..w2 cannot reach (the early out above).
__device__ __forceinline__ bool depth_beaten(const unsigned long long* p, const TriRaster& t) {
  const uint32_t o = (uint32_t)(*(const volatile unsigned long long*)p >> 32);
  if (!(o & 0x80000000u)) return false;  // the pixel holds a depth < +0
  const float wmin = fminf(fminf(-t.w0, -t.w1), -t.w2);
  return wmin > 0.0f && __fmul_rn(__uint_as_float(o & 0x7FFFFFFFu), wmin) > 1.00001f;
}

template <int TS>
__device__ __forceinline__ void depth_candidate(unsigned long long* skey, const TriRaster& t, const TriWide* wide,
                                                uint32_t r, int x, int y, int tx0, int ty0) {
  unsigned long long* p = skey + (y - ty0) * RasterShape<TS>::kStride + (x - tx0);
  if (depth_beaten(p, t)) return;
  bool inside;
  float e12f, e20f;
  edges_at(t, wide, r, x, y, inside, e12f, e20f);
  depth_at(p, t, e12f, e20f);
}

// Depth test of a pixel known to be covered by narrow triangle t.
template <int TS>
__device__ __forceinline__ void depth_covered(unsigned long long* skey, const TriRaster& t, int x, int y, int tx0,
                                              int ty0) {
  unsigned long long* p = skey + (y - ty0) * RasterShape<TS>::kStride + (x - tx0);
  if (depth_beaten(p, t)) return;
  const int e12 = t.a12 * x + t.b12 * y + t.c12;
  const int e20 = t.a20 * x + t.b20 * y + t.c20;
  depth_at(p, t, __int2float_rn(e12), __int2float_rn(e20));
}

// floor(n / d) for d > 0, exact when the quotient lies in [lo - 1, hi + 1];
// otherwise a value on the same side of that range.  The float estimate is
// within one of the quotient (|n| < 2^31, d < 2^15: a few ulps of relative
// error, below 1 while |n / d| < 2^20; beyond that the clamp decides), and
// one exact integer step corrects it.
__device__ __forceinline__ int floor_div_near(int n, int d, int lo, int hi) {
  float q = floorf(__fdividef(__int2float_rn(n), __int2float_rn(d)));
  q = fminf(fmaxf(q, (float)(lo - 1)), (float)(hi + 1));
  int qi = (int)q;
  if (qi * d > n) --qi;
  else if ((qi + 1) * d <= n) ++qi;
  return qi;
}

// Narrows [xl, xr] on row y to the x where a*x + (b*y + c) < 0 (one edge of
// the inside test, rasterizer.go:147).  All products stay in int32 for
// narrow triangles (|a|, |b| < 2^15, |c| < 2^29, 0 <= x, y < 2^14).
__device__ __forceinline__ void span_edge(int a, int b, int c, int y, int& xl, int& xr) {
  const int k = b * y + c;
  const int n = a > 0 ? -k - 1 : k;  // a > 0: x <= floor((-k-1)/a); a < 0: x >= floor(k/-a) + 1
  const int q = floor_div_near(n, a > 0 ? a : max(-a, 1), xl, xr);
  if (a > 0) xr = min(xr, q);
  else if (a < 0) xl = max(xl, q + 1);
  else if (k >= 0) xr = xl - 1;      // a == 0: the whole row is outside this edge
}

// Last lane j with start[j] <= g (start non-decreasing across lanes, lane 0's
// start <= g); zero-length lanes share the next lane's start and are skipped.
__device__ __forceinline__ int owner_lane(int start, int g) {
  int own = 0;
#pragma unroll
  for (int step = 16; step > 0; step >>= 1) {
    const int cand = own + step;
    const int cs = __shfl_sync(FULL_MASK, start, cand & 31);
    if (cand < 32 && cs <= g) own = cand;
  }
  return own;
}

__device__ __forceinline__ int warp_incl_scan(int v) {
  const unsigned lane = threadIdx.x & 31u;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(FULL_MASK, v, o);
    if ((int)lane >= o) v += y;
  }
  return v;
}

// Coverage test of one pixel (rasterizer.go:147).
__device__ __forceinline__ bool covers(const TriRaster& t, const TriWide* wide, uint32_t r, int x, int y) {
  if (!(t.key & 0x80000000u)) {
    return t.a01 * x + t.b01 * y + t.c01 < 0 && t.a12 * x + t.b12 * y + t.c12 < 0 &&
           t.a20 * x + t.b20 * y + t.c20 < 0;
  }
  bool inside;
  float e12f, e20f;
  edges_at(t, wide, r, x, y, inside, e12f, e20f);
  return inside;
}

// Minimum of a narrow edge function over the pixel box [X0,X1] x [Y0,Y1].
__device__ __forceinline__ int edge_min(int a, int b, int c, int X0, int X1, int Y0, int Y1) {
  return c + min(a * X0, a * X1) + min(b * Y0, b * Y1);
}

// Per-warp queue of covered pixels awaiting the exact depth test, so that the
// division-heavy part runs with every lane busy.  Each entry names a slot of
// the warp's triangle table (records staged in shared memory, so a drain
// reads no global memory) and a pixel.  qn is warp-uniform; capacity 64: the
// warp drains 32 whenever qn >= 32.
template <int TS>
struct CandQueue {
  uint32_t* ent;        // slot | x << 8 | y << 20
  const TriRaster* tri; // the warp's triangle table (kSlots entries)
  const uint32_t* rec;  // record index per slot (for int64 edge coefficients)
  int qn;

  __device__ __forceinline__ void run(uint32_t e, unsigned long long* skey, const FrameArgs& a, int tx0, int ty0) {
    const uint32_t slot = e & 0xFFu;
    const TriRaster t = tri[slot];
    depth_candidate<TS>(skey, t, a.wide, rec[slot], tx0 + (int)((e >> 8) & 0xFFFu), ty0 + (int)(e >> 20), tx0,
                        ty0);
  }

  __device__ __forceinline__ void push(bool covered, uint32_t slot, int x, int y, unsigned long long* skey,
                                       const FrameArgs& a, int tx0, int ty0) {
    const unsigned lane = lane_id();
    const unsigned m = __ballot_sync(FULL_MASK, covered);
    if (covered) ent[qn + __popc(m & ((1u << lane) - 1u))] = slot | ((uint32_t)x << 8) | ((uint32_t)y << 20);
    qn += __popc(m);
    if (qn >= 32) {
      __syncwarp();
      run(ent[lane], skey, a, tx0, ty0);
      const int rest = qn - 32;
      uint32_t e = 0;
      if ((int)lane < rest) e = ent[32 + lane];
      __syncwarp();
      if ((int)lane < rest) ent[lane] = e;
      __syncwarp();
      qn = rest;
    }
  }

  __device__ __forceinline__ void flush(unsigned long long* skey, const FrameArgs& a, int tx0, int ty0) {
    const unsigned lane = lane_id();
    __syncwarp();
    if ((int)lane < qn) run(ent[lane], skey, a, tx0, ty0);
    __syncwarp();
    qn = 0;
  }
};


// Walks the 8x4 blocks j = j0, j0 + step, ... of the footprint [bx0,bx1] x
// [by0,by1] of the triangle in table slot `slot`, one pixel per lane.  Blocks
// that one edge excludes entirely are skipped before any per-pixel work;
// covered pixels go to the warp's queue.
template <int TS>
__device__ __forceinline__ void walk_blocks(CandQueue<TS>& q, unsigned long long* skey, const FrameArgs& a,
                                            const TriRaster& tt, uint32_t rr, uint32_t slot, int bx0, int bx1,
                                            int by0, int by1, int j0, int step, int tx0, int ty0) {
  const unsigned lane = lane_id();
  const bool narrow = !(tt.key & 0x80000000u);
  const int px = (int)(lane & 7u), py = (int)(lane >> 3);
  const int nbx = (bx1 - bx0 + 8) >> 3;
  const int nblk = nbx * ((by1 - by0 + 4) >> 2);
  for (int j = j0; j < nblk; j += step) {
    const int bj = j / nbx;
    const int x8 = bx0 + ((j - bj * nbx) << 3), y4 = by0 + (bj << 2);
    const int X1 = min(x8 + 7, bx1), Y1 = min(y4 + 3, by1);
    if (narrow && (edge_min(tt.a01, tt.b01, tt.c01, x8, X1, y4, Y1) >= 0 ||
                   edge_min(tt.a12, tt.b12, tt.c12, x8, X1, y4, Y1) >= 0 ||
                   edge_min(tt.a20, tt.b20, tt.c20, x8, X1, y4, Y1) >= 0))
      continue;
    const int x = x8 + px, y = y4 + py;
    const bool c = x <= X1 && y <= Y1 && covers(tt, a.wide, rr, x, y);
    q.push(c, slot, x - tx0, y - ty0, skey, a, tx0, ty0);
  }
}

// Number of raster slices of a tile holding n bin entries of estimated total
// cost `cost` (kEntryCost per entry plus the boxes of the large ones): about
// one slice per slice_cost, at most kRasterMaxSlices, at least 4 entries each.
__device__ __forceinline__ uint32_t tile_slices(const FrameArgs& a, uint32_t n, uint32_t cost) {
  const uint32_t by_cost = (uint32_t)(((unsigned long long)cost + a.slice_cost - 1) / a.slice_cost);
  return max(1u, min(min(by_cost, (uint32_t)kRasterMaxSlices), (n + 3u) / 4u));
}

template <int TS>
struct RasterSmem {
  static constexpr int kWarps = RasterShape<TS>::kWarps;
  static constexpr uint32_t kWideCap = 128;  // queued wide triangles per round
  static constexpr int kSlots = 64;           // triangle table: 32 lane slots + 32 for wide ones
  __align__(16) unsigned long long skey[TS * RasterShape<TS>::kStride];
  __align__(16) TriRaster tri[kWarps][kSlots];
  uint32_t trec[kWarps][kSlots];
  uint32_t ent[kWarps][64];
  uint32_t wideq[kWideCap + RasterShape<TS>::kThreads];
  uint32_t next, nwide, last;
};

// Final colour and depth of pixel (x, y) of view vw whose visibility key is k:
// deferred shading of the winning triangle (rasterizer.go:149-176), or Clear
// and DotGrid when no triangle won; then overlay marks, the crosshair and fog.
__device__ __forceinline__ void resolve_pixel(const FrameArgs& a, const DevView& vw, int x, int y,
                                              unsigned long long k, uint32_t& out_c, float& out_z) {
  const bool face_ids = vw.flags & kViewFaceIds;
  // overlay marks (k_overlay): the last mark in draw order, if any
  uint32_t ov = 0;
  if (vw.flags & 0xC0u) {
    uint32_t* op = a.ovl_key + vw.pix_base + (size_t)y * (size_t)vw.W + (size_t)x;
    ov = *op;
    if (ov) *op = 0u;  // ready for the next frame
  }
  // vertexColor (255,161,0,255); edgeColor black, or white without faces (renderer.go:17-19, 192-196)
  const uint32_t ovc = (ov & 1u) ? 0xFF00A1FFu : ((vw.flags & 0x02u) ? 0xFF000000u : 0xFFFFFFFFu);
  if (k == BG_KEY) {
    const bool dot = (x % 10 == 0) && (y % 10 == 0) && x >= 10 && y >= 10;  // DotGrid
    out_c = ov ? ovc : face_ids ? kNoFace : dot ? 0xFF646464u : 0xFF323232u;
    out_z = -1.0f;
  } else {
    const uint32_t okey = (uint32_t)k & 0x7FFFFFFFu;
    if (face_ids) {  // the face of order key face * 8 + fan + 1; no depth is output
      out_c = (okey - 1u) / (uint32_t)kKeysPerFace;
      out_z = 0.0f;
      return;
    }
    const uint32_t r = record_of_key(a, okey);
    const TriRaster t = unpack_tri(a, r, vw.W, vw.H);
    bool inside;
    float e12f, e20f, al, be, ga;
    edges_at(t, a.wide, r, x, y, inside, e12f, e20f);
    // The winner's zRec is the depth its key holds (the raster computed it
    // from the same record at this pixel): only the barycentrics are divided
    // out again.  A key depth of +0 may stand for -0, so that case takes the
    // full zRec.
    float z;
    if ((uint32_t)(k >> 32) != 0x80000000u) {
      al = fd(e12f, t.sumf);
      be = fd(e20f, t.sumf);
      ga = fs(fs(1.0f, al), be);
      z = key_depth(k);
    } else {
      z = zrec_of(e12f, e20f, t.sumf, t.w0, t.w1, t.w2, al, be, ga);
    }
    out_z = z;
    const TriShade s = a.shade[r];
    const float I = fa(fa(fm(al, s.i0), fm(be, s.i1)), fm(ga, s.i2));
    uint32_t c;
    if (s.tex >= 0) {
      const TriUV q = a.suv[r];
      const float u = fd(fa(fa(fm(al, q.u0w), fm(be, q.u1w)), fm(ga, q.u2w)), z);
      const float v = fd(fa(fa(fm(al, q.v0w), fm(be, q.v1w)), fm(ga, q.v2w)), z);
      c = color_intensity(tex_sample(a.texs[s.tex], u, v), I);
    } else if (s.tex == -2 || s.tex == -3) {
      float cc[9];
      if (s.tex == -2) {
        const TriColor& tc = a.tcol[r];
#pragma unroll
        for (int q = 0; q < 9; ++q) cc[q] = tc.c[q];
      } else {
        // a kept face: record r is kept face r, whose vertex colours are read
        // again through the kept list, the same floats k_setup saw (not
        // writing them as a record: the 5 M-face stress frame 0.403 -> 0.367 ms)
        const uint2 e = a.kept[r];
        const DevItem& it = a.items[e.x];
        const int* vi = it.vidx + 3 * (size_t)e.y;
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const float* cp = it.vcol + 3 * (size_t)__ldg(vi + k);
          cc[3 * k] = __ldg(cp); cc[3 * k + 1] = __ldg(cp + 1); cc[3 * k + 2] = __ldg(cp + 2);
        }
      }
      uint32_t ch[3];
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const float cq = fa(fa(fm(al, cc[q]), fm(be, cc[3 + q])), fm(ga, cc[6 + q]));
        ch[q] = go_u8(fm(fm(cq, 255.0f), I));
      }
      c = ch[0] | (ch[1] << 8) | (ch[2] << 16) | 0xFF000000u;
    } else {
      c = color_intensity(0xFFC8C8C8u, I);  // faceColor (200,200,200,255)
    }
    // a mark of the winner itself or of a later triangle lies on top of the fill
    out_c = (ov && (ov >> 1) >= okey) ? ovc : c;
  }
  if (face_ids) return;
  if ((vw.flags & 0x100u) && crosshair_hit(vw.W, vw.H, x, y)) out_c = 0xFF00FFFFu;  // (255,255,0,255)
  if (vw.fog_on) out_c = fog_pixel(out_c, out_z, vw.fog_start, vw.fog_end, vw.fog_color);
}

// One raster work item: slice `slice` of global tile `tile` of view `view`.
template <int TS>
__device__ __forceinline__ void raster_item(const FrameArgs& a, uint32_t tile, uint32_t slice, int view,
                                            RasterSmem<TS>& sm) {
  constexpr int kThreads = RasterShape<TS>::kThreads;
  constexpr int kStride = RasterShape<TS>::kStride;
  constexpr int kWarps = RasterShape<TS>::kWarps;
  constexpr uint32_t kWideCap = RasterSmem<TS>::kWideCap;
  unsigned long long* skey = sm.skey;
  auto& s_tri = sm.tri;
  auto& s_trec = sm.trec;
  auto& s_ent = sm.ent;
  uint32_t* s_wideq = sm.wideq;
  uint32_t& s_next = sm.next;
  uint32_t& s_nwide = sm.nwide;
  uint32_t& s_last = sm.last;
  const int tid = threadIdx.x;
  const int warp = tid >> 5;
  const DevView& vw = a.views[view];
  // A tile's bin is split into up to kRasterMaxSlices slices, one work item each.
  const uint4 ti = a.tile_info[tile];  // k_plan: entries, slices, key slot
  const uint32_t n = ti.x;
  const uint32_t nslices = ti.y;
  if (slice >= nslices) return;
  const uint32_t per = (((n + nslices - 1) / nslices) + 31u) & ~31u;
  const uint32_t lo = min(n, slice * per), hi = min(n, lo + per);
  const uint32_t lt = tile - vw.tile_base;
  const int tx0 = (int)(lt % (uint32_t)vw.tiles_x) * TS;
  const int ty0 = (int)(lt / (uint32_t)vw.tiles_x) * TS;
  const int tx1 = min(tx0 + TS - 1, vw.W - 1);
  const int ty1 = min(ty0 + TS - 1, vw.H - 1);

  // A tile with no bin entry is all background: with the resolve in this
  // kernel it needs no keys and goes straight to it (Clear + DotGrid,
  // overlays, crosshair, fog).  Measured: a 256-view batch 5 % faster; for
  // frames shaded by k_resolve the short cut did not pay (their empty tiles
  // still store background keys the ordinary way).
  const bool empty = n == 0 && !a.pkey;
  if (!empty) {
    for (int i = tid; i < TS * kStride; i += kThreads) skey[i] = BG_KEY;
    if (tid == 0) {
      s_next = lo;
      s_nwide = 0;
    }
    __syncthreads();

    const unsigned lane = lane_id();
    const uint32_t* bin = a.bins + (size_t)tile * a.bin_cap;
    TriRaster* tri = s_tri[warp];
    uint32_t* trec = s_trec[warp];
    CandQueue<TS> q{s_ent[warp], tri, trec, 0};
    // Entries per warp chunk: small bins use shorter chunks so that every warp
    // gets some (the span walk below keeps all lanes busy either way).
    const uint32_t chunk = min(32u, max(8u, (hi - lo + 2u * kWarps - 1u) / (2u * kWarps)));
    for (;;) {
      // Phase 1: warps take `chunk` bin entries at a time from a shared cursor.
      // Narrow triangles are walked by the warp that took them (span walk
      // below); int64 ("wide") triangles are queued for the whole CTA.
      for (;;) {
        if (*(volatile uint32_t*)&s_nwide >= kWideCap) break;
        uint32_t b = 0;
        if (lane == 0) b = atomicAdd(&s_next, chunk);
        b = __shfl_sync(FULL_MASK, b, 0);
        if (b >= hi) break;
        const uint32_t i = b + lane;
        const bool valid = lane < chunk && i < hi;
        uint32_t r = 0;
        int lx0 = 0, lx1 = -1, ly0 = 0, ly1 = -1;
        TriRaster t;
        if (valid) {
          r = bin[i];
          t = unpack_tri(a, r, vw.W, vw.H);
          lx0 = max((int)t.bx0, tx0); lx1 = min((int)t.bx1, tx1);
          ly0 = max((int)t.by0, ty0); ly1 = min((int)t.by1, ty1);
        }
        const bool live = valid && lx1 >= lx0 && ly1 >= ly0;
        const int area = live ? (lx1 - lx0 + 1) * (ly1 - ly0 + 1) : 0;
        const bool by_lane = live && !(t.key & 0x80000000u);
        const bool wide = live && !by_lane;
        const unsigned lm = __ballot_sync(FULL_MASK, wide);
        if (lm) {
          uint32_t qb = 0;
          const int ldr = __ffs(lm) - 1;
          if ((int)lane == ldr) qb = atomicAdd(&s_nwide, (uint32_t)__popc(lm));
          qb = __shfl_sync(FULL_MASK, qb, ldr);
          if (wide) s_wideq[qb + __popc(lm & ((1u << lane) - 1u))] = r;
        }
        if (by_lane) {
          tri[lane] = t;
          trec[lane] = r;
        }
        // Span walk.  The chunk's (triangle, footprint row) pairs are numbered
        // consecutively (a warp scan of the row counts), 32 rows per step; each
        // lane narrows its row to the exact covered x-range, and the covered
        // pixels of the 32 spans are numbered again and depth-tested 32 at a
        // time, so no lane tests a pixel that the triangle does not cover.
        // Chunks of tiny footprints take the per-lane box walk instead.
        const int my = by_lane ? ly1 - ly0 + 1 : 0;
        const int incl = warp_incl_scan(my);
        const int excl = incl - my;
        const int total = __shfl_sync(FULL_MASK, incl, 31);
        const int widest = __reduce_max_sync(FULL_MASK, by_lane ? area : 0);
        __syncwarp();
        if (widest * 5 <= ((total + 31) >> 5) * 27) {
          // Footprints of a few pixels: a span costs about five box-pixel tests,
          // so each lane tests its own box, queueing covered pixels.
          int x = lx0, y = ly0;
          for (int it = 0; it < widest; ++it) {
            const bool c = by_lane && it < area && t.a01 * x + t.b01 * y + t.c01 < 0 &&
                           t.a12 * x + t.b12 * y + t.c12 < 0 && t.a20 * x + t.b20 * y + t.c20 < 0;
            q.push(c, lane, x - tx0, y - ty0, skey, a, tx0, ty0);
            if (++x > lx1) {
              x = lx0;
              ++y;
            }
          }
          q.flush(skey, a, tx0, ty0);
          continue;
        }
        for (int g0 = 0; g0 < total; g0 += 32) {
          const int g = g0 + (int)lane;
          const int own = owner_lane(excl, g);
          const int y = __shfl_sync(FULL_MASK, ly0, own) + g - __shfl_sync(FULL_MASK, excl, own);
          int xl = __shfl_sync(FULL_MASK, lx0, own), xr = __shfl_sync(FULL_MASK, lx1, own);
          if (g < total) {
            const TriRaster& tt = tri[own];
            span_edge(tt.a01, tt.b01, tt.c01, y, xl, xr);
            span_edge(tt.a12, tt.b12, tt.c12, y, xl, xr);
            span_edge(tt.a20, tt.b20, tt.c20, y, xl, xr);
          } else {
            xr = xl - 1;
          }
          const int len = max(xr - xl + 1, 0);
          const int incl2 = warp_incl_scan(len);
          const int excl2 = incl2 - len;
          const int total2 = __shfl_sync(FULL_MASK, incl2, 31);
          // two pixels a lane per pass: their depth tests are independent
          // chains of divisions that overlap
          for (int h0 = 0; h0 < total2; h0 += 64) {
            const int ha = h0 + (int)lane, hb = ha + 32;
            const int oa = owner_lane(excl2, ha), ob = owner_lane(excl2, hb);
            const int xa = __shfl_sync(FULL_MASK, xl, oa) + ha - __shfl_sync(FULL_MASK, excl2, oa);
            const int xb = __shfl_sync(FULL_MASK, xl, ob) + hb - __shfl_sync(FULL_MASK, excl2, ob);
            const int ya = __shfl_sync(FULL_MASK, y, oa), yb = __shfl_sync(FULL_MASK, y, ob);
            const int sa = __shfl_sync(FULL_MASK, own, oa), sb = __shfl_sync(FULL_MASK, own, ob);
            if (ha < total2) depth_covered<TS>(skey, tri[sa], xa, ya, tx0, ty0);
            if (hb < total2) depth_covered<TS>(skey, tri[sb], xb, yb, tx0, ty0);
          }
        }
        __syncwarp();  // lane slots are rewritten by the next chunk
      }
      __syncthreads();
      const uint32_t nl = s_nwide;
      const bool more = s_next < hi;
      // Phase 2: every warp walks the queued wide triangles and takes an
      // interleaved share of their 8x4 blocks (global block index mod warps).
      int base = 0;
      for (uint32_t k = 0; k < nl; ++k) {
        const uint32_t slot = 32u + (k & 31u);
        if ((k & 31u) == 0) {
          // slots 32..63 are about to be reused: drain, then stage the next 32
          // wide records with one load per lane
          q.flush(skey, a, tx0, ty0);
          if (k + lane < nl) {
            const uint32_t r2 = s_wideq[k + lane];
            tri[32 + lane] = unpack_tri(a, r2, vw.W, vw.H);
            trec[32 + lane] = r2;
          }
          __syncwarp();
        }
        const TriRaster tt = tri[slot];
        const uint32_t rr = trec[slot];
        const int bx0 = max((int)tt.bx0, tx0), bx1 = min((int)tt.bx1, tx1);
        const int by0 = max((int)tt.by0, ty0), by1 = min((int)tt.by1, ty1);
        const int nblk = ((bx1 - bx0 + 8) >> 3) * ((by1 - by0 + 4) >> 2);
        const int j0 = (warp - base + kWarps) % kWarps;
        walk_blocks<TS>(q, skey, a, tt, rr, slot, bx0, bx1, by0, by1, j0, kWarps, tx0, ty0);
        base = (base + nblk) % kWarps;
      }
      q.flush(skey, a, tx0, ty0);
      __syncthreads();
      if (!more) break;
      if (tid == 0) s_nwide = 0;
      __syncthreads();
    }

    if (nslices > 1 && ti.z != kNoSlot) {
      // One view: this slice's keys go to a slot of their own with plain
      // stores, and k_resolve takes the max over the tile's slots -- the
      // kernel boundary orders them, so no slice waits on a fence or hands
      // over (the merge below took a fifth of this kernel's warp time on
      // single frames).
      unsigned long long* dst = a.slot_keys + (size_t)(ti.z + slice) * (TS * TS);
      for (int i = tid; i < TS * TS; i += kThreads) dst[i] = skey[(i / TS) * kStride + (i % TS)];
      return;
    }
    if (nslices > 1) {
      // Merge this slice's keys into the tile's global keys; the last slice to
      // arrive resolves the tile and returns the global keys to zero (zero is
      // below every key, since no key encodes a NaN depth).
      unsigned long long* g = a.gkey + (size_t)tile * (TS * TS);
      for (int i = tid; i < TS * TS; i += kThreads) {
        const unsigned long long k = skey[(i / TS) * kStride + (i % TS)];
        if (k != BG_KEY) atomicMax(g + i, k);
      }
      __threadfence();
      __syncthreads();
      if (tid == 0) s_last = atomicAdd(&a.tile_done[tile], 1u) == nslices - 1 ? 1u : 0u;
      __syncthreads();
      if (!s_last) return;
      __threadfence();
      for (int i = tid; i < TS * TS; i += kThreads) {
        const unsigned long long k = *(volatile unsigned long long*)(g + i);
        skey[(i / TS) * kStride + (i % TS)] = k > BG_KEY ? k : BG_KEY;
        g[i] = 0ull;
      }
      if (tid == 0) a.tile_done[tile] = 0u;
      __syncthreads();
    }
  }

  if (a.pkey) {
    // the tile's final keys, shaded by k_resolve
    for (int i = tid; i < TS * TS; i += kThreads) {
      const int rr = i / TS, cc = i % TS;
      const int x = tx0 + cc, y = ty0 + rr;
      if (x <= tx1 && y <= ty1)
        a.pkey[vw.pix_base + (size_t)y * (size_t)vw.W + (size_t)x] = empty ? BG_KEY : skey[rr * kStride + cc];
    }
  } else {
    // Resolve + deferred shading, four pixels a thread
    constexpr int kPerRow = TS / 4;
    const int row = tid / kPerRow;
    const int col = (tid % kPerRow) * 4;
    const int y = ty0 + row;
    if (y <= ty1) {
      uint32_t out_c[4];
      float out_z[4];
      unsigned long long keys[4] = {BG_KEY, BG_KEY, BG_KEY, BG_KEY};
      if (!empty) {
        const ulonglong2* kp = reinterpret_cast<const ulonglong2*>(skey + row * kStride + col);
        const ulonglong2 k01 = kp[0], k23 = kp[1];
        keys[0] = k01.x; keys[1] = k01.y; keys[2] = k23.x; keys[3] = k23.y;
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        out_c[j] = 0u;
        out_z[j] = 0.0f;
        if (tx0 + col + j <= tx1) resolve_pixel(a, vw, tx0 + col + j, y, keys[j], out_c[j], out_z[j]);
      }
      const int x = tx0 + col;
      const size_t o = (size_t)y * (size_t)vw.W + (size_t)x;
      const bool with_z = !(vw.flags & kViewFaceIds);  // face-id views output no depth
      if (vw.vec_ok && x + 3 <= tx1) {
        *reinterpret_cast<uint4*>(vw.out_rgba + o) = make_uint4(out_c[0], out_c[1], out_c[2], out_c[3]);
        if (with_z) *reinterpret_cast<float4*>(vw.out_z + o) = make_float4(out_z[0], out_z[1], out_z[2], out_z[3]);
      } else {
        for (int j = 0; j < 4 && x + j <= tx1; ++j) {
          vw.out_rgba[o + j] = out_c[j];
          if (with_z) vw.out_z[o + j] = out_z[j];
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// k_overlay: the marks of ShowEdges / ShowVertices (renderer.go:191-216).
// They are not depth-tested and overwrite whatever was drawn before them, so
// a pixel shows the last mark in draw order unless a later triangle's fill
// (which is necessarily the depth winner: the last fill at a pixel always
// is) covers it.  Each mark records max(order key * 2 + vertex mark) per
// pixel; the raster resolve compares it with the winner's key.  One thread
// per binned triangle: a line's pixels depend on float32 steps accumulated
// one add at a time (FrameBuffer.Line), so each line runs sequentially.
// ---------------------------------------------------------------------------
__device__ __forceinline__ long long go_abs(long long v) {  // utils.go abs: MinInt -> MaxInt
  if (v < 0) v = (long long)(0ull - (unsigned long long)v);
  if (v < 0) v = (long long)((unsigned long long)v - 1ull);
  return v;
}

// FrameBuffer.Pixel (rasterizer.go:25-30): the linear index decides (an x
// outside the row wraps into the next), index 0 is never written.
__device__ __forceinline__ void ovl_plot(const FrameArgs& a, const DevView& vw, long long x, long long y,
                                         uint32_t val) {
  typedef unsigned long long u64;
  const long long idx = (long long)((u64)y * (u64)(long long)vw.W + (u64)x);
  if (idx > 0 && idx < (long long)vw.W * (long long)vw.H) atomicMax(a.ovl_key + vw.pix_base + (u64)idx, val);
}

// FrameBuffer.Line (rasterizer.go:65-79)
__device__ void ovl_line(const FrameArgs& a, const DevView& vw, long long x0, long long y0, long long x1,
                         long long y1, uint32_t val) {
  typedef unsigned long long u64;
  const long long dx = (long long)((u64)x1 - (u64)x0), dy = (long long)((u64)y1 - (u64)y0);
  const long long side = max(go_abs(dx), go_abs(dy));
  if (side > kMaxLineSteps) {
    atomicOr(&a.work->error, 4u);
    return;
  }
  const float xs = fd(__ll2float_rn(dx), __ll2float_rn(side)), ys = fd(__ll2float_rn(dy), __ll2float_rn(side));
  float cx = __ll2float_rn(x0), cy = __ll2float_rn(y0);
  for (long long i = 0; i <= side; ++i) {
    ovl_plot(a, vw, go_int(cx), go_int(cy), val);
    cx = fa(cx, xs);
    cy = fa(cy, ys);
  }
}

// FrameBuffer.Rect (rasterizer.go:54-63), 3 x 3
__device__ __forceinline__ void ovl_rect3(const FrameArgs& a, const DevView& vw, long long x, long long y,
                                          uint32_t val) {
  if (x >= (long long)vw.W || y >= (long long)vw.H) return;
  for (int py = 0; py < 3; ++py)
    for (int px = 0; px < 3; ++px) ovl_plot(a, vw, x + px, y + py, val);
}

__global__ void __launch_bounds__(256) k_overlay(const FrameArgs a) {
  griddep_wait();
  const uint32_t n = min(*(volatile uint32_t*)&a.work->novl, a.ovl_cap);
  for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const Overlay o = a.ovl[q];
    const DevView& vw = a.views[o.view];
    const uint32_t fl = vw.flags;
    const uint32_t edge = o.key * 2u, vert = o.key * 2u + 1u;  // vertex marks come after the edges
    if (fl & 0x40u) {
      ovl_line(a, vw, o.X[0], o.Y[0], o.X[1], o.Y[1], edge);
      ovl_line(a, vw, o.X[1], o.Y[1], o.X[2], o.Y[2], edge);
      ovl_line(a, vw, o.X[2], o.Y[2], o.X[0], o.Y[0], edge);
      if (fl & 0x02u) {
        const float cx = fd(fa(fa(o.sx[0], o.sx[1]), o.sx[2]), 3.0f);
        const float cy = fd(fa(fa(o.sy[0], o.sy[1]), o.sy[2]), 3.0f);
        ovl_rect3(a, vw, (long long)((unsigned long long)go_int(cx) - 1ull),
                  (long long)((unsigned long long)go_int(cy) - 1ull), edge);
      }
    }
    if (fl & 0x80u)
      for (int j = 0; j < 3; ++j)
        ovl_rect3(a, vw, (long long)((unsigned long long)o.X[j] - 1ull), (long long)((unsigned long long)o.Y[j] - 1ull),
                  vert);
  }
}

// ---------------------------------------------------------------------------
// k_plan: the raster work queue.  One thread per global tile.  A tile's
// estimated cost (kEntryCost per bin entry plus the tile-clipped boxes of its
// large triangles) decides its number of slices (about one per slice_cost);
// split tiles and tiles worth at least half a slice go to the front of the
// queue (heavy work starts first), the rest to the back.  One atomic per CTA
// reserves each part; no ordering between CTAs is needed.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_plan(const FrameArgs a) {
  griddep_wait();
  __shared__ uint32_t s_nf, s_nb, s_ne, s_bf, s_bb, s_be, s_max;
  const uint32_t tile = blockIdx.x * 256u + threadIdx.x;
  if (threadIdx.x == 0) {
    s_nf = 0;
    s_nb = 0;
    s_ne = 0;
    s_max = 0;
  }
  __syncthreads();
  const bool valid = tile < a.total_tiles;
  const uint32_t count = valid ? a.bin_count[tile] : 0u;
  const uint32_t cost = valid ? count * (uint32_t)kEntryCost + a.tile_cost[tile] : 0u;
  const uint32_t ns = valid ? tile_slices(a, min(count, a.bin_cap), cost) : 0u;
  if (valid) {  // the bins are complete: ready for the next frame's appends
    a.bin_count[tile] = 0u;
    a.tile_cost[tile] = 0u;
  }
  // the tile's view (last view whose first tile <= tile), packed into the
  // work item beside the slice so the raster CTAs do not search for it
  int view = 0;
  if (valid) {
    int hi = a.num_views - 1;
    while (view < hi) {
      const int mid = (view + hi + 1) >> 1;
      if (a.views[mid].tile_base <= tile) view = mid; else hi = mid - 1;
    }
  }
  const uint32_t vbits = (uint32_t)view << 5;  // slices < kRasterMaxSlices = 32
  // heavy items (split tiles, or whole tiles worth half a slice) go to the
  // front of the queue so that they start first; the rest to the back
  const bool heavy = ns > 1 || cost >= a.slice_cost / 2u;
  // A tile without bin entries of a batch shaded in place goes to the list
  // of tiles to clear instead of the raster queue: all background, no keys.
  const bool clear = count == 0 && a.clear_empty;
  uint32_t mf = 0, mb = 0, me = 0;
  if (valid) {
    atomicMax(&s_max, count);
    if (clear) me = atomicAdd(&s_ne, 1u);
    else if (heavy) mf = atomicAdd(&s_nf, ns);
    else mb = atomicAdd(&s_nb, 1u);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    s_bf = s_nf ? atomicAdd(&a.work->plan_front, s_nf) : 0u;
    s_bb = s_nb ? atomicAdd(&a.work->plan_back, s_nb) : 0u;
    s_be = s_ne ? atomicAdd(&a.work->nempty, s_ne) : 0u;
    if (s_max) atomicMax(&a.work->max_bin, s_max);
  }
  __syncthreads();
  if (!valid) return;
  // A split tile of a one-view frame into at most 8 slices: its slices' keys
  // in the slots of its plan items (the front of the queue), while they fit.
  // k_resolve then reads a key per slice for each of the tile's pixels;
  // beyond 8 slices that cost more than the merge (same-box A/B: heightfield
  // 0.1227 -> 0.1183 ms with the cap, the 5 M-face frame unchanged; without
  // it the latter 1 % slower).
  const uint32_t slot =
      heavy && ns > 1 && ns <= 8u && a.slot_keys && s_bf + mf + ns <= a.slot_cap ? s_bf + mf : kNoSlot;
  a.tile_info[tile] = make_uint4(min(count, a.bin_cap), ns, slot, 0u);
  if (clear) {
    if (s_be + me < a.empty_cap) a.empty_tiles[s_be + me] = make_uint2(tile, (uint32_t)view);
  } else if (heavy) {
    for (uint32_t k = 0; k < ns; ++k) a.plan[s_bf + mf + k] = make_uint2(tile, k | vbits);
  } else {
    a.plan[a.plan_cap - 1u - (s_bb + mb)] = make_uint2(tile, vbits);
  }
}

template <int TS>
__device__ __forceinline__ void clear_quad(const FrameArgs& a, uint2 e, uint32_t qq);

// Persistent raster: CTAs take work items from the queue until it is empty;
// the last CTA to finish publishes and resets the frame's counters.  CLEAR:
// the frame's tiles without bin entries are cleared here too (batches shaded
// in place; a separate instantiation, so the other frames' raster keeps its
// registers free of the clear loop).
template <int TS, bool CLEAR>
__global__ void __launch_bounds__(RasterShape<TS>::kThreads, RasterShape<TS>::kMinBlocks) k_raster(const FrameArgs a) {
  griddep_wait();
  __shared__ RasterSmem<TS> sm;
  __shared__ uint32_t s_item, s_tile, s_slice, s_lastcta, s_clear;
  __shared__ int s_view;
  const uint32_t front = *(volatile uint32_t*)&a.work->plan_front;
  const uint32_t total = front + *(volatile uint32_t*)&a.work->plan_back;
  // The first item of every CTA is its block index; later ones come from the
  // counter, past the grid (no burst of atomics on one address at the start).
  for (bool first = true;; first = false) {
    if (threadIdx.x == 0) {
      const uint32_t i = first ? blockIdx.x : gridDim.x + atomicAdd(&a.work->raster_next, 1u);
      s_item = i;
      if (i < total) {
        const uint2 w = i < front ? a.plan[i] : a.plan[a.plan_cap - 1u - (i - front)];
        s_tile = w.x;
        s_slice = w.y & 31u;       // slice (kRasterMaxSlices = 32)
        s_view = (int)(w.y >> 5);  // view, found by k_plan
      }
    }
    __syncthreads();
    if (s_item >= total) break;
    raster_item<TS>(a, s_tile, s_slice, s_view, sm);
    __syncthreads();  // shared memory is reused by the next item
  }
  // Tiles without bin entries (batches shaded in place, k_plan's list): once
  // the raster queue is empty, the CTAs clear them, kClearGrab tiles a grab,
  // one four-pixel group a thread a tile (TS x TS / 4 = the CTA's threads).
  // Their stores fill the raster's tail instead of a kernel of their own,
  // which could not share an SM with this one (its registers fill the SM).
  if constexpr (CLEAR) {
    constexpr uint32_t kClearGrab = 8;
    const uint32_t ne = min(*(volatile uint32_t*)&a.work->nempty, a.empty_cap);
    // s_clear, not s_item: a warp may still be reading s_item for the loop above
    if (threadIdx.x == 0) s_clear = atomicAdd(&a.work->clear_next, kClearGrab);
    __syncthreads();
    for (;;) {
      const uint32_t e0 = s_clear;
      __syncthreads();  // every thread has read this grab
      if (e0 >= ne) break;
      // the next grab's atomic is in flight while these tiles are cleared
      if (threadIdx.x == 0) s_clear = atomicAdd(&a.work->clear_next, kClearGrab);
      for (uint32_t e = e0; e < min(ne, e0 + kClearGrab); ++e) clear_quad<TS>(a, a.empty_tiles[e], threadIdx.x);
      __syncthreads();  // the next grab is in s_clear
    }
  }
  if (threadIdx.x == 0) {
    // outputs in host memory (a synchronous draw): this CTA's writes become
    // visible to the host before it counts itself done
    if (a.result_host) __threadfence_system();
    else __threadfence();
    s_lastcta = atomicAdd(&a.work->raster_exit, 1u) == gridDim.x - 1 ? 1u : 0u;
  }
  __syncthreads();
  if (!s_lastcta) return;
  __threadfence();
  if (threadIdx.x == 0) {
    DevWork* w = a.work;
    DevResult* r = a.result;
    r->tpf = 0;
    r->nrec = w->nkept + w->nrec;
    r->nbig = w->nbig;
    r->bin_need = w->bin_need;
    r->rec_need = w->rec_need;
    r->big_need = w->big_need;
    r->error = w->error;
    r->nclip = w->nclip;
    r->clip_need = w->clip_need;
    r->max_bin = w->max_bin;
    r->items = total;
    r->novl = w->novl;
    r->ovl_need = w->ovl_need;
    w->novl = 0; w->ovl_need = 0;
    w->tpf = 0; w->nrec = 0; w->nbig = 0; w->bin_need = 0; w->rec_need = 0; w->big_need = 0; w->error = 0;
    w->nclip = 0; w->clip_need = 0; w->max_bin = 0; w->nkept = 0;
    w->plan_front = 0; w->plan_back = 0; w->raster_next = 0; w->raster_exit = 0;
    w->nempty = 0; w->clear_next = 0;
  }
  __syncthreads();
  for (int v = threadIdx.x; v < a.num_views; v += blockDim.x) {
    const unsigned long long t = a.view_tpf[v];
    a.view_tpf_out[v] = t;
    a.view_tpf[v] = 0ull;
    if (t) atomicAdd(&a.result->tpf, t);
  }
  if (a.result_host) {  // the finished counters straight into page-locked host memory
    __syncthreads();
    constexpr int kWords = (int)(sizeof(DevResult) / sizeof(unsigned));
    if (threadIdx.x < kWords)
      reinterpret_cast<unsigned*>(a.result_host)[threadIdx.x] =
          __ldcg(reinterpret_cast<const unsigned*>(a.result) + threadIdx.x);
    __syncthreads();
    if (threadIdx.x == 0) {  // the frame is complete: counters and every output are visible to the host
      __threadfence_system();
      reinterpret_cast<volatile unsigned*>(a.result_host)[kWords] = 1u;
    }
  }
}

// ---------------------------------------------------------------------------
// k_resolve: one thread per pixel of every view; shades the winners whose
// keys k_raster stored (the shading of resolve_pixel, at full occupancy so
// that its chain of dependent loads overlaps across many warps).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_resolve(const FrameArgs a) {
  griddep_wait();
  const unsigned long long p = (unsigned long long)blockIdx.x * 256u + threadIdx.x;
  if (p >= a.total_pixels) return;
  int v = 0;
  if (a.num_views > 1) {  // last view whose first pixel <= p
    int hi = a.num_views - 1;
    while (v < hi) {
      const int mid = (v + hi + 1) >> 1;
      if (a.views[mid].pix_base <= p) v = mid; else hi = mid - 1;
    }
  }
  const DevView& vw = a.views[v];
  const uint32_t o = (uint32_t)(p - vw.pix_base);
  const int y = (int)(o / (uint32_t)vw.W), x = (int)(o - (uint32_t)y * (uint32_t)vw.W);
  // The pixel's key is loaded beside its tile's info rather than after it (a
  // split tile, keyed in slots, ignores it): one dependent load less a pixel.
  unsigned long long k = a.pkey[p];
  const int sh = a.tile_shift, ts = 1 << sh;
  const uint4 ti = a.tile_info[vw.tile_base + (uint32_t)(y >> sh) * (uint32_t)vw.tiles_x + (uint32_t)(x >> sh)];
  if (ti.y > 1 && ti.z != kNoSlot) {  // a split tile: the max over its slices' slots
    const unsigned long long* sk = a.slot_keys + (size_t)ti.z * (size_t)(ts * ts) + (size_t)((y & (ts - 1)) * ts + (x & (ts - 1)));
    k = sk[0];
    for (uint32_t s = 1; s < ti.y; ++s) k = max(k, sk[(size_t)s * (size_t)(ts * ts)]);
  }
  uint32_t c;
  float z;
  resolve_pixel(a, vw, x, y, k, c, z);
  vw.out_rgba[o] = c;
  if (!(vw.flags & kViewFaceIds)) vw.out_z[o] = z;  // face-id views output no depth
}

// ---------------------------------------------------------------------------
// Tiles without bin entries of frames shaded in place (k_plan's list), which
// k_raster<TS, true> clears once its queue is empty.
// ---------------------------------------------------------------------------
// Four-pixel group qq of tile e (tile, view) without bin entries: Clear and
// DotGrid (rasterizer.go:36-52), overlay marks, crosshair and fog through
// resolve_pixel with the background key.
template <int TS>
__device__ __forceinline__ void clear_quad(const FrameArgs& a, uint2 e, uint32_t qq) {
  {
    const DevView& vw = a.views[e.y];
    const uint32_t lt = e.x - vw.tile_base;
    const int x = (int)(lt % (uint32_t)vw.tiles_x) * TS + (int)(qq % (TS / 4)) * 4;
    const int y = (int)(lt / (uint32_t)vw.tiles_x) * TS + (int)(qq / (TS / 4));
    if (y >= vw.H) return;
    uint32_t c[4];
    float z[4];
    if (!(vw.flags & (0xC0u | 0x100u | kViewFaceIds)) && !vw.fog_on) {
      // plain background: Clear, and DotGrid at x, y multiples of 10 from 10
      // on (the same values resolve_pixel gives with these flags)
      const bool dot_row = y >= 10 && y % 10 == 0;
      const int xr = x % 10;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const bool dot = dot_row && x + j >= 10 && (xr + j == 0 || xr + j == 10);
        c[j] = dot ? 0xFF646464u : 0xFF323232u;
        z[j] = -1.0f;
      }
    } else {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        c[j] = 0u;
        z[j] = 0.0f;
        if (x + j < vw.W) resolve_pixel(a, vw, x + j, y, BG_KEY, c[j], z[j]);
      }
    }
    const size_t o = (size_t)y * (size_t)vw.W + (size_t)x;
    const bool with_z = !(vw.flags & kViewFaceIds);  // face-id views output no depth
    if (vw.vec_ok && x + 3 < vw.W) {
      *reinterpret_cast<uint4*>(vw.out_rgba + o) = make_uint4(c[0], c[1], c[2], c[3]);
      if (with_z) *reinterpret_cast<float4*>(vw.out_z + o) = make_float4(z[0], z[1], z[2], z[3]);
    } else {
      for (int j = 0; j < 4 && x + j < vw.W; ++j) {
        vw.out_rgba[o + j] = c[j];
        if (with_z) vw.out_z[o + j] = z[j];
      }
    }
  }
}

// k_stage: a draw's tables from their page-locked staging slot (read through
// its device address, uncached: the host rewrites the slot between frames)
// into the device tables, as the first kernel of the frame, so the frame's
// kernels follow a kernel on their stream instead of a copy-engine transfer.
// One 16-byte word a thread, so the reads that cross to host memory are all
// in flight at once (a 64-item table is 23.5 KB); the thread after the last
// whole word copies the remaining bytes one by one.
__global__ void __launch_bounds__(128) k_stage(uint4* __restrict__ dst, const uint4* __restrict__ src, uint32_t n16,
                                               uint32_t tail) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n16) {
    dst[i] = __ldcv(src + i);
  } else if (i == n16) {
    const unsigned char* s = reinterpret_cast<const unsigned char*>(src + n16);
    unsigned char* d = reinterpret_cast<unsigned char*>(dst + n16);
    for (uint32_t k = 0; k < tail; ++k) d[k] = __ldcv(s + k);
  }
}

int launch_stage(void* dst, const void* src, size_t bytes, void* stream) {
  const uint32_t n16 = (uint32_t)(bytes / 16), tail = (uint32_t)(bytes % 16);
  const uint32_t threads = n16 + (tail ? 1u : 0u);
  if (!threads) return 0;
  k_stage<<<(threads + 127) / 128, 128, 0, (cudaStream_t)stream>>>((uint4*)dst, (const uint4*)src, n16, tail);
  return (int)cudaGetLastError();
}

int raster_grid(int tile_shift, int waves) {
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (tile_shift == 4)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_raster<16, false>, RasterShape<16>::kThreads, 0);
  else
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_raster<32, false>, RasterShape<32>::kThreads, 0);
  return max(1, sms) * max(1, per) * max(1, waves);
}

// Launches kern<<<grid, block, 0, s>>>(a), after a kernel on the same stream
// with programmatic stream serialization (the kernel waits in griddep_wait).
template <typename K>
static void launch_after(K kern, unsigned grid, unsigned block, cudaStream_t s, const FrameArgs& a) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kern, a);
}

int launch_frame(const FrameArgs& a, int big_blocks, void* stream, int* launches, void* const* events,
                 const AuxStream* aux) {
  cudaStream_t s = (cudaStream_t)stream;
  // Independent kernels go on two branches when an auxiliary stream is given
  // (inside a capture the branches become parallel graph nodes): k_light
  // beside k_vertex, k_clip beside k_bin_big.
  cudaStream_t s2 = aux ? (cudaStream_t)aux->stream : s;
  auto fork = [&](int k) {
    if (!aux) return;
    cudaEventRecord((cudaEvent_t)aux->fork[k], s);
    cudaStreamWaitEvent(s2, (cudaEvent_t)aux->fork[k], 0);
  };
  auto join = [&](int k) {
    if (!aux) return;
    cudaEventRecord((cudaEvent_t)aux->join[k], s2);
    cudaStreamWaitEvent(s, (cudaEvent_t)aux->join[k], 0);
  };
  int n = 0;
  if (events) cudaEventRecord((cudaEvent_t)events[0], s);
  if (a.total_blocks > 0) {
    const bool light = a.light_blocks > 0;
    if (light) {
      fork(0);
      if (a.project_g == 4) k_light<4><<<a.light_blocks, 256, 0, s2>>>(a);
      else if (a.project_g == 2) k_light<2><<<a.light_blocks, 256, 0, s2>>>(a);
      else k_light<1><<<a.light_blocks, 256, 0, s2>>>(a);
      ++n;
    }
    if (a.project_g == 4) launch_after(k_vertex<4>, a.vert_blocks, 256, s, a);
    else if (a.project_g == 2) launch_after(k_vertex<2>, a.vert_blocks, 256, s, a);
    else launch_after(k_vertex<1>, a.vert_blocks, 256, s, a);
    ++n;
    if (light) join(0);
    if (a.project_g == 4) launch_after(k_cull<4>, a.total_blocks, kProjectThreads, s, a);
    else if (a.project_g == 2) launch_after(k_cull<2>, a.total_blocks, kProjectThreads, s, a);
    else launch_after(k_cull<1>, a.total_blocks, kProjectThreads, s, a);
    ++n;
    const bool clip = a.flags_any & 0x01u;
    if (clip) {  // needs only k_cull's queue: runs beside k_setup and k_bin_big
      fork(1);
      k_clip<<<kClipBlocks, 128, 0, s2>>>(a);
      ++n;
    }
    if (setup_ctas_per_sm(a.project_g) == 3) launch_after(k_setup<3>, a.setup_blocks, kProjectThreads, s, a);
    else launch_after(k_setup<2>, a.setup_blocks, kProjectThreads, s, a);
    ++n;
    if (events) cudaEventRecord((cudaEvent_t)events[1], s);
    if (events) k_bin_big<<<big_blocks, 256, 0, s>>>(a);  // timed stages: plain launches
    else launch_after(k_bin_big, big_blocks, 256, s, a);
    ++n;
    if (clip) join(1);
    if (a.flags_any & 0xC0u) {
      k_overlay<<<big_blocks, 256, 0, s>>>(a);
      ++n;
    }
    if (events) cudaEventRecord((cudaEvent_t)events[2], s);
  } else if (events) {
    cudaEventRecord((cudaEvent_t)events[1], s);
    cudaEventRecord((cudaEvent_t)events[2], s);
  }
  if (events) k_plan<<<(a.total_tiles + 255) / 256, 256, 0, s>>>(a);
  else launch_after(k_plan, (a.total_tiles + 255) / 256, 256, s, a);
  ++n;
  if (a.tile_shift == 4)
    launch_after(a.clear_empty ? k_raster<16, true> : k_raster<16, false>, a.raster_ctas, RasterShape<16>::kThreads, s, a);
  else
    launch_after(a.clear_empty ? k_raster<32, true> : k_raster<32, false>, a.raster_ctas, RasterShape<32>::kThreads, s, a);
  ++n;
  if (a.pkey && a.total_pixels) {
    launch_after(k_resolve, (unsigned)((a.total_pixels + 255) / 256), 256, s, a);
    ++n;
  }
  if (events) cudaEventRecord((cudaEvent_t)events[3], s);
  if (launches) *launches = n;
  return (int)cudaGetLastError();
}

}  // namespace gr
