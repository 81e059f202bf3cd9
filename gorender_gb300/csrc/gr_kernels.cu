// gr_kernels.cu -- sm_103a kernels of the frame pipeline.
//
// A frame runs as three kernels on one stream:
//   k_project  one thread per face: vertex transform, backface cull, lighting,
//              frustum clip, perspective divide + screen map, one-tile bin test
//              and edge-function setup; triangles are compacted with a warp
//              scan + one atomic per warp and appended to per-tile bins with
//              warp-aggregated atomics (__match_any_sync) or, when they span
//              more than four tiles, to a multi-tile queue.
//   k_bin_big  one CTA per multi-tile triangle: appends it to every 32x32 tile
//              its edge functions can reach.
//   k_raster   one CTA per 32x32 tile: resolves visibility in shared memory as
//              a 64-bit max of (ordered zRec, draw-order key), walking 8x8
//              pixel blocks per warp; then shades each pixel once for its
//              winner (deferred), fused with Clear + DotGrid, and writes the
//              tile back with 16-byte stores.
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

__device__ __forceinline__ SV to_screen(const PV& q, const float* S) {
  float W = q.p.w;
  float dx = fd(q.p.x, W), dy = fd(q.p.y, W), dz = fd(q.p.z, W), dw = fd(q.p.w, W);
  SV s;
  s.sx = fa(fa(fa(fm(S[0], dx), fm(S[1], dy)), fm(S[2], dz)), fm(S[3], dw));
  s.sy = fa(fa(fa(fm(S[4], dx), fm(S[5], dy)), fm(S[6], dz)), fm(S[7], dw));
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

// identifyTriangleTiles with the single screen tile (renderer.go:226-244):
// Go's min/max propagate NaN, so a NaN coordinate drops the triangle.
__device__ __forceinline__ bool bin_test(const SV& a, const SV& b, const SV& c, float Wf, float Hf) {
  if (isnan(a.sx) || isnan(b.sx) || isnan(c.sx) || isnan(a.sy) || isnan(b.sy) || isnan(c.sy)) return false;
  float minX = fminf(fminf(a.sx, b.sx), c.sx), maxX = fmaxf(fmaxf(a.sx, b.sx), c.sx);
  float minY = fminf(fminf(a.sy, b.sy), c.sy), maxY = fmaxf(fmaxf(a.sy, b.sy), c.sy);
  return maxX >= 0.0f && minX <= Wf && maxY >= 0.0f && minY <= Hf;
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
    s.w.pad = 0;
    s.r.a01 = s.r.b01 = s.r.c01 = s.r.a12 = s.r.b12 = s.r.c12 = s.r.a20 = s.r.b20 = s.r.c20 = 0;
    s.r.sumf = __ll2float_rn((long long)sum);
    s.wide = true;
  }
  return true;
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

// Barycentrics and zRec at a covered pixel (rasterizer.go:149-153).
__device__ __forceinline__ float zrec_of(float e12f, float e20f, float sumf, float w0, float w1, float w2,
                                         float& al, float& be, float& ga) {
  al = fd(e12f, sumf);
  be = fd(e20f, sumf);
  ga = fs(fs(1.0f, al), be);
  return -fa(fa(fd(al, w0), fd(be, w1)), fd(ga, w2));
}

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// Appends record r to tile t's bin; over capacity the position is recorded
// so the host can grow the bins and re-run the frame.
__device__ __forceinline__ void bin_store(const FrameArgs& a, uint32_t tile, uint32_t pos, uint32_t r) {
  if (pos < a.bin_cap)
    a.bins[(size_t)tile * a.bin_cap + pos] = r;
  else
    atomicMax(&a.work->bin_need, pos + 1);
}

// ---------------------------------------------------------------------------
// k_project
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kProjectThreads) k_project(const FrameArgs a) {
  __shared__ float s_mvp[16];
  __shared__ float s_world[16];
  __shared__ int s_item;
  __shared__ int s_vis;
  __shared__ unsigned s_out[8];

  const int tid = threadIdx.x;
  if (tid == 0) {
    int lo = 0, hi = a.num_items - 1;
    while (lo < hi) {  // last item with block_base <= blockIdx.x
      int mid = (lo + hi + 1) >> 1;
      if (a.items[mid].block_base <= (int)blockIdx.x) lo = mid; else hi = mid - 1;
    }
    s_item = lo;
  }
  __syncthreads();
  const DevItem& it = a.items[s_item];
  if (tid < 16) {
    s_mvp[tid] = it.mvp[tid];
    s_world[tid] = it.world[tid];
  }
  __syncthreads();
  // Frustum.BoxVisibility of the transformed bounding box (renderer.go:268-275).
  if (tid < 8) {
    V4 c = mat_vec(s_mvp, V4{it.bbox[4 * tid], it.bbox[4 * tid + 1], it.bbox[4 * tid + 2], it.bbox[4 * tid + 3]});
    unsigned bits = 0;
    for (int i = 0; i < 6; ++i) {
      float d = fs(dot4(plane_n(i), c), dot4(plane_n(i), plane_p(i)));  // DistanceToVertex
      if (d > 0.0f) bits |= 1u << i;
    }
    s_out[tid] = bits;
  }
  __syncthreads();
  if (tid == 0) {
    int vis = 2;  // Inside
    for (int i = 0; i < 6; ++i) {
      int outside = 0;
      for (int k = 0; k < 8; ++k) outside += (s_out[k] >> i) & 1u;
      if (outside == 8) { vis = 0; break; }
      if (outside > 0) { vis = 1; break; }
    }
    s_vis = vis;
  }
  __syncthreads();
  const int vis = s_vis;
  if (vis == 0) return;  // whole block: object outside the frustum

  const uint32_t fl = a.flags;
  const int f = ((int)blockIdx.x - it.block_base) * kProjectThreads + tid;
  const bool valid = f < it.nf;
  const unsigned lane = lane_id();

  PV poly[9];
  PV tmp[9];
  int pcount = 0;
  int tex = -1;
  if (valid) {
    const int i0 = __ldg(it.vidx + 3 * f), i1 = __ldg(it.vidx + 3 * f + 1), i2 = __ldg(it.vidx + 3 * f + 2);
    V4 v0 = mat_vec(s_mvp, ld4(it.pos + 4 * (size_t)i0));
    V4 v1 = mat_vec(s_mvp, ld4(it.pos + 4 * (size_t)i1));
    V4 v2 = mat_vec(s_mvp, ld4(it.pos + 4 * (size_t)i2));
    bool draw = true;
    if (fl & 0x04u) {  // BackfaceCulling: facingCamera (renderer.go:246-250)
      float e1x = fs(v1.x, v0.x), e1y = fs(v1.y, v0.y), e1z = fs(v1.z, v0.z);
      float e2x = fs(v2.x, v0.x), e2y = fs(v2.y, v0.y), e2z = fs(v2.z, v0.z);
      float nx = fs(fm(e1y, e2z), fm(e1z, e2y));
      float ny = fs(fm(e1z, e2x), fm(e1x, e2z));
      float nz = fs(fm(e1x, e2y), fm(e1y, e2x));
      float d = fa(fa(fm(nx, fs(0.0f, v0.x)), fm(ny, fs(0.0f, v0.y))), fm(nz, fs(0.0f, v0.z)));
      draw = d > 0.0f;
    }
    if (draw) {
      float in0, in1, in2;
      if (fl & 0x08u) {  // Lighting (renderer.go:326-346)
        if (it.nn != 0 && !(fl & 0x10u)) {
          float in[3];
          for (int k = 0; k < 3; ++k) {
            int ni = __ldg(it.nidx + 3 * f + k);
            V4 n = mat_vec(s_world, ld4(it.vnrm + 4 * (size_t)ni));
            float len = __fsqrt_rn(fa(fa(fa(fm(n.x, n.x), fm(n.y, n.y)), fm(n.z, n.z)), fm(n.w, n.w)));
            float x = fd(n.x, len), y = fd(n.y, len), z = fd(n.z, len);
            float d = fa(fa(fm(x, a.L[0]), fm(y, a.L[1])), fm(z, a.L[2]));
            in[k] = fa(0.5f, fm(d, 0.5f));
          }
          in0 = in[0]; in1 = in[1]; in2 = in[2];
        } else {
          V4 n = mat_vec(s_world, ld4(it.fnrm + 4 * (size_t)f));
          float len = __fsqrt_rn(fa(fa(fa(fm(n.x, n.x), fm(n.y, n.y)), fm(n.z, n.z)), fm(n.w, n.w)));
          float x = fd(n.x, len), y = fd(n.y, len), z = fd(n.z, len);
          float d = fa(fa(fm(x, a.L[0]), fm(y, a.L[1])), fm(z, a.L[2]));
          in0 = in1 = in2 = fa(0.5f, fm(d, 0.5f));
        }
      } else {
        in0 = in1 = in2 = 0.5f;
      }
      poly[0].p = v0; poly[1].p = v1; poly[2].p = v2;
      poly[0].in = in0; poly[1].in = in1; poly[2].in = in2;
      if (it.uv) {
        const float* uv = it.uv + 6 * (size_t)f;
        poly[0].u = __ldg(uv); poly[0].v = __ldg(uv + 1);
        poly[1].u = __ldg(uv + 2); poly[1].v = __ldg(uv + 3);
        poly[2].u = __ldg(uv + 4); poly[2].v = __ldg(uv + 5);
      } else {
        poly[0].u = poly[0].v = poly[1].u = poly[1].v = poly[2].u = poly[2].v = 0.0f;
      }
      if (it.vcol) {
        const float* c0 = it.vcol + 3 * (size_t)i0;
        const float* c1 = it.vcol + 3 * (size_t)i1;
        const float* c2 = it.vcol + 3 * (size_t)i2;
        poly[0].r = __ldg(c0); poly[0].g = __ldg(c0 + 1); poly[0].b = __ldg(c0 + 2);
        poly[1].r = __ldg(c1); poly[1].g = __ldg(c1 + 1); poly[1].b = __ldg(c1 + 2);
        poly[2].r = __ldg(c2); poly[2].g = __ldg(c2 + 1); poly[2].b = __ldg(c2 + 2);
      } else {
        poly[0].r = poly[0].g = poly[0].b = poly[1].r = poly[1].g = poly[1].b = 0.0f;
        poly[2].r = poly[2].g = poly[2].b = 0.0f;
      }
      int t = it.tex ? __ldg(it.tex + f) : -1;
      tex = ((fl & 0x20u) && t >= 0) ? t : (it.vcol ? -2 : -1);  // renderer.go:176-178
      pcount = 3;
      if ((fl & 0x01u) && vis != 2) {  // FrustumClipping (renderer.go:349-359)
        bool all_in = true;
        for (int i = 0; i < 6 && all_in; ++i)
          all_in = plane_inside(i, v0) && plane_inside(i, v1) && plane_inside(i, v2);
        if (!all_in) {  // six all-inside passes rotate the triangle back to itself
          pcount = clip_polygon(poly, tmp);
          if (pcount < 0) {
            atomicOr(&a.work->error, 1u);
            pcount = 0;
          }
        }
      }
    }
  }

  // Divide + screen map per polygon vertex, bin test and setup per fan triangle.
  SV sv[9];
  unsigned fanmask = 0;
  int ntpf = 0;
  const float Wf = (float)a.W, Hf = (float)a.H;
  for (int k = 0; k < pcount; ++k) sv[k] = to_screen(poly[k], a.S);
  for (int t = 0; t + 2 < pcount; ++t) {
    if (!bin_test(sv[0], sv[t + 1], sv[t + 2], Wf, Hf)) continue;
    ++ntpf;
    Setup s;
    // ShowFaces off: triangles still count in TPF but are not rasterised (renderer.go:180)
    if ((fl & 0x02u) && setup_tri(sv[0], sv[t + 1], sv[t + 2], a.W, a.H, s)) fanmask |= 1u << t;
  }

  // TPF: one atomic per warp.
  int wt = __reduce_add_sync(FULL_MASK, ntpf);
  if (lane == 0 && wt) atomicAdd(&a.work->tpf, (unsigned long long)wt);

  // Compact records: warp exclusive scan of per-lane counts, one atomic per warp.
  const int nmine = __popc(fanmask);
  int incl = nmine;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int y = __shfl_up_sync(FULL_MASK, incl, o);
    if ((int)lane >= o) incl += y;
  }
  const int total = __shfl_sync(FULL_MASK, incl, 31);
  if (total == 0) return;
  unsigned base = 0;
  if (lane == 31) base = atomicAdd(&a.work->nrec, (unsigned)total);
  base = __shfl_sync(FULL_MASK, base, 31);
  if (lane == 31 && base + (unsigned)total > a.rec_cap) atomicMax(&a.work->rec_need, base + (unsigned)total);
  unsigned my = base + (unsigned)(incl - nmine);
  const int maxn = __reduce_max_sync(FULL_MASK, nmine);
  const uint32_t face_key = (it.face_base + (uint32_t)(valid ? f : 0)) * (uint32_t)kKeysPerFace;

  unsigned rem = fanmask;
  for (int iter = 0; iter < maxn; ++iter) {
    bool has = rem != 0;
    int t = has ? __ffs(rem) - 1 : 0;
    if (has) rem &= rem - 1;
    uint32_t r = my;
    bool ok = has && r < a.rec_cap;
    if (has) ++my;
    uint32_t tx0 = 0, tx1 = 0, ty0 = 0, ty1 = 0;
    if (ok) {
      Setup s;
      setup_tri(sv[0], sv[t + 1], sv[t + 2], a.W, a.H, s);
      uint32_t okey = face_key + (uint32_t)t + 1u;
      s.r.key = okey | (s.wide ? 0x80000000u : 0u);
      const int4* src = reinterpret_cast<const int4*>(&s.r);
      int4* dst = reinterpret_cast<int4*>(a.rast + r);
      dst[0] = src[0]; dst[1] = src[1]; dst[2] = src[2]; dst[3] = src[3];
      if (s.wide) {
        const int4* ws = reinterpret_cast<const int4*>(&s.w);
        int4* wd = reinterpret_cast<int4*>(a.wide + r);
#pragma unroll
        for (int q = 0; q < 5; ++q) wd[q] = ws[q];
      }
      const SV& p0 = sv[0];
      const SV& p1 = sv[t + 1];
      const SV& p2 = sv[t + 2];
      TriShade sh;
      sh.u0w = fd(p0.u, p0.W); sh.v0w = fd(p0.v, p0.W);
      sh.u1w = fd(p1.u, p1.W); sh.v1w = fd(p1.v, p1.W);
      sh.u2w = fd(p2.u, p2.W); sh.v2w = fd(p2.v, p2.W);
      sh.i0 = p0.in; sh.i1 = p1.in; sh.i2 = p2.in;
      sh.tex = tex;
      sh.pad[0] = sh.pad[1] = 0.0f;
      const float4* ss = reinterpret_cast<const float4*>(&sh);
      float4* sd = reinterpret_cast<float4*>(a.shade + r);
      sd[0] = ss[0]; sd[1] = ss[1]; sd[2] = ss[2];
      if (tex == -2) {
        TriColor* c = a.tcol + r;
        c->c[0] = p0.r; c->c[1] = p0.g; c->c[2] = p0.b;
        c->c[3] = p1.r; c->c[4] = p1.g; c->c[5] = p1.b;
        c->c[6] = p2.r; c->c[7] = p2.g; c->c[8] = p2.b;
      }
      if (okey < a.key_cap) a.rec_of_key[okey] = r;
      tx0 = (uint32_t)s.r.bx0 >> kTileShift;
      tx1 = (uint32_t)s.r.bx1 >> kTileShift;
      ty0 = (uint32_t)s.r.by0 >> kTileShift;
      ty1 = (uint32_t)s.r.by1 >> kTileShift;
    }
    const uint32_t ntiles = ok ? (tx1 - tx0 + 1) * (ty1 - ty0 + 1) : 0u;
    // single-tile triangles: warp-aggregated append per distinct tile
    const bool one = ntiles == 1;
    const unsigned m1 = __ballot_sync(FULL_MASK, one);
    if (one) {
      const uint32_t tile = ty0 * (uint32_t)a.tiles_x + tx0;
      const unsigned grp = __match_any_sync(m1, tile);
      const int leader = __ffs(grp) - 1;
      const unsigned rank = __popc(grp & ((1u << lane) - 1u));
      uint32_t pos = 0;
      if ((int)lane == leader) pos = atomicAdd(&a.bin_count[tile], (uint32_t)__popc(grp));
      pos = __shfl_sync(grp, pos, leader) + rank;
      bin_store(a, tile, pos, r);
    }
    // two to four tiles: direct appends
    if (ntiles > 1 && ntiles <= (uint32_t)kBinDirectMax) {
      for (uint32_t ty = ty0; ty <= ty1; ++ty)
        for (uint32_t tx = tx0; tx <= tx1; ++tx) {
          const uint32_t tile = ty * (uint32_t)a.tiles_x + tx;
          bin_store(a, tile, atomicAdd(&a.bin_count[tile], 1u), r);
        }
    }
    // more: the multi-tile queue, one atomic per warp
    const bool many = ntiles > (uint32_t)kBinDirectMax;
    const unsigned mm = __ballot_sync(FULL_MASK, many);
    if (mm) {
      uint32_t qb = 0;
      const int ldr = __ffs(mm) - 1;
      if ((int)lane == ldr) qb = atomicAdd(&a.work->nbig, (uint32_t)__popc(mm));
      qb = __shfl_sync(FULL_MASK, qb, ldr);
      if (many) {
        const uint32_t q = qb + __popc(mm & ((1u << lane) - 1u));
        if (q < a.big_cap) a.big[q] = r;
        else atomicMax(&a.work->big_need, q + 1);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// k_bin_big: one CTA per multi-tile triangle
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_bin_big(const FrameArgs a) {
  const uint32_t nbig = min(*(volatile uint32_t*)&a.work->nbig, a.big_cap);
  for (uint32_t q = blockIdx.x; q < nbig; q += gridDim.x) {
    const uint32_t r = a.big[q];
    const TriRaster t = a.rast[r];
    const uint32_t tx0 = (uint32_t)t.bx0 >> kTileShift, tx1 = (uint32_t)t.bx1 >> kTileShift;
    const uint32_t ty0 = (uint32_t)t.by0 >> kTileShift, ty1 = (uint32_t)t.by1 >> kTileShift;
    const uint32_t nx = tx1 - tx0 + 1, n = nx * (ty1 - ty0 + 1);
    const bool wide = (t.key & 0x80000000u) != 0;
    for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) {
      const uint32_t tx = tx0 + j % nx, ty = ty0 + j / nx;
      if (!wide) {
        // conservative reject: an edge that is >= 0 over the whole
        // tile-clipped box excludes every pixel of it
        const long long X0 = max((int)(tx << kTileShift), (int)t.bx0);
        const long long X1 = min((int)((tx << kTileShift) + kTileSize - 1), (int)t.bx1);
        const long long Y0 = max((int)(ty << kTileShift), (int)t.by0);
        const long long Y1 = min((int)((ty << kTileShift) + kTileSize - 1), (int)t.by1);
        const long long e01 = t.c01 + min(t.a01 * X0, t.a01 * X1) + min(t.b01 * Y0, t.b01 * Y1);
        const long long e12 = t.c12 + min(t.a12 * X0, t.a12 * X1) + min(t.b12 * Y0, t.b12 * Y1);
        const long long e20 = t.c20 + min(t.a20 * X0, t.a20 * X1) + min(t.b20 * Y0, t.b20 * Y1);
        if (e01 >= 0 || e12 >= 0 || e20 >= 0) continue;
      }
      const uint32_t tile = ty * (uint32_t)a.tiles_x + tx;
      bin_store(a, tile, atomicAdd(&a.bin_count[tile], 1u), r);
    }
  }
}

// ---------------------------------------------------------------------------
// k_raster: one CTA per 32x32 tile
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

__device__ __forceinline__ void raster_pixel(unsigned long long* skey, const TriRaster& t, const TriWide* wide,
                                             uint32_t r, int x, int y, int tx0, int ty0) {
  bool inside;
  float e12f, e20f;
  edges_at(t, wide, r, x, y, inside, e12f, e20f);
  if (!inside) return;
  float al, be, ga;
  float z = zrec_of(e12f, e20f, t.sumf, t.w0, t.w1, t.w2, al, be, ga);
  if (!(z >= -1.0f)) return;  // rasterizer.go:156 against the cleared Z of -1
  unsigned long long k = depth_key(z, t.key);
  unsigned long long* p = skey + (y - ty0) * kTileSize + (x - tx0);
  if (k > *(volatile unsigned long long*)p) atomicMax(p, k);
}

__global__ void __launch_bounds__(kRasterThreads) k_raster(const FrameArgs a) {
  __shared__ unsigned long long skey[kTileSize * kTileSize];
  const int tid = threadIdx.x;
  const uint32_t tile = blockIdx.x;
  const int tx0 = (int)(tile % (uint32_t)a.tiles_x) << kTileShift;
  const int ty0 = (int)(tile / (uint32_t)a.tiles_x) << kTileShift;
  const int tx1 = min(tx0 + kTileSize - 1, a.W - 1);
  const int ty1 = min(ty0 + kTileSize - 1, a.H - 1);

  for (int i = tid; i < kTileSize * kTileSize; i += kRasterThreads) skey[i] = BG_KEY;
  const uint32_t count = a.bin_count[tile];
  const uint32_t n = min(count, a.bin_cap);
  if (tid == 0 && blockIdx.x == 0) {
    // publish and reset the frame counters (all appends are complete)
    DevWork* w = a.work;
    a.result->tpf = w->tpf;
    a.result->nrec = w->nrec;
    a.result->nbig = w->nbig;
    a.result->bin_need = w->bin_need;
    a.result->rec_need = w->rec_need;
    a.result->big_need = w->big_need;
    a.result->error = w->error;
    w->tpf = 0; w->nrec = 0; w->nbig = 0; w->bin_need = 0; w->rec_need = 0; w->big_need = 0; w->error = 0;
  }
  __syncthreads();

  const unsigned lane = lane_id();
  const int warp = tid >> 5;
  const uint32_t* bin = a.bins + (size_t)tile * a.bin_cap;
  for (uint32_t b = (uint32_t)warp * 32u; b < n; b += kRasterThreads) {
    const uint32_t i = b + lane;
    const bool valid = i < n;
    uint32_t r = 0;
    int lx0 = 0, lx1 = -1, ly0 = 0, ly1 = -1;
    TriRaster t;
    if (valid) {
      r = bin[i];
      t = a.rast[r];
      lx0 = max((int)t.bx0, tx0); lx1 = min((int)t.bx1, tx1);
      ly0 = max((int)t.by0, ty0); ly1 = min((int)t.by1, ty1);
    }
    const int area = (lx1 >= lx0 && ly1 >= ly0) ? (lx1 - lx0 + 1) * (ly1 - ly0 + 1) : 0;
    const bool small = valid && area > 0 && area <= 16;
    if (small) {
      for (int y = ly0; y <= ly1; ++y)
        for (int x = lx0; x <= lx1; ++x) raster_pixel(skey, t, a.wide, r, x, y, tx0, ty0);
    }
    // larger footprints: the whole warp walks 8x8 blocks, 2 pixels per lane
    unsigned bigm = __ballot_sync(FULL_MASK, valid && area > 16);
    while (bigm) {
      const int src = __ffs(bigm) - 1;
      bigm &= bigm - 1;
      const uint32_t rr = __shfl_sync(FULL_MASK, r, src);
      const int bx0 = __shfl_sync(FULL_MASK, lx0, src), bx1 = __shfl_sync(FULL_MASK, lx1, src);
      const int by0 = __shfl_sync(FULL_MASK, ly0, src), by1 = __shfl_sync(FULL_MASK, ly1, src);
      const TriRaster tt = a.rast[rr];
      const int px = (int)(lane & 7u), py = (int)(lane >> 3);
      for (int y8 = by0; y8 <= by1; y8 += 8)
        for (int x8 = bx0; x8 <= bx1; x8 += 8) {
          const int x = x8 + px;
          if (x > bx1) continue;
          const int y = y8 + py;
          if (y <= by1) raster_pixel(skey, tt, a.wide, rr, x, y, tx0, ty0);
          if (y + 4 <= by1) raster_pixel(skey, tt, a.wide, rr, x, y + 4, tx0, ty0);
        }
    }
  }
  __syncthreads();

  // Resolve + deferred shading; Clear and DotGrid for uncovered pixels.
  const int row = tid >> 3;
  const int col = (tid & 7) << 2;
  const int y = ty0 + row;
  if (y <= ty1) {
    uint32_t out_c[4];
    float out_z[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int x = tx0 + col + j;
      const unsigned long long k = skey[row * kTileSize + col + j];
      if (k == BG_KEY || x > tx1) {
        const bool dot = (x % 10 == 0) && (y % 10 == 0) && x >= 10 && y >= 10;  // DotGrid
        out_c[j] = dot ? 0xFF646464u : 0xFF323232u;
        out_z[j] = -1.0f;
        continue;
      }
      const uint32_t okey = (uint32_t)k & 0x7FFFFFFFu;
      const uint32_t r = a.rec_of_key[okey];
      const TriRaster t = a.rast[r];
      const TriShade s = a.shade[r];
      bool inside;
      float e12f, e20f, al, be, ga;
      edges_at(t, a.wide, r, x, y, inside, e12f, e20f);
      const float z = zrec_of(e12f, e20f, t.sumf, t.w0, t.w1, t.w2, al, be, ga);
      const float I = fa(fa(fm(al, s.i0), fm(be, s.i1)), fm(ga, s.i2));
      uint32_t c;
      if (s.tex >= 0) {
        const float u = fd(fa(fa(fm(al, s.u0w), fm(be, s.u1w)), fm(ga, s.u2w)), z);
        const float v = fd(fa(fa(fm(al, s.v0w), fm(be, s.v1w)), fm(ga, s.v2w)), z);
        c = color_intensity(tex_sample(a.texs[s.tex], u, v), I);
      } else if (s.tex == -2) {
        const TriColor& tc = a.tcol[r];
        uint32_t ch[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          const float cq = fa(fa(fm(al, tc.c[q]), fm(be, tc.c[3 + q])), fm(ga, tc.c[6 + q]));
          ch[q] = go_u8(fm(fm(cq, 255.0f), I));
        }
        c = ch[0] | (ch[1] << 8) | (ch[2] << 16) | 0xFF000000u;
      } else {
        c = color_intensity(0xFFC8C8C8u, I);  // faceColor (200,200,200,255)
      }
      out_c[j] = c;
      out_z[j] = z;
    }
    const int x = tx0 + col;
    const size_t o = (size_t)y * (size_t)a.W + (size_t)x;
    if (a.vec_ok && x + 3 <= tx1) {
      *reinterpret_cast<uint4*>(a.out_rgba + o) = make_uint4(out_c[0], out_c[1], out_c[2], out_c[3]);
      *reinterpret_cast<float4*>(a.out_z + o) = make_float4(out_z[0], out_z[1], out_z[2], out_z[3]);
    } else {
      for (int j = 0; j < 4 && x + j <= tx1; ++j) {
        a.out_rgba[o + j] = out_c[j];
        a.out_z[o + j] = out_z[j];
      }
    }
  }
  if (tid == 0) a.bin_count[tile] = 0;  // ready for the next frame
}

int launch_frame(const FrameArgs& a, int big_blocks, void* stream, int* launches, void* const* events) {
  cudaStream_t s = (cudaStream_t)stream;
  int n = 0;
  if (events) cudaEventRecord((cudaEvent_t)events[0], s);
  if (a.total_blocks > 0) {
    k_project<<<a.total_blocks, kProjectThreads, 0, s>>>(a);
    ++n;
    if (events) cudaEventRecord((cudaEvent_t)events[1], s);
    k_bin_big<<<big_blocks, 256, 0, s>>>(a);
    ++n;
    if (events) cudaEventRecord((cudaEvent_t)events[2], s);
  } else if (events) {
    cudaEventRecord((cudaEvent_t)events[1], s);
    cudaEventRecord((cudaEvent_t)events[2], s);
  }
  k_raster<<<a.tiles_x * a.tiles_y, kRasterThreads, 0, s>>>(a);
  ++n;
  if (events) cudaEventRecord((cudaEvent_t)events[3], s);
  if (launches) *launches = n;
  return (int)cudaGetLastError();
}

}  // namespace gr
