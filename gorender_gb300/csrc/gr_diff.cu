// gr_diff.cu -- differentiable shading on top of the exact visibility pass.
//
// This is an extension with no counterpart in the reference renderer.  The
// frame pipeline (gr_kernels.cu) resolves visibility exactly as
// FrameBuffer.Triangle does (rasterizer.go:90-183) and, for views flagged
// kViewFaceIds, writes the winning face per pixel instead of a colour.  The
// kernels here add a smooth shading model over that fixed visibility:
//
//   screen position of corner i   s_i = S * (clip_i / W_i)          clip_i = MVP * p_i
//   edge functions at pixel (x,y) e_0 = (x1-x)(y2-y) - (x2-x)(y1-y)  (and cyclic)
//   perspective barycentrics      b_i = (e_i / W_i) / sum_j (e_j / W_j)
//   clipped to the triangle       l_i = max(b_i, 0) / sum_j max(b_j, 0)
//
// The barycentrics are evaluated in the 2D homogeneous form (Olano and Greer,
// "Triangle scan conversion using 2D homogeneous coordinates", 1997), which
// needs no perspective divide: with Q = S * MVP,
//   u_i = (Q_0 - x Q_3) . p_i,  v_i = (Q_1 - y Q_3) . p_i       (= (s_i - pixel) * W_i)
//   D_0 = u_1 v_2 - u_2 v_1 (and cyclic),  b_i = D_i / (D_0 + D_1 + D_2)
// u and v cancel screen positions of hundreds of pixels down to a few, and on
// thin faces D amplifies what is left, so float32 would leave relative errors
// up to ~1e-3: hx = Q_0.p, hy = Q_1.p and W = Q_3.p are computed once per
// (view, vertex) in double and kept as float-float pairs, and u, v and D are
// formed per pixel in float-float arithmetic (error-free sums and products,
// Dekker 1971; Knuth, TAOCP vol. 2) on the float32 pipes, which on this GPU
// run about 64 times as many operations as the double-precision ones.
// The barycentrics are homogeneous of degree 0 in D, so the clip and the
// normalisation run in float32 on D's correctly signed values:
//   l_i = max(s D_i, 0) / sum_j max(s D_j, 0),  s = sign(D_0 + D_1 + D_2).
// The backward chain runs in float32 from those values and from per-column
// and per-row tables of Q_0 - x Q_3 and Q_1 - y Q_3 (exact in double, then
// rounded).
//   colour                        c   = sum_i l_i c_i               (vertex RGB)
//   intensity                     I   = sum_i l_i (0.5 + 0.5 nhat_i . L)
//   texel                         t   = tex[floor(v th) mod th][floor(u tw) mod tw],  (u,v) = sum_i l_i uv_i
//   pixel                         out = (I c_r t_r, I c_g t_g, I c_b t_b, t_a)
//   loss                          sum over pixels and channels of (out - target)^2
//
// nhat_i is the renderer's Gouraud normal, xyz of Vec4.Normalize(world * n)
// (renderer.go:328-331); vertex normals are fixed inputs.  The forward pass
// stores per pixel the face, the texel and (l0, l1); the backward pass reads
// them back, recomputes the shading and accumulates the gradients of the loss
// with respect to vertex colours, texels, the light direction and vertex
// positions.  Position gradients flow through the barycentrics only (the
// interior term): visibility and texel choices are held fixed.

#include <cuda_runtime.h>

#include <algorithm>

#include "gr_internal.h"

namespace gr {

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ float go_min(float a, float b) {
  // Go's min: NaN wins, -0 below +0
  if (a != a || b != b) return __int_as_float(0x7fc00000);
  if (a < b) return a;
  if (b < a) return b;
  return signbit(a) ? a : b;
}
__device__ __forceinline__ float go_max(float a, float b) {
  if (a != a || b != b) return __int_as_float(0x7fc00000);
  if (a > b) return a;
  if (b > a) return b;
  return signbit(a) ? b : a;
}

// Mesh.BoundingBox (mesh.go:28-51) of pos; min and max are order-free, so a
// tree reduction gives the sequential loop's result.  Each CTA reduces a
// grid-strided share into partial[6 * block]; the last CTA to finish (an
// atomic counter, no waiting) reduces the partials and writes the corners.
__global__ void __launch_bounds__(1024) k_diff_bbox(const float* __restrict__ pos, int nv, DevItem* items,
                                                    int num_items, float* partial, unsigned* done) {
  __shared__ float s_v[6][32];
  __shared__ float s_b[32];
  __shared__ unsigned s_last;
  const int tid = threadIdx.x;
  float mn[3] = {pos[0], pos[1], pos[2]}, mx[3] = {pos[0], pos[1], pos[2]};
  for (int i = blockIdx.x * blockDim.x + tid; i < nv; i += gridDim.x * blockDim.x) {
    const float4 p = reinterpret_cast<const float4*>(pos)[i];
    mn[0] = go_min(mn[0], p.x); mn[1] = go_min(mn[1], p.y); mn[2] = go_min(mn[2], p.z);
    mx[0] = go_max(mx[0], p.x); mx[1] = go_max(mx[1], p.y); mx[2] = go_max(mx[2], p.z);
  }
  for (int o = 16; o > 0; o >>= 1) {
    for (int k = 0; k < 3; ++k) {
      mn[k] = go_min(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
      mx[k] = go_max(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
    }
  }
  const int warp = tid >> 5, lane = tid & 31;
  if (lane == 0) {
    for (int k = 0; k < 3; ++k) {
      s_v[k][warp] = mn[k];
      s_v[3 + k][warp] = mx[k];
    }
  }
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    for (int k = 0; k < 3; ++k) {
      mn[k] = lane < nw ? s_v[k][lane] : s_v[k][0];
      mx[k] = lane < nw ? s_v[3 + k][lane] : s_v[3 + k][0];
    }
    for (int o = 16; o > 0; o >>= 1) {
      for (int k = 0; k < 3; ++k) {
        mn[k] = go_min(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
        mx[k] = go_max(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
      }
    }
    if (lane == 0) {
      for (int k = 0; k < 3; ++k) {
        partial[6 * blockIdx.x + k] = mn[k];
        partial[6 * blockIdx.x + 3 + k] = mx[k];
      }
      __threadfence();
      s_last = atomicAdd(done, 1u) == gridDim.x - 1u ? 1u : 0u;
    }
  }
  __syncthreads();
  if (!s_last) return;
  if (warp == 0) {
    __threadfence();
    const volatile float* pv = partial;
    for (int k = 0; k < 3; ++k) {
      mn[k] = pv[k];
      mx[k] = pv[3 + k];
    }
    for (unsigned b = (unsigned)lane; b < gridDim.x; b += 32) {
      for (int k = 0; k < 3; ++k) {
        mn[k] = go_min(mn[k], pv[6 * b + k]);
        mx[k] = go_max(mx[k], pv[6 * b + 3 + k]);
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      for (int k = 0; k < 3; ++k) {
        mn[k] = go_min(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
        mx[k] = go_max(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
      }
    }
    if (lane == 0) {
      *done = 0u;  // ready for the next forward pass
      // corners in mesh.go's order: x outermost, then y, then z; w = 1
      for (int c = 0; c < 8; ++c) {
        s_b[4 * c + 0] = (c & 4) ? mx[0] : mn[0];
        s_b[4 * c + 1] = (c & 2) ? mx[1] : mn[1];
        s_b[4 * c + 2] = (c & 1) ? mx[2] : mn[2];
        s_b[4 * c + 3] = 1.0f;
      }
    }
  }
  __syncthreads();
  for (int i = tid; i < num_items * 32; i += blockDim.x) items[i / 32].bbox[i % 32] = s_b[i % 32];
  // and each view's BoxVisibility of this box, which k_cull reads
  for (int i = tid; i < num_items; i += blockDim.x) items[i].vis = box_visibility(items[i].mvp, s_b);
}

__device__ __forceinline__ float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

__device__ __forceinline__ float4 mvp_apply(const float* m, float4 v) {
  float4 r;
  r.x = m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3] * v.w;
  r.y = m[4] * v.x + m[5] * v.y + m[6] * v.z + m[7] * v.w;
  r.z = m[8] * v.x + m[9] * v.y + m[10] * v.z + m[11] * v.w;
  r.w = m[12] * v.x + m[13] * v.y + m[14] * v.z + m[15] * v.w;
  return r;
}

__global__ void __launch_bounds__(kThreads) k_diff_normals(const float* __restrict__ world,
                                                           const float* __restrict__ vnrm, int nn, float* nhat) {
  const int n = blockIdx.x * kThreads + threadIdx.x;
  if (n >= nn) return;
  const float4 v = mvp_apply(world, ldg4(vnrm + 4 * (size_t)n));
  const float len = __fsqrt_rn(v.x * v.x + v.y * v.y + v.z * v.z + v.w * v.w);
  reinterpret_cast<float4*>(nhat)[n] = make_float4(v.x / len, v.y / len, v.z / len, 0.0f);
}

// Per view: Q_0 - x Q_3 for every column x and Q_1 - y Q_3 for every row y
// (d u / d p and d v / d p), evaluated in double and rounded to float.
__global__ void __launch_bounds__(kThreads) k_diff_tables(const DiffArgs a) {
  const DiffView& vw = a.views[blockIdx.y];
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i < vw.W) {
    float4 r;
    r.x = (float)__fma_rn(-(double)i, vw.Q[8], vw.Q[0]);
    r.y = (float)__fma_rn(-(double)i, vw.Q[9], vw.Q[1]);
    r.z = (float)__fma_rn(-(double)i, vw.Q[10], vw.Q[2]);
    r.w = 0.0f;
    a.col_tab[vw.col_base + i] = r;
  }
  if (i < vw.H) {
    float4 r;
    r.x = (float)__fma_rn(-(double)i, vw.Q[8], vw.Q[4]);
    r.y = (float)__fma_rn(-(double)i, vw.Q[9], vw.Q[5]);
    r.z = (float)__fma_rn(-(double)i, vw.Q[10], vw.Q[6]);
    r.w = 0.0f;
    a.row_tab[vw.row_base + i] = r;
  }
}

// Float-float arithmetic: a value is hi + lo with |lo| <= ulp(hi) / 2.
struct FF {
  float hi, lo;
};
__device__ __forceinline__ FF two_sum(float a, float b) {  // exact: s + e = a + b
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return FF{s, e};
}
__device__ __forceinline__ FF fast_two_sum(float a, float b) {  // exact when |a| >= |b|
  const float s = __fadd_rn(a, b);
  return FF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ FF ff_sub(FF a, FF b) {
  FF s = two_sum(a.hi, -b.hi);
  s.lo = __fadd_rn(s.lo, __fsub_rn(a.lo, b.lo));
  return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  FF s = two_sum(a.hi, b.hi);
  s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ FF ff_mul(FF a, FF b) {  // the product of the his is exact with an FMA
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fadd_rn(e, __fadd_rn(__fmul_rn(a.hi, b.lo), __fmul_rn(a.lo, b.hi)));
  return fast_two_sum(p, e);
}
__device__ __forceinline__ FF ff_mul_f(FF a, float b) {
  const float p = __fmul_rn(a.hi, b);
  float e = __fmaf_rn(a.hi, b, -p);
  e = __fadd_rn(e, __fmul_rn(a.lo, b));
  return fast_two_sum(p, e);
}

// Per (view, vertex): homogeneous screen x and y and clip W as float pairs,
// Q.p formed in float-float from Q's float pairs (the products of Q's hi and
// the float coordinates are exact with an FMA; ~48-bit significands, more
// than the geometry needs, with no FP64 instruction).
__global__ void __launch_bounds__(kThreads) k_diff_vertices(const DiffArgs a) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= a.nv) return;
  const DiffView& vw = a.views[blockIdx.y];
  const float4 p = ldg4(a.pos + 4 * (size_t)i);
  const float c[3] = {p.x, p.y, p.z};
  float* o = a.vh + 6 * ((size_t)blockIdx.y * (size_t)a.nv + (size_t)i);
#pragma unroll
  for (int r = 0; r < 3; ++r) {
    const float* q = vw.Qf + 8 * r;
    FF d{q[6], q[7]};
#pragma unroll
    for (int j = 0; j < 3; ++j) d = ff_add(d, ff_mul_f(FF{q[2 * j], q[2 * j + 1]}, c[j]));
    o[2 * r] = d.hi;
    o[2 * r + 1] = d.lo;
  }
}

// Geometry of one face at one pixel, shared by the forward and backward passes
// so that both compute bit-identical values.
struct FaceGeom {
  int vi[3];
  float u[3], v[3];   // (s_i - pixel) * W_i, rounded from double
  float d[3];         // s * D_i, rounded from double (s = sign of the sum)
  float m[3], M;      // max(d_i, 0) and their sum
  float sg;           // s
  bool ok;
};

__device__ __forceinline__ void face_geom(const DiffArgs& a, int view, int f, int px, int py, FaceGeom& g) {
  const int* vi = a.vidx + 3 * (size_t)f;
  const float X = (float)px, Y = (float)py;  // exact (< 2^24)
  FF u[3], v[3];
  g.ok = true;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    g.vi[k] = __ldg(vi + k);
    const float2* h = reinterpret_cast<const float2*>(a.vh + 6 * ((size_t)view * (size_t)a.nv + (size_t)g.vi[k]));
    const float2 hx = __ldg(h), hy = __ldg(h + 1), w = __ldg(h + 2);
    const FF W{w.x, w.y};
    g.ok = g.ok && W.hi < 0.0f;  // in front of the camera (W is negative there)
    u[k] = ff_sub(FF{hx.x, hx.y}, ff_mul_f(W, X));
    v[k] = ff_sub(FF{hy.x, hy.y}, ff_mul_f(W, Y));
    g.u[k] = __fadd_rn(u[k].hi, u[k].lo);
    g.v[k] = __fadd_rn(v[k].hi, v[k].lo);
  }
  const FF D0 = ff_sub(ff_mul(u[1], v[2]), ff_mul(u[2], v[1]));
  const FF D1 = ff_sub(ff_mul(u[2], v[0]), ff_mul(u[0], v[2]));
  const FF D2 = ff_sub(ff_mul(u[0], v[1]), ff_mul(u[1], v[0]));
  const FF T = ff_add(ff_add(D0, D1), D2);
  g.sg = T.hi < 0.0f ? -1.0f : 1.0f;
  g.d[0] = g.sg * __fadd_rn(D0.hi, D0.lo);
  g.d[1] = g.sg * __fadd_rn(D1.hi, D1.lo);
  g.d[2] = g.sg * __fadd_rn(D2.hi, D2.lo);
#pragma unroll
  for (int k = 0; k < 3; ++k) g.m[k] = fmaxf(g.d[k], 0.0f);
  g.M = g.m[0] + g.m[1] + g.m[2];
  g.ok = g.ok && T.hi != 0.0f && g.M > 0.0f && isfinite(g.M);
}

struct Shade {
  float l[3];
  float c[3][3];    // vertex colours
  float Ii[3];      // corner intensities
  float col[3];     // interpolated colour
  float I;
  float4 t;         // texel
  float4 out;
};

__device__ __forceinline__ void shade(const DiffArgs& a, const FaceGeom& g, float l0, float l1, uint32_t texel,
                                      const int* ni, Shade& s) {
  s.l[0] = l0;
  s.l[1] = l1;
  s.l[2] = 1.0f - l0 - l1;
  s.I = 0.0f;
#pragma unroll
  for (int ch = 0; ch < 3; ++ch) s.col[ch] = 0.0f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float* cp = a.vcol + 3 * (size_t)g.vi[k];
    const float4 n = ldg4(a.nhat + 4 * (size_t)__ldg(ni + k));
    s.Ii[k] = 0.5f + 0.5f * (n.x * a.L[0] + n.y * a.L[1] + n.z * a.L[2]);
    s.I += s.l[k] * s.Ii[k];
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
      s.c[k][ch] = __ldg(cp + ch);
      s.col[ch] += s.l[k] * s.c[k][ch];
    }
  }
  s.t = texel != kNoFace ? ldg4(a.tex + 4 * (size_t)texel) : make_float4(1.0f, 1.0f, 1.0f, 1.0f);
  s.out = make_float4(s.I * s.col[0] * s.t.x, s.I * s.col[1] * s.t.y, s.I * s.col[2] * s.t.z, s.t.w);
}

__device__ __forceinline__ int wrap_index(float u, int n) {
  const float f = floorf(u * (float)n);
  if (!(f > -2.0e9f && f < 2.0e9f)) return 0;
  int i = (int)f % n;
  return i < 0 ? i + n : i;
}

// The calling warp's slot of DiffArgs::partials (warps spread over the slots
// so that their atomics rarely meet).
__device__ __forceinline__ int diff_slot() {
  return (int)(((blockIdx.y * gridDim.x + blockIdx.x) * (kThreads / 32) + (threadIdx.x >> 5)) & (kDiffSlots - 1));
}

// Forward: per pixel record, shaded pixel and the loss.  Grid (pixels/256, views).
__global__ void __launch_bounds__(kThreads) k_diff_shade(const DiffArgs a) {
  const DiffView& vw = a.views[blockIdx.y];
  const int p = blockIdx.x * kThreads + threadIdx.x;
  float lp = 0.0f;
  if (p < vw.W * vw.H) {
    const size_t gp = (size_t)vw.pix_base + (size_t)p;
    const uint32_t gf = a.ids[gp];
    DiffRecord rec{kNoFace, kNoFace, 0.0f, 0.0f};
    float4 out = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (gf != kNoFace) {
      const int f = (int)(gf - vw.face_base);
      FaceGeom g;
      face_geom(a, blockIdx.y, f, p % vw.W, p / vw.W, g);
      if (g.ok) {
        // the visibility pass snaps corners to whole pixels, so a pixel may lie
        // just outside the unsnapped face: its barycentrics are clipped to it
        const float l0 = g.m[0] / g.M, l1 = g.m[1] / g.M;
        uint32_t texel = kNoFace;
        if (a.tex && a.uv) {
          const float l2 = 1.0f - l0 - l1;
          const float* uv = a.uv + 6 * (size_t)f;
          const float u = l0 * __ldg(uv) + l1 * __ldg(uv + 2) + l2 * __ldg(uv + 4);
          const float v = l0 * __ldg(uv + 1) + l1 * __ldg(uv + 3) + l2 * __ldg(uv + 5);
          texel = (uint32_t)(wrap_index(v, a.th) * a.tw + wrap_index(u, a.tw));
        }
        Shade s;
        shade(a, g, l0, l1, texel, a.nidx + 3 * (size_t)f, s);
        out = s.out;
        rec = DiffRecord{gf, texel, l0, l1};
      }
    }
    a.rec[gp] = rec;
    if (a.image) reinterpret_cast<float4*>(a.image)[gp] = out;
    const float4 tg = reinterpret_cast<const float4*>(a.target)[gp];
    const float dx = out.x - tg.x, dy = out.y - tg.y, dz = out.z - tg.z, dw = out.w - tg.w;
    lp = dx * dx + dy * dy + dz * dz + dw * dw;
  }
  // the loss in FP64: within the warp, then one atomic into the warp's slot
  // (k_diff_sum adds the slots up), so warps never wait for each other
  double t = (double)lp;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if ((threadIdx.x & 31) == 0 && t != 0.0) atomicAdd(a.partials + 4 * diff_slot(), t);
}

// Backward: gradients of the loss of the last forward pass.
__global__ void __launch_bounds__(kThreads) k_diff_grad(const DiffArgs a) {
  const DiffView& vw = a.views[blockIdx.y];
  const int p = blockIdx.x * kThreads + threadIdx.x;
  float gl[3] = {0.0f, 0.0f, 0.0f};
  if (p < vw.W * vw.H) {
    const size_t gp = (size_t)vw.pix_base + (size_t)p;
    const DiffRecord rec = a.rec[gp];
    if (rec.face != kNoFace) {
      const int f = (int)(rec.face - vw.face_base);
      const int px = p % vw.W, py = p / vw.W;
      FaceGeom g;
      face_geom(a, blockIdx.y, f, px, py, g);
      const int* ni = a.nidx + 3 * (size_t)f;
      Shade s;
      shade(a, g, rec.l0, rec.l1, rec.texel, ni, s);
      const float4 tg = reinterpret_cast<const float4*>(a.target)[gp];
      const float go[4] = {2.0f * (s.out.x - tg.x), 2.0f * (s.out.y - tg.y), 2.0f * (s.out.z - tg.z),
                           2.0f * (s.out.w - tg.w)};
      const float t3[3] = {s.t.x, s.t.y, s.t.z};
      // texels
      if (rec.texel != kNoFace)
        atomicAdd(reinterpret_cast<float4*>(a.g_tex) + rec.texel,
                  make_float4(go[0] * s.I * s.col[0], go[1] * s.I * s.col[1], go[2] * s.I * s.col[2], go[3]));
      // vertex colours, and d loss / d intensity
      float dI = 0.0f;
#pragma unroll
      for (int ch = 0; ch < 3; ++ch) dI += go[ch] * s.col[ch] * t3[ch];
      // colour and position gradients go to the face's corners first
      // (k_diff_scatter adds them to the vertices): a vertex is shared by
      // about six faces, so per-face sums meet far fewer atomics at one
      // address (measured: the backward pass 20 % faster).  Each corner's six
      // sums are two float4 (padded to eight floats), and the texel's four
      // one float4: seven vector reductions a pixel instead of 22 scalar ones
      // (the 64-view workload's backward 0.79 -> 0.47 ms; spreading a warp's
      // lanes over different faces instead made it slower, 0.90 ms)
      float4* gf = reinterpret_cast<float4*>(a.g_face + 24 * (size_t)f);
      // light: dI/dL = sum_k l_k 0.5 nhat_k
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float4 n = ldg4(a.nhat + 4 * (size_t)__ldg(ni + k));
        const float w = dI * 0.5f * s.l[k];
        gl[0] += w * n.x;
        gl[1] += w * n.y;
        gl[2] += w * n.z;
      }
      // positions through the barycentrics: G_k = d loss / d l_k
      float G[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        float gk = dI * s.Ii[k];
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) gk += go[ch] * s.I * t3[ch] * s.c[k][ch];
        G[k] = gk;
      }
      // l_k = m_k / M, m_k = max(s D_k, 0): d l / d D_j = s [m_j > 0] (G_j - G.l) / M
      const float Gl = G[0] * s.l[0] + G[1] * s.l[1] + G[2] * s.l[2];
      float dD[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) dD[k] = g.m[k] > 0.0f ? g.sg * (G[k] - Gl) / g.M : 0.0f;
      // D_0 = u1 v2 - u2 v1, D_1 = u2 v0 - u0 v2, D_2 = u0 v1 - u1 v0
      const float gu[3] = {dD[2] * g.v[1] - dD[1] * g.v[2], dD[0] * g.v[2] - dD[2] * g.v[0],
                           dD[1] * g.v[0] - dD[0] * g.v[1]};
      const float gv[3] = {dD[1] * g.u[2] - dD[2] * g.u[1], dD[2] * g.u[0] - dD[0] * g.u[2],
                           dD[0] * g.u[1] - dD[1] * g.u[0]};
      // u_k = (Q_0 - x Q_3) . p_k, v_k = (Q_1 - y Q_3) . p_k
      const float4 A = a.col_tab[vw.col_base + px];
      const float4 B = a.row_tab[vw.row_base + py];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        atomicAdd(gf + 2 * k, make_float4(go[0] * s.I * t3[0] * s.l[k], go[1] * s.I * t3[1] * s.l[k],
                                          go[2] * s.I * t3[2] * s.l[k], gu[k] * A.x + gv[k] * B.x));
        atomicAdd(gf + 2 * k + 1, make_float4(gu[k] * A.y + gv[k] * B.y, gu[k] * A.z + gv[k] * B.z, 0.0f, 0.0f));
      }
    }
  }
  // light gradient: float sums within the warp, then FP64 atomics into the
  // warp's slot (k_diff_sum adds the slots up)
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    gl[0] += __shfl_xor_sync(0xffffffffu, gl[0], o);
    gl[1] += __shfl_xor_sync(0xffffffffu, gl[1], o);
    gl[2] += __shfl_xor_sync(0xffffffffu, gl[2], o);
  }
  if ((threadIdx.x & 31) == 0) {
    double* p = a.partials + 4 * diff_slot();
#pragma unroll
    for (int j = 0; j < 3; ++j)
      if (gl[j] != 0.0f) atomicAdd(p + 1 + j, (double)gl[j]);
  }
}

// Adds every face's corner sums (k_diff_grad) to its vertices' colour and
// position gradients and returns the sums to zero.  One thread per face.
__global__ void __launch_bounds__(kThreads) k_diff_scatter(const DiffArgs a) {
  const int f = blockIdx.x * kThreads + threadIdx.x;
  if (f >= a.nf) return;
  float* gf = a.g_face + 24 * (size_t)f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const int v = __ldg(a.vidx + 3 * (size_t)f + k);
#pragma unroll
    for (int j = 0; j < 6; ++j) {
      const float x = gf[8 * k + j];
      if (x == 0.0f) continue;
      gf[8 * k + j] = 0.0f;
      if (j < 3) atomicAdd(a.g_vcol + 3 * (size_t)v + j, x);
      else atomicAdd(a.g_pos + 4 * (size_t)v + (j - 3), x);
    }
  }
}

// Writes the sums of components [c0, c0 + n) of the per-warp slots to
// dst[0 .. n) (page-locked host memory, through its device address: no copy
// follows) and returns the slots to zero.  One block of kDiffSlots threads.
__global__ void __launch_bounds__(kDiffSlots) k_diff_sum(const DiffArgs a, int c0, int n, double* dst) {
  __shared__ double s_w[kDiffSlots / 32];
  for (int j = 0; j < n; ++j) {
    double* p = a.partials + 4 * threadIdx.x + c0 + j;
    double t = *p;
    *p = 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
      double sum = 0.0;
      for (int w = 0; w < kDiffSlots / 32; ++w) sum += s_w[w];
      dst[j] = sum;
    }
    __syncthreads();
  }
}

}  // namespace

int launch_diff_bbox(const float* pos, int nv, DevItem* items, int num_items, float* partial, unsigned* done,
                     void* stream) {
  if (nv <= 0 || num_items <= 0) return 0;
  const int blocks = std::min(kBBoxBlocks, (nv + 1023) / 1024);
  k_diff_bbox<<<blocks, 1024, 0, (cudaStream_t)stream>>>(pos, nv, items, num_items, partial, done);
  return (int)cudaGetLastError();
}

int launch_diff_normals(const float* world, const float* vnrm, int nn, float* nhat, void* stream) {
  if (nn <= 0) return 0;
  k_diff_normals<<<(nn + kThreads - 1) / kThreads, kThreads, 0, (cudaStream_t)stream>>>(world, vnrm, nn, nhat);
  return (int)cudaGetLastError();
}

int launch_diff_forward(const DiffArgs& a, int max_side, void* stream) {
  cudaStream_t s = (cudaStream_t)stream;
  k_diff_vertices<<<dim3((unsigned)((a.nv + kThreads - 1) / kThreads), (unsigned)a.num_views), kThreads, 0, s>>>(a);
  k_diff_tables<<<dim3((unsigned)((max_side + kThreads - 1) / kThreads), (unsigned)a.num_views), kThreads, 0, s>>>(a);
  const dim3 grid((unsigned)((a.max_pixels + kThreads - 1) / kThreads), (unsigned)a.num_views);
  k_diff_shade<<<grid, kThreads, 0, s>>>(a);
  k_diff_sum<<<1, kDiffSlots, 0, s>>>(a, 0, 1, a.loss);
  return (int)cudaGetLastError();
}

int launch_diff_backward(const DiffArgs& a, void* stream) {
  const dim3 grid((unsigned)((a.max_pixels + kThreads - 1) / kThreads), (unsigned)a.num_views);
  k_diff_grad<<<grid, kThreads, 0, (cudaStream_t)stream>>>(a);
  k_diff_scatter<<<(unsigned)((a.nf + kThreads - 1) / kThreads), kThreads, 0, (cudaStream_t)stream>>>(a);
  k_diff_sum<<<1, kDiffSlots, 0, (cudaStream_t)stream>>>(a, 1, 3, a.g_light);
  return (int)cudaGetLastError();
}

}  // namespace gr
