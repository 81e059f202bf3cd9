/*
 * gorender_oracle.c -- CPU restatement of gorender's frame pipeline.
 *
 * TEST INFRASTRUCTURE ONLY (the checker).  See gorender_oracle.h for the
 * contract and the parity status ("parity unpinned": the reference ships no
 * golden vectors and cannot be built here).
 *
 * Build: cc -O2 -ffp-contract=off -fno-fast-math -fPIC -shared -pthread.
 * Every float expression below is written in the reference's source order so
 * that, with contraction disabled, each operation rounds exactly as Go's SSE
 * scalar code does.  References are file:line into the Go sources.
 */
#include "gorender_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef struct { float x, y, z, w; } V4;
typedef struct { float x, y, z; } V3;
typedef struct { float u, v; } UV;

/* ------------------------------------------------------------------ */
/* Go amd64 conversion semantics                                       */
/* ------------------------------------------------------------------ */

/* int(float32) compiles to CVTTSS2SQ: truncation toward zero; NaN and values
 * outside [-2^63, 2^63) give the "integer indefinite" value INT64_MIN. */
int64_t orc_go_int(float f) {
  if (f >= -9223372036854775808.0f && f < 9223372036854775808.0f) return (int64_t)f;
  return INT64_MIN;
}

/* uint8(float32) converts through int32 (CVTTSS2SL, indefinite 0x80000000)
 * and keeps the low byte (rasterizer.go:83-85). */
uint8_t orc_go_uint8(float f) {
  if (f >= -2147483648.0f && f < 2147483648.0f) return (uint8_t)(uint32_t)(int32_t)f;
  return 0;
}

/* Go `int` arithmetic wraps modulo 2^64. */
static inline int64_t wadd(int64_t a, int64_t b) { return (int64_t)((uint64_t)a + (uint64_t)b); }
static inline int64_t wsub(int64_t a, int64_t b) { return (int64_t)((uint64_t)a - (uint64_t)b); }
static inline int64_t wmul(int64_t a, int64_t b) { return (int64_t)((uint64_t)a * (uint64_t)b); }
static inline int64_t imin(int64_t a, int64_t b) { return a < b ? a : b; }
static inline int64_t imax(int64_t a, int64_t b) { return a > b ? a : b; }

/* sqrt32 (math32.go:11-13): float32(math.Sqrt(float64(x))). */
static inline float sqrt32(float x) { return (float)sqrt((double)x); }

/* ------------------------------------------------------------------ */
/* vector.go                                                           */
/* ------------------------------------------------------------------ */

static inline V3 v3sub(V3 a, V3 b) { V3 r = {a.x - b.x, a.y - b.y, a.z - b.z}; return r; }
static inline V3 v3cross(V3 a, V3 b) {      /* vector.go:55-60 */
  V3 r;
  r.x = a.y * b.z - a.z * b.y;
  r.y = a.z * b.x - a.x * b.z;
  r.z = a.x * b.y - a.y * b.x;
  return r;
}
static inline float v3dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }  /* vector.go:62-64 */
static inline V3 v3normalize(V3 v) {        /* vector.go:51-53, 66-68, 78-80 */
  float len = sqrt32(v.x * v.x + v.y * v.y + v.z * v.z);
  V3 r = {v.x / len, v.y / len, v.z / len};
  return r;
}
static inline V3 v4to3(V4 v) { V3 r = {v.x, v.y, v.z}; return r; }
static inline V4 v4add(V4 a, V4 b) { V4 r = {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; return r; }
static inline V4 v4sub(V4 a, V4 b) { V4 r = {a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; return r; }
static inline V4 v4mul(V4 a, float s) { V4 r = {a.x * s, a.y * s, a.z * s, a.w * s}; return r; }
static inline V4 v4div(V4 a, float s) { V4 r = {a.x / s, a.y / s, a.z / s, a.w / s}; return r; }
static inline float v4dot(V4 a, V4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
static inline V4 v4normalize(V4 v) {        /* vector.go:115-125: length includes w */
  float len = sqrt32(v.x * v.x + v.y * v.y + v.z * v.z + v.w * v.w);
  return v4div(v, len);
}

void orc_normalize3(const float* v, float* out) {
  V3 a = {v[0], v[1], v[2]};
  V3 r = v3normalize(a);
  out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

/* ------------------------------------------------------------------ */
/* matrix.go                                                           */
/* ------------------------------------------------------------------ */

/* matrixMultiplyVec4Inplace (matrix.go:167-173) and the batch transform
 * (asm_purego.go:11-17; asm_amd64.s:24-42 sums ((x*c0 + y*c1) + z*c2) + w*c3,
 * the same order). */
static inline V4 mat_vec(const float* m, V4 v) {
  V4 r;
  r.x = m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3] * v.w;
  r.y = m[4] * v.x + m[5] * v.y + m[6] * v.z + m[7] * v.w;
  r.z = m[8] * v.x + m[9] * v.y + m[10] * v.z + m[11] * v.w;
  r.w = m[12] * v.x + m[13] * v.y + m[14] * v.z + m[15] * v.w;
  return r;
}

void orc_transform_batch(const float* m, float* vecs, int64_t n) {
  for (int64_t i = 0; i < n; i++) {
    V4 v = {vecs[4 * i], vecs[4 * i + 1], vecs[4 * i + 2], vecs[4 * i + 3]};
    V4 r = mat_vec(m, v);
    vecs[4 * i] = r.x; vecs[4 * i + 1] = r.y; vecs[4 * i + 2] = r.z; vecs[4 * i + 3] = r.w;
  }
}

/* Matrix.Multiply (matrix.go:155-165): res[i][j] accumulates from zero. */
void orc_matrix_multiply(const float* a, const float* b, float* out) {
  float res[16];
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) {
      float acc = 0.0f;
      for (int k = 0; k < 4; k++) acc += a[i * 4 + k] * b[k * 4 + j];
      res[i * 4 + j] = acc;
    }
  memcpy(out, res, sizeof(res));
}

static void mat_identity(float* m) {
  memset(m, 0, 16 * sizeof(float));
  m[0] = m[5] = m[10] = m[15] = 1.0f;
}

/* ---- Go's math.Sin / math.Cos / math.Tan (math32.go:15-25 call them on
 * float64(x)).  On amd64 these are pure Go (no assembly), compiled without FMA
 * fusion: the Cephes library's sin.c / tan.c algorithm (S. L. Moshier) as Go's
 * math package restates it.  Argument reduction by pi/4: below 2^29 the
 * Cody-Waite three-part split of pi/4, above it the Payne-Hanek reduction
 * (K. C. Ng, "Argument reduction for huge arguments: good to the last bit",
 * 1992) with 64-bit words of 4/pi; then the Cephes minimax polynomials on
 * [-pi/4, pi/4] (sin: degree 13 odd, cos: degree 14 even, tan: a 3/4
 * rational in z^2).  glibc's sin/cos/tan are a different algorithm and differ
 * from Go's in the last bit of the double for about a quarter of arguments,
 * which can survive the float32 rounding.  Evaluated in the order Go writes
 * the expressions; this file is built with -ffp-contract=off. */
static const double GO_PI4A = 7.85398125648498535156e-1;  /* pi/4 = A + B + C */
static const double GO_PI4B = 3.77489470793079817668e-8;
static const double GO_PI4C = 2.69515142907905952645e-15;
static const double GO_4_OVER_PI = 0x1.45f306dc9c883p+0;  /* 4/pi correctly rounded */
static const double GO_PI4 = 0x1.921fb54442d18p-1;        /* pi/4 correctly rounded */
static const double GO_REDUCE_THRESHOLD = 536870912.0;    /* 2^29 */
static const double GO_SIN[6] = {1.58962301576546568060e-10, -2.50507477628578072866e-8,
                                 2.75573136213857245213e-6,  -1.98412698295895385996e-4,
                                 8.33333333332211858878e-3,  -1.66666666666666307295e-1};
static const double GO_COS[6] = {-1.13585365213876817300e-11, 2.08757008419747316778e-9,
                                 -2.75573141792967388112e-7,  2.48015872888517045348e-5,
                                 -1.38888888888730564116e-3,  4.16666666666665929218e-2};
static const double GO_TANP[3] = {-1.30936939181383777646e4, 1.15351664838587416140e6,
                                  -1.79565251976484877988e7};
static const double GO_TANQ[5] = {1.0, 1.36812963470692954678e4, -1.32089234440210967447e6,
                                  2.50083801823357915839e7, -5.38695755929454629881e7};
/* 4/pi = sum_i W[i] * 2^(-64 i): its binary digits, computed from pi to 700
 * digits.  Eight words cover every float64 converted from a float32
 * (exponent <= 127); math32.go only ever passes those. */
static const uint64_t GO_4PI_BITS[8] = {
    0x0000000000000001ull, 0x45f306dc9c882a53ull, 0xf84eafa3ea69bb81ull, 0xb6c52b3278872083ull,
    0xfca2c757bd778ac3ull, 0x6e48dc74849ba5c0ull, 0x0c925dd413a32439ull, 0xfc3bd63962534e7dull};

static inline uint64_t dbits(double x) { uint64_t u; memcpy(&u, &x, 8); return u; }
static inline double dfrom(uint64_t u) { double x; memcpy(&x, &u, 8); return x; }
static inline uint64_t shl64(uint64_t v, unsigned n) { return n >= 64 ? 0 : v << n; }
static inline uint64_t shr64(uint64_t v, unsigned n) { return n >= 64 ? 0 : v >> n; }

/* Payne-Hanek: x >= 2^29 -> octant j (0..7, zeros mapped to the origin) and
 * the reduced argument z in [-pi/4, pi/4]. */
static void go_trig_reduce(double x, uint64_t* j_out, double* z_out) {
  if (x < GO_PI4) { *j_out = 0; *z_out = x; return; }
  uint64_t ix = dbits(x);
  const int exp = (int)((ix >> 52) & 0x7FF) - 1023 - 52;  /* x = mantissa * 2^exp */
  ix &= ~(0x7FFull << 52);
  ix |= 1ull << 52;
  const unsigned digit = (unsigned)(exp + 61) / 64, bitshift = (unsigned)(exp + 61) % 64;
  const uint64_t z0 = shl64(GO_4PI_BITS[digit], bitshift) | shr64(GO_4PI_BITS[digit + 1], 64 - bitshift);
  const uint64_t z1 = shl64(GO_4PI_BITS[digit + 1], bitshift) | shr64(GO_4PI_BITS[digit + 2], 64 - bitshift);
  const uint64_t z2 = shl64(GO_4PI_BITS[digit + 2], bitshift) | shr64(GO_4PI_BITS[digit + 3], 64 - bitshift);
  const unsigned __int128 p2 = (unsigned __int128)z2 * ix, p1 = (unsigned __int128)z1 * ix;
  const uint64_t z2hi = (uint64_t)(p2 >> 64), z1hi = (uint64_t)(p1 >> 64), z1lo = (uint64_t)p1;
  const uint64_t z0lo = z0 * ix;
  const uint64_t lo = z1lo + z2hi;
  const uint64_t carry = lo < z1lo;
  uint64_t hi = z0lo + z1hi + carry;
  uint64_t j = hi >> 61;
  hi = hi << 3 | lo >> 61;
  const unsigned lz = hi ? (unsigned)__builtin_clzll(hi) : 64;
  const uint64_t e = (uint64_t)(1023 - (lz + 1));
  hi = shl64(hi, lz + 1) | shr64(lo, 64 - (lz + 1));
  hi >>= 64 - 52;
  hi |= e << 52;
  double z = dfrom(hi);
  if (j & 1) { j++; j &= 7; z = z - 1.0; }
  *j_out = j;
  *z_out = z * GO_PI4;
}

/* x >= 0 below 2^29: octant (odd ones rounded up) and the reduced argument. */
static void go_reduce(double x, uint64_t* j_out, double* z_out) {
  if (x >= GO_REDUCE_THRESHOLD) { go_trig_reduce(x, j_out, z_out); return; }
  uint64_t j = (uint64_t)(x * GO_4_OVER_PI);
  double y = (double)j;
  if (j & 1) { j++; y++; }
  *j_out = j;
  *z_out = ((x - y * GO_PI4A) - y * GO_PI4B) - y * GO_PI4C;
}

static inline double go_sin_poly(double z, double zz) {
  return z + z * zz * ((((((GO_SIN[0] * zz) + GO_SIN[1]) * zz + GO_SIN[2]) * zz + GO_SIN[3]) * zz + GO_SIN[4]) * zz + GO_SIN[5]);
}
static inline double go_cos_poly(double zz) {
  return 1.0 - 0.5 * zz + zz * zz * ((((((GO_COS[0] * zz) + GO_COS[1]) * zz + GO_COS[2]) * zz + GO_COS[3]) * zz + GO_COS[4]) * zz + GO_COS[5]);
}

double orc_go_sin(double x) {
  if (x == 0 || isnan(x)) return x;
  if (isinf(x)) return NAN;
  int sign = 0;
  if (x < 0) { x = -x; sign = 1; }
  uint64_t j; double z;
  go_reduce(x, &j, &z);
  j &= 7;
  if (j > 3) { sign = !sign; j -= 4; }
  const double zz = z * z;
  const double y = (j == 1 || j == 2) ? go_cos_poly(zz) : go_sin_poly(z, zz);
  return sign ? -y : y;
}

double orc_go_cos(double x) {
  if (isnan(x) || isinf(x)) return NAN;
  int sign = 0;
  x = fabs(x);
  uint64_t j; double z;
  go_reduce(x, &j, &z);
  j &= 7;
  if (j > 3) { j -= 4; sign = !sign; }
  if (j > 1) sign = !sign;
  const double zz = z * z;
  const double y = (j == 1 || j == 2) ? go_sin_poly(z, zz) : go_cos_poly(zz);
  return sign ? -y : y;
}

double orc_go_tan(double x) {
  if (x == 0 || isnan(x)) return x;
  if (isinf(x)) return NAN;
  int sign = 0;
  if (x < 0) { x = -x; sign = 1; }
  uint64_t j; double z;
  go_reduce(x, &j, &z);
  const double zz = z * z;
  double y;
  if (zz > 1e-14)
    y = z + z * (zz * (((GO_TANP[0] * zz) + GO_TANP[1]) * zz + GO_TANP[2]) /
                 ((((zz + GO_TANQ[1]) * zz + GO_TANQ[2]) * zz + GO_TANQ[3]) * zz + GO_TANQ[4]));
  else
    y = z;
  if (j & 2) y = -1 / y;
  return sign ? -y : y;
}

static inline float sin32(float x) { return (float)orc_go_sin((double)x); }  /* math32.go:15-17 */
static inline float cos32(float x) { return (float)orc_go_cos((double)x); }  /* math32.go:19-21 */
static inline float tan32(float x) { return (float)orc_go_tan((double)x); }  /* math32.go:23-25 */

static void rot_x(float a, float* m) {      /* matrix.go:32-44 */
  mat_identity(m);
  if (a == 0) return;
  float s = sin32(a), c = cos32(a);
  m[5] = c; m[6] = -s; m[9] = s; m[10] = c;
}
static void rot_y(float a, float* m) {      /* matrix.go:46-58 */
  mat_identity(m);
  if (a == 0) return;
  float s = sin32(a), c = cos32(a);
  m[0] = c; m[2] = s; m[8] = -s; m[10] = c;
}
static void rot_z(float a, float* m) {      /* matrix.go:60-72 */
  mat_identity(m);
  if (a == 0) return;
  float s = sin32(a), c = cos32(a);
  m[0] = c; m[1] = -s; m[4] = s; m[5] = c;
}

void orc_world_matrix(const float* scale3, const float* rot3, const float* trans3, float* out) {
  float m[16], t[16], r[16], rx[16], ry[16], rz[16];
  mat_identity(m);                                        /* matrix.go:83 */
  mat_identity(t);                                        /* NewScaleMatrix */
  t[0] = scale3[0]; t[5] = scale3[1]; t[10] = scale3[2];
  orc_matrix_multiply(t, m, m);                           /* matrix.go:84 */
  mat_identity(r);                                        /* NewRotationMatrix, matrix.go:74-80 */
  rot_x(rot3[0], rx); rot_y(rot3[1], ry); rot_z(rot3[2], rz);
  orc_matrix_multiply(r, rx, r);
  orc_matrix_multiply(r, ry, r);
  orc_matrix_multiply(r, rz, r);
  orc_matrix_multiply(r, m, m);                           /* matrix.go:85 */
  mat_identity(t);                                        /* NewTranslationMatrix */
  t[3] = trans3[0]; t[7] = trans3[1]; t[11] = trans3[2];
  orc_matrix_multiply(t, m, out);                         /* matrix.go:86 */
}

void orc_view_matrix(const float* eye3, const float* dir3, const float* up3, float* out) {
  V3 eye = {eye3[0], eye3[1], eye3[2]};
  V3 dir = {dir3[0], dir3[1], dir3[2]};
  V3 up = {up3[0], up3[1], up3[2]};
  V3 z = v3normalize(dir);                                /* matrix.go:134 */
  V3 x = v3normalize(v3cross(up, z));                     /* matrix.go:135 */
  V3 y = v3normalize(v3cross(z, x));                      /* matrix.go:136 */
  float m[16] = {x.x, x.y, x.z, -v3dot(x, eye),
                 y.x, y.y, y.z, -v3dot(y, eye),
                 z.x, z.y, z.z, -v3dot(z, eye),
                 0, 0, 0, 1};
  memcpy(out, m, sizeof(m));
}

void orc_perspective_matrix(float fov, float aspect, float znear, float zfar, float* out) {
  float tan_half = tan32(fov / 2.0f);                     /* matrix.go:93 */
  float m00 = 1 / (aspect * tan_half);
  float m11 = 1 / tan_half;
  float m22 = (zfar + znear) / (znear - zfar);
  float m23 = (2 * zfar * znear) / (znear - zfar);
  float m[16] = {m00, 0, 0, 0,
                 0, m11, 0, 0,
                 0, 0, -m22, -m23,
                 0, 0, -1, 0};
  memcpy(out, m, sizeof(m));
}

void orc_screen_matrix(int32_t width, int32_t height, float* out) {
  float hw = (float)width / 2;                            /* matrix.go:109-110 */
  float hh = (float)height / 2;
  float m[16] = {hw, 0, 0, hw,
                 0, hh, 0, hh,
                 0, 0, 0.5f, 0.5f,
                 0, 0, 0, 1};
  memcpy(out, m, sizeof(m));
}

/* ------------------------------------------------------------------ */
/* mesh.go                                                             */
/* ------------------------------------------------------------------ */

void orc_mesh_face_normals(const float* pos, const int32_t* vidx, int32_t nf, float* fnrm_out) {
  for (int32_t i = 0; i < nf; i++) {                      /* mesh.go:55-60 */
    const float* a = pos + 4 * (int64_t)vidx[3 * i];
    const float* b = pos + 4 * (int64_t)vidx[3 * i + 1];
    const float* c = pos + 4 * (int64_t)vidx[3 * i + 2];
    V3 v0 = {a[0], a[1], a[2]}, v1 = {b[0], b[1], b[2]}, v2 = {c[0], c[1], c[2]};
    V3 n = v3normalize(v3cross(v3sub(v1, v0), v3sub(v2, v0)));
    fnrm_out[4 * i] = n.x; fnrm_out[4 * i + 1] = n.y; fnrm_out[4 * i + 2] = n.z;
    fnrm_out[4 * i + 3] = 1.0f;                            /* Vec3.ToVec4: w = 1 */
  }
}

/* Go's builtin min/max on float32 return NaN when any argument is NaN. */
static inline float gomin(float a, float b) { return (a != a || b != b) ? NAN : (a < b ? a : (b < a ? b : (signbit(a) ? a : b))); }
static inline float gomax(float a, float b) { return (a != a || b != b) ? NAN : (a > b ? a : (b > a ? b : (signbit(a) ? b : a))); }

void orc_mesh_bbox(const float* pos, int32_t nv, float* out) {  /* mesh.go:28-51 */
  float minx = pos[0], miny = pos[1], minz = pos[2];
  float maxx = minx, maxy = miny, maxz = minz;
  for (int32_t i = 0; i < nv; i++) {
    const float* v = pos + 4 * (int64_t)i;
    minx = gomin(minx, v[0]); miny = gomin(miny, v[1]); minz = gomin(minz, v[2]);
    maxx = gomax(maxx, v[0]); maxy = gomax(maxy, v[1]); maxz = gomax(maxz, v[2]);
  }
  float b[8][4] = {{minx, miny, minz, 1}, {minx, miny, maxz, 1}, {minx, maxy, minz, 1},
                   {minx, maxy, maxz, 1}, {maxx, miny, minz, 1}, {maxx, miny, maxz, 1},
                   {maxx, maxy, minz, 1}, {maxx, maxy, maxz, 1}};
  memcpy(out, b, sizeof(b));
}

/* ------------------------------------------------------------------ */
/* clipping.go                                                         */
/* ------------------------------------------------------------------ */

#define MAX_CLIP 9   /* clipping.go:10 */

typedef struct { V4 point, normal; } Plane;

static void frustum_planes(float znear, float zfar, Plane p[6]) {  /* clipping.go:93-129 */
  Plane l = {{-1, 0, 0, 1}, {1, 0, 0, 1}};
  Plane r = {{1, 0, 0, 1}, {-1, 0, 0, 1}};
  Plane t = {{0, -1, 0, 1}, {0, 1, 0, 1}};
  Plane b = {{0, 1, 0, 1}, {0, -1, 0, 1}};
  Plane n = {{0, 0, znear, 1}, {0, 0, -1, 0}};
  Plane f = {{0, 0, zfar, 1}, {0, 0, 1, 0}};
  p[0] = l; p[1] = r; p[2] = t; p[3] = b; p[4] = n; p[5] = f;
}

static inline float plane_distance(const Plane* p, V4 v) {  /* clipping.go:69-71 */
  return v4dot(p->normal, v) - v4dot(p->normal, p->point);
}
static inline int plane_inside(const Plane* p, V4 q) {     /* clipping.go:74-76 */
  return v4dot(v4sub(q, p->point), p->normal) <= 0;
}
static inline V4 plane_intersect(const Plane* p, V4 q0, V4 q1, float* factor) {  /* 79-86 */
  V4 u = v4sub(q1, q0);
  V4 w = v4sub(q0, p->point);
  float d = v4dot(p->normal, u);
  float n = -v4dot(p->normal, w);
  *factor = n / d;
  return v4add(q0, v4mul(u, *factor));
}

int orc_box_visibility(const float* c, float znear, float zfar) {  /* clipping.go:131-154 */
  Plane pl[6];
  frustum_planes(znear, zfar, pl);
  for (int i = 0; i < 6; i++) {
    int outside = 0;
    for (int k = 0; k < 8; k++) {
      V4 pt = {c[4 * k], c[4 * k + 1], c[4 * k + 2], c[4 * k + 3]};
      if (plane_distance(&pl[i], pt) > 0) outside++;
    }
    if (outside == 8) return 0;   /* BoxVisibilityOutside */
    if (outside > 0) return 1;    /* BoxVisibilityIntersect */
  }
  return 2;                       /* BoxVisibilityInside */
}

typedef struct {
  float inten[MAX_CLIP];
  V4 pts[MAX_CLIP];
  UV uvs[MAX_CLIP];
  V3 col[MAX_CLIP];   /* per-vertex RGB extension, lerped like intensity */
  int count;
} Poly;

static inline int poly_add(Poly* p, V4 v, UV uv, float in, V3 col) {  /* clipping.go:35-40 */
  if (p->count >= MAX_CLIP) return -1;   /* Go would panic: index out of range */
  p->inten[p->count] = in;
  p->pts[p->count] = v;
  p->uvs[p->count] = uv;
  p->col[p->count] = col;
  p->count++;
  return 0;
}

typedef struct { V4 p[3]; UV uv[3]; float in[3]; V3 col[3]; } ClipTri;

static inline float lerp32(float a, float b, float f) { return a + (b - a) * f; }  /* 163-165 */

/* Frustum.ClipTriangle (clipping.go:167-236).  Returns count or -3. */
static int clip_triangle(const Plane* planes, const V4* pin, const UV* uvin, const float* inin,
                         const V3* colin, ClipTri* out) {
  Poly a, b;
  Poly* poly = &a;
  Poly* poly2 = &b;
  poly->count = 0;
  for (int i = 0; i < 3; i++) poly_add(poly, pin[i], uvin[i], inin[i], colin[i]);
  for (int pi = 0; pi < 6; pi++) {
    const Plane* plane = &planes[pi];
    poly2->count = 0;
    for (int bi = 0; bi < poly->count; bi++) {
      int ai = (bi + 1) % poly->count;
      UV uvA = poly->uvs[ai], uvB = poly->uvs[bi];
      V4 vA = poly->pts[ai], vB = poly->pts[bi];
      float iA = poly->inten[ai], iB = poly->inten[bi];
      V3 cA = poly->col[ai], cB = poly->col[bi];
      if (plane_inside(plane, vA)) {
        if (!plane_inside(plane, vB)) {
          float f;
          V4 x = plane_intersect(plane, vA, vB, &f);
          float in = lerp32(iA, iB, f);
          UV uv = {uvA.u + (uvB.u - uvA.u) * f, uvA.v + (uvB.v - uvA.v) * f};
          V3 c = {lerp32(cA.x, cB.x, f), lerp32(cA.y, cB.y, f), lerp32(cA.z, cB.z, f)};
          if (poly_add(poly2, x, uv, in, c)) return -3;
        }
        if (poly_add(poly2, vA, uvA, iA, cA)) return -3;
      } else if (plane_inside(plane, vB)) {
        float f;
        V4 x = plane_intersect(plane, vA, vB, &f);
        float in = lerp32(iA, iB, f);
        UV uv = {uvA.u + (uvB.u - uvA.u) * f, uvA.v + (uvB.v - uvA.v) * f};
        V3 c = {lerp32(cA.x, cB.x, f), lerp32(cA.y, cB.y, f), lerp32(cA.z, cB.z, f)};
        if (poly_add(poly2, x, uv, in, c)) return -3;
      }
    }
    if (poly2->count == 0) return 0;
    Poly* t = poly; poly = poly2; poly2 = t;
  }
  if (poly->count < 3) return 0;                        /* Polygon.Triangulate, 42-62 */
  int n = 0;
  for (int i = 0; i < poly->count - 2; i++) {
    int k[3] = {0, i + 1, i + 2};
    for (int j = 0; j < 3; j++) {
      out[n].p[j] = poly->pts[k[j]];
      out[n].uv[j] = poly->uvs[k[j]];
      out[n].in[j] = poly->inten[k[j]];
      out[n].col[j] = poly->col[k[j]];
    }
    n++;
  }
  return n;
}

int orc_clip_triangle(const float* pts, const float* uvs, const float* inten, const float* col,
                      float znear, float zfar, float* pts_out, float* uv_out, float* inten_out,
                      float* col_out) {
  Plane pl[6];
  frustum_planes(znear, zfar, pl);
  V4 p[3]; UV uv[3]; float in[3]; V3 c[3];
  for (int i = 0; i < 3; i++) {
    V4 v = {pts[4 * i], pts[4 * i + 1], pts[4 * i + 2], pts[4 * i + 3]};
    p[i] = v;
    uv[i].u = uvs[2 * i]; uv[i].v = uvs[2 * i + 1];
    in[i] = inten[i];
    if (col) { c[i].x = col[3 * i]; c[i].y = col[3 * i + 1]; c[i].z = col[3 * i + 2]; }
    else { c[i].x = c[i].y = c[i].z = 0; }
  }
  ClipTri out[MAX_CLIP];
  int n = clip_triangle(pl, p, uv, in, c, out);
  for (int t = 0; t < n; t++)
    for (int j = 0; j < 3; j++) {
      float* po = pts_out + (t * 3 + j) * 4;
      po[0] = out[t].p[j].x; po[1] = out[t].p[j].y; po[2] = out[t].p[j].z; po[3] = out[t].p[j].w;
      uv_out[(t * 3 + j) * 2] = out[t].uv[j].u;
      uv_out[(t * 3 + j) * 2 + 1] = out[t].uv[j].v;
      inten_out[t * 3 + j] = out[t].in[j];
      if (col_out) {
        col_out[(t * 3 + j) * 3] = out[t].col[j].x;
        col_out[(t * 3 + j) * 3 + 1] = out[t].col[j].y;
        col_out[(t * 3 + j) * 3 + 2] = out[t].col[j].z;
      }
    }
  return n;
}

/* ------------------------------------------------------------------ */
/* texture.go / rasterizer.go                                          */
/* ------------------------------------------------------------------ */

static const uint8_t kFaceColor[4] = {200, 200, 200, 255};  /* renderer.go:17 */

void orc_texture_sample(const orc_texture* t, float u, float v, uint8_t* out) {  /* texture.go:69-89 */
  switch (t->type) {
    case ORC_TEX_SOLID:
      memcpy(out, t->color, 4);
      return;
    case ORC_TEX_IMAGE_FAST: {
      float wf = (float)t->width, hf = (float)t->height;
      int64_t x = orc_go_int((1 - u) * t->scale * wf) & (int64_t)(t->width - 1);
      int64_t y = orc_go_int(v * t->scale * hf) & (int64_t)(t->height - 1);
      memcpy(out, t->pixels + 4 * (y * t->width + x), 4);
      return;
    }
    case ORC_TEX_IMAGE: {
      float wf = (float)t->width, hf = (float)t->height;
      int64_t x = orc_go_int((1 - u) * t->scale * wf) % (int64_t)t->width;
      int64_t y = orc_go_int(v * t->scale * hf) % (int64_t)t->height;
      int64_t idx = y * t->width + x;
      if (idx < 0) idx = 0;
      memcpy(out, t->pixels + 4 * idx, 4);
      return;
    }
    default: {
      uint8_t m[4] = {255, 0, 255, 255};
      memcpy(out, m, 4);
    }
  }
}

/* Shading inputs of one binned triangle (the Triangle struct of
 * renderer.go:29-34 after drawProjection's int() conversions). */
typedef struct {
  int64_t x[3], y[3];
  float w[3];
  float u[3], v[3];
  float in[3];
  float col[3][3];
  int32_t tex;      /* -1 = nil */
  int32_t has_col;  /* per-vertex RGB extension active */
  uint32_t face;    /* global face index: earlier objects' faces + face index */
  float sx[3], sy[3];  /* screen coordinates before int() (the centroid mark uses them) */
} RTri;

/* FrameBuffer.Triangle (rasterizer.go:90-183) restricted to rows
 * [band_y0, band_y1).  With the full band this is the reference loop.  The
 * per-vertex colour extension replaces faceColor by the interpolated RGB. */
static void raster_tri(uint8_t* rgba, float* zb, uint32_t* ids, int32_t width, int32_t height, const RTri* t,
                       int64_t tsx, int64_t tsy, int64_t tex_, int64_t tey,
                       const orc_texture* texture, int64_t band_y0, int64_t band_y1) {
  int64_t x0 = t->x[0], y0 = t->y[0], x1 = t->x[1], y1 = t->y[1], x2 = t->x[2], y2 = t->y[2];
  float z0 = t->w[0], z1 = t->w[1], z2 = t->w[2];
  int64_t minX = imin(imin(x0, x1), x2), maxX = imax(imax(x0, x1), x2);
  int64_t minY = imin(imin(y0, y1), y2), maxY = imax(imax(y0, y1), y2);
  minX = imax(imax(minX, tsx), 0); maxX = imin(imin(maxX, tex_), (int64_t)width - 1);
  minY = imax(imax(minY, tsy), 0); maxY = imin(imin(maxY, tey), (int64_t)height - 1);
  if (minY < band_y0) minY = band_y0;
  if (maxY > band_y1 - 1) maxY = band_y1 - 1;

  int64_t f01 = wadd(wadd(wmul(wsub(y0, y1), minX), wmul(wsub(x1, x0), minY)), wsub(wmul(x0, y1), wmul(x1, y0)));
  int64_t f12 = wadd(wadd(wmul(wsub(y1, y2), minX), wmul(wsub(x2, x1), minY)), wsub(wmul(x1, y2), wmul(x2, y1)));
  int64_t f20 = wadd(wadd(wmul(wsub(y2, y0), minX), wmul(wsub(x0, x2), minY)), wsub(wmul(x2, y0), wmul(x0, y2)));
  int64_t f01dx = wsub(y0, y1), f01dy = wsub(x1, x0);
  int64_t f12dx = wsub(y1, y2), f12dy = wsub(x2, x1);
  int64_t f20dx = wsub(y2, y0), f20dy = wsub(x0, x2);
  /* top-left rule (rasterizer.go:120-129) */
  if (!(f01dy > 0 || (f01dy == 0 && f01dx > 0))) f01 = wsub(f01, 1);
  if (!(f12dy > 0 || (f12dy == 0 && f12dx > 0))) f12 = wsub(f12, 1);
  if (!(f20dy > 0 || (f20dy == 0 && f20dx > 0))) f20 = wsub(f20, 1);

  float v0z0 = t->v[0] / z0, u0z0 = t->u[0] / z0;
  float u1z1 = t->u[1] / z1, v1z1 = t->v[1] / z1;
  float u2z2 = t->u[2] / z2, v2z2 = t->v[2] / z2;

  for (int64_t y = minY; y <= maxY; y++) {
    int64_t fx01 = f01, fx12 = f12, fx20 = f20;
    for (int64_t x = minX; x <= maxX; x++) {
      if (fx01 < 0 && fx12 < 0 && fx20 < 0) {
        int64_t s = wadd(wadd(fx12, fx20), fx01);
        float alpha = (float)fx12 / (float)s;
        float beta = (float)fx20 / (float)s;
        float gamma = 1 - alpha - beta;
        float zRec = -(alpha / z0 + beta / z1 + gamma / z2);
        int64_t index = y * width + x;
        if (zRec >= zb[index]) {
          float u = (alpha * u0z0 + beta * u1z1 + gamma * u2z2) / zRec;
          float v = (alpha * v0z0 + beta * v1z1 + gamma * v2z2) / zRec;
          float intensity = alpha * t->in[0] + beta * t->in[1] + gamma * t->in[2];
          uint8_t c[4];
          if (texture) {
            orc_texture_sample(texture, u, v, c);
          } else if (t->has_col) {
            /* extension: base colour = 255 * interpolated RGB, alpha 255 */
            for (int k = 0; k < 3; k++) {
              float ck = alpha * t->col[0][k] + beta * t->col[1][k] + gamma * t->col[2][k];
              float base = ck * 255.0f;
              c[k] = orc_go_uint8(base * intensity);
            }
            c[3] = 255;
            zb[index] = zRec;
            memcpy(rgba + 4 * index, c, 4);
            if (ids) ids[index] = t->face;
            goto next;
          } else {
            memcpy(c, kFaceColor, 4);
          }
          zb[index] = zRec;
          if (ids) ids[index] = t->face;
          /* colorIntensity (rasterizer.go:81-88) */
          rgba[4 * index + 0] = orc_go_uint8((float)c[0] * intensity);
          rgba[4 * index + 1] = orc_go_uint8((float)c[1] * intensity);
          rgba[4 * index + 2] = orc_go_uint8((float)c[2] * intensity);
          rgba[4 * index + 3] = c[3];
        }
      }
    next:
      fx01 = wadd(fx01, f01dx);
      fx12 = wadd(fx12, f12dx);
      fx20 = wadd(fx20, f20dx);
    }
    f01 = wadd(f01, f01dy);
    f12 = wadd(f12, f12dy);
    f20 = wadd(f20, f20dy);
  }
}

void orc_fb_triangle(uint8_t* rgba, float* z, int32_t width, int32_t height,
                     int64_t x0, int64_t y0, float z0, float u0, float v0,
                     int64_t x1, int64_t y1, float z1, float u1, float v1,
                     int64_t x2, int64_t y2, float z2, float u2, float v2,
                     int64_t tsx, int64_t tsy, int64_t tex_, int64_t tey,
                     float ia, float ib, float ic, const orc_texture* texture) {
  RTri t;
  memset(&t, 0, sizeof(t));
  t.x[0] = x0; t.y[0] = y0; t.w[0] = z0; t.u[0] = u0; t.v[0] = v0;
  t.x[1] = x1; t.y[1] = y1; t.w[1] = z1; t.u[1] = u1; t.v[1] = v1;
  t.x[2] = x2; t.y[2] = y2; t.w[2] = z2; t.u[2] = u2; t.v[2] = v2;
  t.in[0] = ia; t.in[1] = ib; t.in[2] = ic;
  t.tex = -1;
  raster_tri(rgba, z, NULL, width, height, &t, tsx, tsy, tex_, tey, texture, INT64_MIN, INT64_MAX);
}

/* ------------------------------------------------------------------ */
/* renderer.go: projection                                             */
/* ------------------------------------------------------------------ */

static int facing(V4 a, V4 b, V4 c) {         /* renderer.go:246-250 */
  V3 v0 = v4to3(a), v1 = v4to3(b), v2 = v4to3(c);
  V3 n = v3cross(v3sub(v1, v0), v3sub(v2, v0));
  V3 zero = {0, 0, 0};
  return v3dot(n, v3sub(zero, v0)) > 0;
}

int orc_facing_camera(const float* a, const float* b, const float* c) {
  V4 va = {a[0], a[1], a[2], a[3]}, vb = {b[0], b[1], b[2], b[3]}, vc = {c[0], c[1], c[2], c[3]};
  return facing(va, vb, vc);
}

typedef struct {
  RTri* v;
  int64_t n, cap;
} TriList;

static int tl_push(TriList* l, const RTri* t) {
  if (l->n == l->cap) {
    int64_t nc = l->cap ? l->cap * 2 : 1024;
    RTri* nv = (RTri*)realloc(l->v, (size_t)nc * sizeof(RTri));
    if (!nv) return -4;
    l->v = nv;
    l->cap = nc;
  }
  l->v[l->n++] = *t;
  return 0;
}

static inline V4 ld4(const float* p) { V4 v = {p[0], p[1], p[2], p[3]}; return v; }

/* projectObject (renderer.go:254-407) for one item, appending binned
 * triangles in face order.  Sequential mode: one tile spanning the screen. */
static int project_object(const orc_item* it, const orc_frame* fr, uint32_t face_base, TriList* out) {
  const orc_mesh* m = it->mesh;
  const uint32_t fl = fr->flags;
  const float znear = 0.0f, zfar = 50.0f;   /* renderer.go:121 */
  Plane pl[6];
  frustum_planes(znear, zfar, pl);
  V3 light = {fr->light[0], fr->light[1], fr->light[2]};

  float corners[32];
  memcpy(corners, m->bbox, sizeof(corners));
  orc_transform_batch(it->mvp, corners, 8);            /* renderer.go:268-269 */
  int vis = orc_box_visibility(corners, znear, zfar);  /* renderer.go:272 */
  if (vis == 0) return 0;

  int has_vn = m->nn != 0;                             /* renderer.go:313 */
  float wf = (float)fr->width, hf = (float)fr->height; /* tile bounds, one tile */

  for (int32_t fi = 0; fi < m->nf; fi++) {
    int32_t i0 = m->vidx[3 * fi], i1 = m->vidx[3 * fi + 1], i2 = m->vidx[3 * fi + 2];
    if (i0 < 0 || i0 >= m->nv || i1 < 0 || i1 >= m->nv || i2 < 0 || i2 >= m->nv) return -1;
    V4 vert[3];
    vert[0] = mat_vec(it->mvp, ld4(m->pos + 4 * (int64_t)i0));   /* renderer.go:303-304, 318-320 */
    vert[1] = mat_vec(it->mvp, ld4(m->pos + 4 * (int64_t)i1));
    vert[2] = mat_vec(it->mvp, ld4(m->pos + 4 * (int64_t)i2));

    if ((fl & ORC_BACKFACE_CULLING) && !facing(vert[0], vert[1], vert[2])) continue;

    float vin[3];
    if (fl & ORC_LIGHTING) {                            /* renderer.go:326-346 */
      if (has_vn && !(fl & ORC_FLAT_SHADING)) {
        for (int k = 0; k < 3; k++) {
          int32_t ni = m->nidx ? m->nidx[3 * fi + k] : -1;
          if (ni < 0 || ni >= m->nn) return -2;
          V3 vn = v4to3(v4normalize(mat_vec(it->world, ld4(m->vnrm + 4 * (int64_t)ni))));
          vin[k] = 0.5f + v3dot(vn, light) * 0.5f;
        }
      } else {
        V3 fn = v4to3(v4normalize(mat_vec(it->world, ld4(m->fnrm + 4 * (int64_t)fi))));
        float diffuse = v3dot(fn, light) * 0.5f;
        float in = 0.5f + diffuse;
        vin[0] = vin[1] = vin[2] = in;
      }
    } else {
      vin[0] = vin[1] = vin[2] = 0.5f;
    }

    UV fuv[3] = {{0, 0}, {0, 0}, {0, 0}};
    if (m->uv)
      for (int k = 0; k < 3; k++) { fuv[k].u = m->uv[6 * fi + 2 * k]; fuv[k].v = m->uv[6 * fi + 2 * k + 1]; }
    V3 fcol[3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    int32_t vi[3] = {i0, i1, i2};
    if (m->vcolor)
      for (int k = 0; k < 3; k++) {
        const float* cp = m->vcolor + 3 * (int64_t)vi[k];
        fcol[k].x = cp[0]; fcol[k].y = cp[1]; fcol[k].z = cp[2];
      }
    int32_t tex = m->tex ? m->tex[fi] : -1;
    if (tex >= fr->ntextures) return -5;

    ClipTri ct[MAX_CLIP];
    int cnt;
    if ((fl & ORC_FRUSTUM_CLIPPING) && vis != 2) {      /* renderer.go:349-359 */
      cnt = clip_triangle(pl, vert, fuv, vin, fcol, ct);
      if (cnt < 0) return cnt;
    } else {
      for (int k = 0; k < 3; k++) {
        ct[0].p[k] = vert[k]; ct[0].uv[k] = fuv[k]; ct[0].in[k] = vin[k]; ct[0].col[k] = fcol[k];
      }
      cnt = 1;
    }

    for (int i = 0; i < cnt; i++) {                     /* renderer.go:361-395 */
      V4 sp[3];
      for (int j = 0; j < 3; j++) {
        float origW = ct[i].p[j].w;
        sp[j] = mat_vec(fr->screen, v4div(ct[i].p[j], ct[i].p[j].w));
        sp[j].w = origW;
      }
      /* identifyTriangleTiles (renderer.go:226-244) with one tile */
      float minX = gomin(gomin(sp[0].x, sp[1].x), sp[2].x);
      float maxX = gomax(gomax(sp[0].x, sp[1].x), sp[2].x);
      float minY = gomin(gomin(sp[0].y, sp[1].y), sp[2].y);
      float maxY = gomax(gomax(sp[0].y, sp[1].y), sp[2].y);
      if (!(maxX >= 0.0f && minX <= wf && maxY >= 0.0f && minY <= hf)) continue;
      RTri t;
      for (int j = 0; j < 3; j++) {                     /* drawProjection, renderer.go:181-184 */
        t.x[j] = orc_go_int(sp[j].x);
        t.y[j] = orc_go_int(sp[j].y);
        t.w[j] = sp[j].w;
        t.u[j] = ct[i].uv[j].u;
        t.v[j] = ct[i].uv[j].v;
        t.in[j] = ct[i].in[j];
        t.col[j][0] = ct[i].col[j].x; t.col[j][1] = ct[i].col[j].y; t.col[j][2] = ct[i].col[j].z;
      }
      t.tex = tex;
      t.has_col = m->vcolor != NULL;
      t.face = face_base + (uint32_t)fi;
      for (int j = 0; j < 3; j++) { t.sx[j] = sp[j].x; t.sy[j] = sp[j].y; }
      int e = tl_push(out, &t);
      if (e) return e;
    }
  }
  return 0;
}

/* ------------------------------------------------------------------ */
/* renderer.go: Draw                                                   */
/* ------------------------------------------------------------------ */

typedef struct {
  const orc_item* items;
  int32_t nitems;
  const orc_frame* fr;
  TriList* lists;
  int* errs;
  int32_t next;           /* next item to project (claimed under lock) */
  pthread_mutex_t mu;
  uint8_t* rgba;
  float* z;
  uint32_t* ids;          /* optional: face that wrote each pixel */
  uint32_t* face_base;    /* per item */
  int band_err;           /* overlay error seen by a raster band */
  int32_t nthreads;
  int32_t band;           /* band index for the raster phase */
} DrawCtx;

/* ---- overlays: ShowEdges / ShowVertices (renderer.go:191-216) ---- */

static const uint8_t kEdgeColor[4] = {0, 0, 0, 255};        /* renderer.go:19 */
static const uint8_t kVertexColor[4] = {255, 161, 0, 255};  /* renderer.go:18 */
static const uint8_t kWhite[4] = {255, 255, 255, 255};      /* renderer.go:195 */

typedef struct {
  uint8_t* rgba;
  int64_t width, npx;
  int64_t y0, y1;          /* band: rows of the linear index that this pass owns */
  int err;
} Plot;

/* FrameBuffer.Pixel (rasterizer.go:25-30): the linear index decides, so an
 * x outside [0, width) wraps into a neighbouring row, and index 0 is never
 * written. */
static void plot(Plot* p, int64_t x, int64_t y, const uint8_t* c) {
  const int64_t idx = wadd(wmul(y, p->width), x);
  if (!(idx > 0 && idx < p->npx)) return;
  const int64_t row = idx / p->width;
  if (row < p->y0 || row >= p->y1) return;
  memcpy(p->rgba + 4 * idx, c, 4);
}

/* utils.go abs: MinInt maps to MaxInt */
static int64_t go_abs(int64_t v) {
  if (v < 0) v = (int64_t)(0 - (uint64_t)v);
  if (v < 0) v = (int64_t)((uint64_t)v - 1);
  return v;
}

/* FrameBuffer.Line (rasterizer.go:65-79): DDA with float32 steps accumulated
 * one add at a time.  Lines of more than ORC_MAX_LINE_STEPS steps are refused
 * (error -6): the reference would plot them for a very long time. */
#define ORC_MAX_LINE_STEPS (1ll << 22)
static void draw_line(Plot* p, int64_t x0, int64_t y0, int64_t x1, int64_t y1, const uint8_t* c) {
  const int64_t dx = wsub(x1, x0), dy = wsub(y1, y0);
  const int64_t ax = go_abs(dx), ay = go_abs(dy);
  const int64_t side = ax > ay ? ax : ay;
  if (side > ORC_MAX_LINE_STEPS) { p->err = -6; return; }
  const float xs = (float)dx / (float)side, ys = (float)dy / (float)side;
  float cx = (float)x0, cy = (float)y0;
  for (int64_t i = 0; i <= side; i++) {
    plot(p, orc_go_int(cx), orc_go_int(cy), c);
    cx += xs;
    cy += ys;
  }
}

/* FrameBuffer.Rect (rasterizer.go:54-63) */
static void draw_rect(Plot* p, int64_t x, int64_t y, int64_t w, int64_t h, const uint8_t* c) {
  if (x >= p->width || y >= p->npx / p->width) return;
  for (int64_t py = y; py < wadd(y, h); py++)
    for (int64_t px = x; px < wadd(x, w); px++) plot(p, px, py, c);
}

/* FrameBuffer.Fog (rasterizer.go:193-207) with blendRGBA (185-191):
 * uint8(float32(a)*(1-f) + float32(b)*f) per channel, alpha included. */
void orc_fog(uint8_t* rgba, const float* z, int32_t width, int32_t height, float fog_start, float fog_end,
             const uint8_t* color) {
  const int64_t n = (int64_t)width * height;
  for (int64_t i = 0; i < n; i++) {
    const float depth = z[i];
    if (depth >= fog_start) continue;
    if (depth <= fog_end) {
      memcpy(rgba + 4 * i, color, 4);
      continue;
    }
    const float f = 1 - ((fog_end - depth) / (fog_end - fog_start));
    for (int k = 0; k < 4; k++) rgba[4 * i + k] = orc_go_uint8((float)rgba[4 * i + k] * (1 - f) + (float)color[k] * f);
  }
}

int orc_fb_line(uint8_t* rgba, int32_t width, int32_t height, int64_t x0, int64_t y0, int64_t x1, int64_t y1,
                const uint8_t* color) {
  Plot p = {rgba, width, (int64_t)width * height, 0, height, 0};
  draw_line(&p, x0, y0, x1, y1, color);
  return p.err;
}

void orc_fb_rect(uint8_t* rgba, int32_t width, int32_t height, int64_t x, int64_t y, int64_t w, int64_t h,
                 const uint8_t* color) {
  Plot p = {rgba, width, (int64_t)width * height, 0, height, 0};
  draw_rect(&p, x, y, w, h, color);
}

static void overlays(Plot* p, const RTri* t, uint32_t fl) {
  if (fl & ORC_SHOW_EDGES) {
    const uint8_t* col = (fl & ORC_SHOW_FACES) ? kEdgeColor : kWhite;
    draw_line(p, t->x[0], t->y[0], t->x[1], t->y[1], col);
    draw_line(p, t->x[1], t->y[1], t->x[2], t->y[2], col);
    draw_line(p, t->x[2], t->y[2], t->x[0], t->y[0], col);
    if (fl & ORC_SHOW_FACES) {
      const float cx = (t->sx[0] + t->sx[1] + t->sx[2]) / 3;
      const float cy = (t->sy[0] + t->sy[1] + t->sy[2]) / 3;
      draw_rect(p, wsub(orc_go_int(cx), 1), wsub(orc_go_int(cy), 1), 3, 3, col);
    }
  }
  if (fl & ORC_SHOW_VERTICES)
    for (int j = 0; j < 3; j++) draw_rect(p, wsub(t->x[j], 1), wsub(t->y[j], 1), 3, 3, kVertexColor);
}

static void raster_band(DrawCtx* c, int64_t y0, int64_t y1) {
  const orc_frame* fr = c->fr;
  const uint32_t fl = fr->flags;
  Plot pl = {c->rgba, fr->width, (int64_t)fr->width * fr->height, y0, y1, 0};
  for (int32_t i = 0; i < c->nitems; i++) {
    const TriList* l = &c->lists[i];
    for (int64_t k = 0; k < l->n; k++) {
      const RTri* t = &l->v[k];
      if (fl & ORC_SHOW_FACES) {
        const orc_texture* tx = NULL;
        if ((fl & ORC_SHOW_TEXTURES) && t->tex >= 0) tx = &fr->textures[t->tex];  /* renderer.go:176-178 */
        raster_tri(c->rgba, c->z, c->ids, fr->width, fr->height, t, 0, 0, fr->width, fr->height, tx, y0, y1);
      }
      if (fl & (ORC_SHOW_EDGES | ORC_SHOW_VERTICES)) overlays(&pl, t, fl);
    }
  }
  if (pl.err) __atomic_store_n(&c->band_err, pl.err, __ATOMIC_RELAXED);
}

static void* project_worker(void* arg) {
  DrawCtx* c = (DrawCtx*)arg;
  for (;;) {
    pthread_mutex_lock(&c->mu);
    int32_t i = c->next++;
    pthread_mutex_unlock(&c->mu);
    if (i >= c->nitems) break;
    c->errs[i] = project_object(&c->items[i], c->fr, c->face_base[i], &c->lists[i]);
  }
  return NULL;
}

typedef struct { DrawCtx* c; int64_t y0, y1; } BandArg;

static void* raster_worker(void* arg) {
  BandArg* b = (BandArg*)arg;
  raster_band(b->c, b->y0, b->y1);
  return NULL;
}

int64_t orc_project(const orc_item* items, int32_t nitems, const orc_frame* fr, int64_t* xy_out,
                    float* w_out, int64_t cap) {
  int64_t n = 0;
  for (int32_t i = 0; i < nitems; i++) {
    TriList l = {0, 0, 0};
    int e = project_object(&items[i], fr, 0u, &l);
    if (e) { free(l.v); return e; }
    for (int64_t k = 0; k < l.n; k++, n++) {
      if (n >= cap) continue;
      for (int j = 0; j < 3; j++) {
        xy_out[6 * n + 2 * j] = l.v[k].x[j];
        xy_out[6 * n + 2 * j + 1] = l.v[k].y[j];
        w_out[3 * n + j] = l.v[k].w[j];
      }
    }
    free(l.v);
  }
  return n;
}

int orc_draw(const orc_item* items, int32_t nitems, const orc_frame* fr, uint8_t* rgba, float* z,
             int64_t* tpf, int32_t nthreads) {
  return orc_draw_ids(items, nitems, fr, rgba, z, NULL, tpf, nthreads);
}

int orc_draw_ids(const orc_item* items, int32_t nitems, const orc_frame* fr, uint8_t* rgba, float* z,
                 uint32_t* ids, int64_t* tpf, int32_t nthreads) {
  const int64_t npx = (int64_t)fr->width * fr->height;
  if (ids)
    for (int64_t i = 0; i < npx; i++) ids[i] = 0xFFFFFFFFu;
  /* FrameBuffer.Clear (rasterizer.go:36-44) and DotGrid (rasterizer.go:46-52) */
  for (int64_t i = 0; i < npx; i++) {
    rgba[4 * i] = 50; rgba[4 * i + 1] = 50; rgba[4 * i + 2] = 50; rgba[4 * i + 3] = 255;
    z[i] = -1.0f;
  }
  for (int64_t y = 10; y < fr->height; y += 10)
    for (int64_t x = 10; x < fr->width; x += 10) {
      int64_t idx = y * fr->width + x;
      if (idx > 0 && idx < npx) {                          /* FrameBuffer.Pixel, 25-30 */
        rgba[4 * idx] = 100; rgba[4 * idx + 1] = 100; rgba[4 * idx + 2] = 100; rgba[4 * idx + 3] = 255;
      }
    }

  const uint32_t fl_all = fr->flags;
  DrawCtx c;
  memset(&c, 0, sizeof(c));
  c.items = items; c.nitems = nitems; c.fr = fr; c.rgba = rgba; c.z = z; c.ids = ids;
  c.lists = (TriList*)calloc((size_t)(nitems > 0 ? nitems : 1), sizeof(TriList));
  c.errs = (int*)calloc((size_t)(nitems > 0 ? nitems : 1), sizeof(int));
  c.face_base = (uint32_t*)calloc((size_t)(nitems > 0 ? nitems : 1), sizeof(uint32_t));
  if (!c.lists || !c.errs || !c.face_base) { free(c.lists); free(c.errs); free(c.face_base); return -4; }
  for (int32_t i = 1; i < nitems; i++) c.face_base[i] = c.face_base[i - 1] + (uint32_t)items[i - 1].mesh->nf;
  pthread_mutex_init(&c.mu, NULL);
  if (nthreads < 1) nthreads = 1;

  /* Phase 1: projection, one task per object (renderer.go:451-459). */
  if (nthreads == 1 || nitems <= 1) {
    for (int32_t i = 0; i < nitems; i++) c.errs[i] = project_object(&items[i], fr, c.face_base[i], &c.lists[i]);
  } else {
    int nt = nthreads < nitems ? nthreads : nitems;
    pthread_t th[256];
    if (nt > 256) nt = 256;
    for (int k = 0; k < nt; k++) pthread_create(&th[k], NULL, project_worker, &c);
    for (int k = 0; k < nt; k++) pthread_join(th[k], NULL);
  }
  int err = 0;
  int64_t n = 0;
  for (int32_t i = 0; i < nitems; i++) {
    if (c.errs[i] && !err) err = c.errs[i];
    n += c.lists[i].n;
  }
  if (tpf) *tpf = n;

  /* Phase 2: raster (renderer.go:461-473), order-preserving in each band. */
  if (!err) {
    if (nthreads == 1) {
      raster_band(&c, 0, fr->height);
    } else {
      int nt = nthreads > 256 ? 256 : nthreads;
      pthread_t th[256];
      BandArg ba[256];
      int64_t h = fr->height;
      for (int k = 0; k < nt; k++) {
        ba[k].c = &c;
        ba[k].y0 = h * k / nt;
        ba[k].y1 = h * (k + 1) / nt;
        pthread_create(&th[k], NULL, raster_worker, &ba[k]);
      }
      for (int k = 0; k < nt; k++) pthread_join(th[k], NULL);
    }
    if (c.band_err) err = c.band_err;
    if (!err && (fl_all & ORC_CROSSHAIR)) {
      /* FrameBuffer.CrossHair (rasterizer.go:209-217), drawn after the scene
       * when the reference's demoMode is off (renderer.go:476-478) */
      static const uint8_t kYellow[4] = {255, 255, 0, 255};
      Plot pl = {rgba, fr->width, npx, 0, fr->height, 0};
      const int64_t x = fr->width / 2, y = fr->height / 2;
      draw_line(&pl, x - 5, y, x - 3, y, kYellow);
      draw_line(&pl, x + 3, y, x + 5, y, kYellow);
      draw_line(&pl, x, y - 5, x, y - 3, kYellow);
      draw_line(&pl, x, y + 3, x, y + 5, kYellow);
    }
  }
  for (int32_t i = 0; i < nitems; i++) free(c.lists[i].v);
  free(c.lists);
  free(c.errs);
  free(c.face_base);
  pthread_mutex_destroy(&c.mu);
  return err;
}
