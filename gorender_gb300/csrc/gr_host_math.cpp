// gr_host_math.cpp -- host-side matrix and mesh math (stays on the host).
//
// C++ restatement of matrix.go / vector.go / mesh.go in float32 with the
// reference's operation order.  Built with -ffp-contract=off so no a*b+c is
// fused (Go on amd64 never fuses; on arm64 Go would, which is why the
// reference's arm64 build is a timing baseline, not the parity contract).
#include <cmath>
#include <cstdint>
#include <cstring>

#include "gr_host_math.h"

namespace gr {

static inline float sqrt32(float x) { return (float)std::sqrt((double)x); }  // math32.go:11-13

// Go's math.Sin / math.Cos / math.Tan, which math32.go:15-25 call on
// float64(x).  On amd64 they are pure Go compiled without FMA: the Cephes
// sin.c / tan.c algorithm (S. L. Moshier) as Go's math package states it.
// Reduction by pi/4 uses the Cody-Waite three-part split below 2^29 and the
// Payne-Hanek method (K. C. Ng, "Argument reduction for huge arguments: good
// to the last bit", 1992) above it, then the Cephes minimax polynomials on
// [-pi/4, pi/4].  The C library's sin/cos/tan are other algorithms whose
// doubles differ from Go's in the last bit for about a quarter of arguments.
namespace gotrig {

constexpr double kPi4A = 7.85398125648498535156e-1;  // pi/4 = A + B + C
constexpr double kPi4B = 3.77489470793079817668e-8;
constexpr double kPi4C = 2.69515142907905952645e-15;
constexpr double k4OverPi = 0x1.45f306dc9c883p+0;    // 4/pi, correctly rounded
constexpr double kPi4 = 0x1.921fb54442d18p-1;        // pi/4, correctly rounded
constexpr double kReduceThreshold = 536870912.0;     // 2^29
constexpr double kSin[6] = {1.58962301576546568060e-10, -2.50507477628578072866e-8, 2.75573136213857245213e-6,
                            -1.98412698295895385996e-4, 8.33333333332211858878e-3,  -1.66666666666666307295e-1};
constexpr double kCos[6] = {-1.13585365213876817300e-11, 2.08757008419747316778e-9, -2.75573141792967388112e-7,
                            2.48015872888517045348e-5,   -1.38888888888730564116e-3, 4.16666666666665929218e-2};
constexpr double kTanP[3] = {-1.30936939181383777646e4, 1.15351664838587416140e6, -1.79565251976484877988e7};
constexpr double kTanQ[5] = {1.0, 1.36812963470692954678e4, -1.32089234440210967447e6, 2.50083801823357915839e7,
                             -5.38695755929454629881e7};
// Binary digits of 4/pi, 64 to a word (4/pi = sum W[i] 2^(-64 i)); eight words
// cover every double converted from a float32.
constexpr uint64_t k4PiBits[8] = {0x0000000000000001ull, 0x45f306dc9c882a53ull, 0xf84eafa3ea69bb81ull,
                                  0xb6c52b3278872083ull, 0xfca2c757bd778ac3ull, 0x6e48dc74849ba5c0ull,
                                  0x0c925dd413a32439ull, 0xfc3bd63962534e7dull};

inline uint64_t shl(uint64_t v, unsigned n) { return n >= 64 ? 0 : v << n; }
inline uint64_t shr(uint64_t v, unsigned n) { return n >= 64 ? 0 : v >> n; }

// Payne-Hanek for x >= pi/4 (used from 2^29): octant j (0..7, odd octants
// mapped to the next zero) and the reduced argument.
void payne_hanek(double x, uint64_t& j_out, double& z_out) {
  if (x < kPi4) { j_out = 0; z_out = x; return; }
  uint64_t ix;
  std::memcpy(&ix, &x, 8);
  const int exp = (int)((ix >> 52) & 0x7FF) - 1023 - 52;
  ix = (ix & ~(0x7FFull << 52)) | (1ull << 52);
  const unsigned digit = (unsigned)(exp + 61) / 64, sh = (unsigned)(exp + 61) % 64;
  auto word = [&](unsigned k) { return shl(k4PiBits[k], sh) | shr(k4PiBits[k + 1], 64 - sh); };
  const uint64_t z0 = word(digit), z1 = word(digit + 1), z2 = word(digit + 2);
  const unsigned __int128 p2 = (unsigned __int128)z2 * ix, p1 = (unsigned __int128)z1 * ix;
  const uint64_t lo = (uint64_t)p1 + (uint64_t)(p2 >> 64);
  uint64_t hi = z0 * ix + (uint64_t)(p1 >> 64) + (lo < (uint64_t)p1 ? 1u : 0u);
  uint64_t j = hi >> 61;
  hi = hi << 3 | lo >> 61;
  const unsigned lz = hi ? (unsigned)__builtin_clzll(hi) : 64;
  hi = (shl(hi, lz + 1) | shr(lo, 64 - (lz + 1))) >> 12;
  hi |= (uint64_t)(1023 - (lz + 1)) << 52;
  double z;
  std::memcpy(&z, &hi, 8);
  if (j & 1) { j = (j + 1) & 7; z = z - 1.0; }
  j_out = j;
  z_out = z * kPi4;
}

void reduce(double x, uint64_t& j_out, double& z_out) {
  if (x >= kReduceThreshold) { payne_hanek(x, j_out, z_out); return; }
  uint64_t j = (uint64_t)(x * k4OverPi);
  double y = (double)j;
  if (j & 1) { j++; y++; }
  j_out = j;
  z_out = ((x - y * kPi4A) - y * kPi4B) - y * kPi4C;
}

inline double sin_poly(double z, double zz) {
  return z + z * zz * ((((((kSin[0] * zz) + kSin[1]) * zz + kSin[2]) * zz + kSin[3]) * zz + kSin[4]) * zz + kSin[5]);
}
inline double cos_poly(double zz) {
  return 1.0 - 0.5 * zz + zz * zz * ((((((kCos[0] * zz) + kCos[1]) * zz + kCos[2]) * zz + kCos[3]) * zz + kCos[4]) * zz + kCos[5]);
}

double sin(double x) {
  if (x == 0 || std::isnan(x)) return x;
  if (std::isinf(x)) return std::nan("");
  bool sign = false;
  if (x < 0) { x = -x; sign = true; }
  uint64_t j;
  double z;
  reduce(x, j, z);
  j &= 7;
  if (j > 3) { sign = !sign; j -= 4; }
  const double zz = z * z;
  const double y = (j == 1 || j == 2) ? cos_poly(zz) : sin_poly(z, zz);
  return sign ? -y : y;
}

double cos(double x) {
  if (std::isnan(x) || std::isinf(x)) return std::nan("");
  bool sign = false;
  x = std::fabs(x);
  uint64_t j;
  double z;
  reduce(x, j, z);
  j &= 7;
  if (j > 3) { j -= 4; sign = !sign; }
  if (j > 1) sign = !sign;
  const double zz = z * z;
  const double y = (j == 1 || j == 2) ? sin_poly(z, zz) : cos_poly(zz);
  return sign ? -y : y;
}

double tan(double x) {
  if (x == 0 || std::isnan(x)) return x;
  if (std::isinf(x)) return std::nan("");
  bool sign = false;
  if (x < 0) { x = -x; sign = true; }
  uint64_t j;
  double z;
  reduce(x, j, z);
  const double zz = z * z;
  double y = z;
  if (zz > 1e-14)
    y = z + z * (zz * (((kTanP[0] * zz) + kTanP[1]) * zz + kTanP[2]) /
                 ((((zz + kTanQ[1]) * zz + kTanQ[2]) * zz + kTanQ[3]) * zz + kTanQ[4]));
  if (j & 2) y = -1 / y;
  return sign ? -y : y;
}

}  // namespace gotrig

static inline float sin32(float x) { return (float)gotrig::sin((double)x); }  // math32.go:15-17
static inline float cos32(float x) { return (float)gotrig::cos((double)x); }  // math32.go:19-21
static inline float tan32(float x) { return (float)gotrig::tan((double)x); }  // math32.go:23-25

struct V3 {
  float x, y, z;
};
static inline V3 cross(V3 a, V3 b) {  // vector.go:55-60
  return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
static inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline V3 normalize(V3 v) {  // vector.go:51-53, 78-80
  float len = sqrt32(v.x * v.x + v.y * v.y + v.z * v.z);
  return V3{v.x / len, v.y / len, v.z / len};
}

void mat_identity(float* m) {
  std::memset(m, 0, 16 * sizeof(float));
  m[0] = m[5] = m[10] = m[15] = 1.0f;
}

// Matrix.Multiply (matrix.go:155-165).
void mat_multiply(const float* a, const float* b, float* out) {
  float r[16];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      float acc = 0.0f;
      for (int k = 0; k < 4; ++k) acc += a[i * 4 + k] * b[k * 4 + j];
      r[i * 4 + j] = acc;
    }
  std::memcpy(out, r, sizeof(r));
}

static void rotation(int axis, float angle, float* m) {  // matrix.go:32-72
  mat_identity(m);
  if (angle == 0) return;
  float s = sin32(angle), c = cos32(angle);
  if (axis == 0) { m[5] = c; m[6] = -s; m[9] = s; m[10] = c; }
  if (axis == 1) { m[0] = c; m[2] = s; m[8] = -s; m[10] = c; }
  if (axis == 2) { m[0] = c; m[1] = -s; m[4] = s; m[5] = c; }
}

// NewWorldMatrix (matrix.go:82-88).
void world_matrix(const float* scale, const float* rot, const float* trans, float* out) {
  float m[16], t[16], r[16], rr[16];
  mat_identity(m);
  mat_identity(t);
  t[0] = scale[0]; t[5] = scale[1]; t[10] = scale[2];
  mat_multiply(t, m, m);
  mat_identity(r);  // NewRotationMatrix (matrix.go:74-80)
  for (int a = 0; a < 3; ++a) {
    rotation(a, rot[a], rr);
    mat_multiply(r, rr, r);
  }
  mat_multiply(r, m, m);
  mat_identity(t);
  t[3] = trans[0]; t[7] = trans[1]; t[11] = trans[2];
  mat_multiply(t, m, out);
}

// NewViewMatrix (matrix.go:133-144).
void view_matrix(const float* eye3, const float* dir3, const float* up3, float* out) {
  V3 eye{eye3[0], eye3[1], eye3[2]}, dir{dir3[0], dir3[1], dir3[2]}, up{up3[0], up3[1], up3[2]};
  V3 z = normalize(dir);
  V3 x = normalize(cross(up, z));
  V3 y = normalize(cross(z, x));
  float m[16] = {x.x, x.y, x.z, -dot(x, eye), y.x, y.y, y.z, -dot(y, eye),
                 z.x, z.y, z.z, -dot(z, eye), 0,   0,   0,   1};
  std::memcpy(out, m, sizeof(m));
}

// NewPerspectiveMatrix (matrix.go:92-106).
void perspective_matrix(float fov, float aspect, float znear, float zfar, float* out) {
  float tan_half = tan32(fov / 2.0f);
  float m00 = 1 / (aspect * tan_half);
  float m11 = 1 / tan_half;
  float m22 = (zfar + znear) / (znear - zfar);
  float m23 = (2 * zfar * znear) / (znear - zfar);
  float m[16] = {m00, 0, 0, 0, 0, m11, 0, 0, 0, 0, -m22, -m23, 0, 0, -1, 0};
  std::memcpy(out, m, sizeof(m));
}

// NewScreenMatrix (matrix.go:108-118).
void screen_matrix(int width, int height, float* out) {
  float hw = (float)width / 2;
  float hh = (float)height / 2;
  float m[16] = {hw, 0, 0, hw, 0, hh, 0, hh, 0, 0, 0.5f, 0.5f, 0, 0, 0, 1};
  std::memcpy(out, m, sizeof(m));
}

// projectObject's matrices (renderer.go:255-262): mvp = I*P*V*W.
void object_matrices(const float* scale, const float* rot, const float* trans, const float* eye,
                     const float* dir, const float* up, int width, int height, float fov_y,
                     float* mvp, float* world) {
  float aspect = (float)width / (float)height;  // NewRenderer (renderer.go:115)
  float v[16], p[16];
  world_matrix(scale, rot, trans, world);
  view_matrix(eye, dir, up, v);
  perspective_matrix(fov_y, aspect, 0.0f, 50.0f, p);  // renderer.go:121
  mat_identity(mvp);
  mat_multiply(mvp, p, mvp);
  mat_multiply(mvp, v, mvp);
  mat_multiply(mvp, world, mvp);
}

void normalize3(const float* v, float* out) {
  V3 r = normalize(V3{v[0], v[1], v[2]});
  out[0] = r.x; out[1] = r.y; out[2] = r.z;
}

// NewMesh face normals (mesh.go:55-60).
void face_normals(const float* pos, const int* vidx, int nf, float* out) {
  for (int i = 0; i < nf; ++i) {
    const float* a = pos + 4 * (long)vidx[3 * i];
    const float* b = pos + 4 * (long)vidx[3 * i + 1];
    const float* c = pos + 4 * (long)vidx[3 * i + 2];
    V3 v0{a[0], a[1], a[2]}, v1{b[0], b[1], b[2]}, v2{c[0], c[1], c[2]};
    V3 e1{v1.x - v0.x, v1.y - v0.y, v1.z - v0.z};
    V3 e2{v2.x - v0.x, v2.y - v0.y, v2.z - v0.z};
    V3 n = normalize(cross(e1, e2));
    out[4 * i] = n.x; out[4 * i + 1] = n.y; out[4 * i + 2] = n.z; out[4 * i + 3] = 1.0f;
  }
}

// boundingBox (mesh.go:28-51).  Go's min/max return NaN if either operand is NaN.
static inline float gomin(float a, float b) {
  if (a != a || b != b) return NAN;
  if (a < b) return a;
  if (b < a) return b;
  return std::signbit(a) ? a : b;
}
static inline float gomax(float a, float b) {
  if (a != a || b != b) return NAN;
  if (a > b) return a;
  if (b > a) return b;
  return std::signbit(a) ? b : a;
}
void bounding_box(const float* pos, int nv, float* out) {
  float mnx = pos[0], mny = pos[1], mnz = pos[2], mxx = mnx, mxy = mny, mxz = mnz;
  for (int i = 0; i < nv; ++i) {
    const float* v = pos + 4 * (long)i;
    mnx = gomin(mnx, v[0]); mny = gomin(mny, v[1]); mnz = gomin(mnz, v[2]);
    mxx = gomax(mxx, v[0]); mxy = gomax(mxy, v[1]); mxz = gomax(mxz, v[2]);
  }
  float b[32] = {mnx, mny, mnz, 1, mnx, mny, mxz, 1, mnx, mxy, mnz, 1, mnx, mxy, mxz, 1,
                 mxx, mny, mnz, 1, mxx, mny, mxz, 1, mxx, mxy, mnz, 1, mxx, mxy, mxz, 1};
  std::memcpy(out, b, sizeof(b));
}

}  // namespace gr
