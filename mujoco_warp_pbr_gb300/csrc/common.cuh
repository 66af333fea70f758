// Device math shared by the render kernels of libmjpbr.
//
// Arithmetic rules (the library is compiled with -fmad=false):
//  * Geometry (camera rays, intersections, hit points, shadow and mirror ray set-up) uses plain
//    IEEE float operations only (no fused multiply-add, correctly rounded division and sqrt), so
//    every geometric decision is reproducible bit for bit by a scalar C implementation that
//    evaluates the same expressions in the same order.
//  * Shading arithmetic may use explicit fmaf (fdot, fmadd) and the fast intrinsics: it only feeds
//    colours, which are compared within 1/255.
#pragma once

#include <cstdint>
#include <cuda_fp16.h>

#include "mjpbr.h"

#define MJ_DEV __device__ __forceinline__
#define MJ_HD __host__ __device__ __forceinline__

namespace mjpbr {

// MuJoCo's mjMINVAL / mjMAXVAL.
constexpr float kMinVal = 1.0e-15f;
constexpr float kMaxVal = 1.0e10f;
// Relative and absolute hit-distance tolerance of the closest-hit tie-break (higher geom id wins
// within kRayTolRel * max(dist, 1)); the traversal cut-off widens by the same amounts.
constexpr float kRayTolRel = 1.0e-5f;
constexpr float kRayTolAbs = 1.0e-7f;
// Origin offset of secondary rays along the normal; shadow rays stop this short of a light;
// length of shadow rays towards directional lights and the environment.
constexpr float kRayOffset = 1.0e-4f;
constexpr float kShadowGap = 1.0e-3f;
constexpr float kUnboundedShadow = 1.0e8f;
constexpr float kPi = 3.14159265358979323846f;
// Error bits OR-ed into MjpbrScene.error_word.
constexpr int32_t kErrStackOverflow = 1;
constexpr int32_t kErrWorkQueue = 2;
constexpr int32_t kErrWaitTimeout = 4;
constexpr int32_t kErrPoseIndex = 8;  // a pose input named a body or shape out of range (skipped)
constexpr int32_t kErrBvhInput = 16;  // a BVH build face named a vertex outside its mesh (clamped)
// Most worlds of one scene (grids of more than kMaxGridWorlds worlds are split into launches).
constexpr int32_t kMaxWorlds = 1 << 24;
// Most worlds one launch puts in grid y (CUDA's limit on gridDim.y); more worlds take more launches.
constexpr int32_t kMaxGridWorlds = 65535;
// Most traversal stack entries per ray (settings.stack_depth sizes a launch's stacks, at most this).
constexpr int32_t kStackDepth = 32;

struct V3 {
  float x, y, z;
};

MJ_HD V3 v3(float x, float y, float z) { return V3{x, y, z}; }
MJ_HD V3 v3(float s) { return V3{s, s, s}; }
MJ_HD V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
MJ_HD V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
MJ_HD V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
MJ_HD V3 operator*(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
MJ_HD V3 operator*(float s, V3 a) { return V3{a.x * s, a.y * s, a.z * s}; }
MJ_HD V3 operator/(V3 a, float s) { return V3{a.x / s, a.y / s, a.z / s}; }
MJ_HD V3 cmul(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
MJ_HD V3& operator+=(V3& a, V3 b) {
  a = a + b;
  return a;
}
// Plain-arithmetic dot product: ((x + y) + z), the order the C restatement uses.
MJ_HD float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
MJ_HD V3 cross(V3 a, V3 b) { return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
MJ_HD float length_sq(V3 a) { return dot(a, a); }
MJ_HD float length(V3 a) { return sqrtf(dot(a, a)); }
MJ_HD V3 normalize(V3 a) {
  float l = sqrtf(dot(a, a));
  return l > 0.0f ? a / l : a;
}
MJ_HD V3 vmax(V3 a, V3 b) { return V3{fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)}; }
MJ_HD V3 vmin(V3 a, V3 b) { return V3{fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)}; }
MJ_HD float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
MJ_HD float vmax3(V3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }

// Shading-only fused helpers.
MJ_DEV float fdot(V3 a, V3 b) { return __fmaf_rn(a.x, b.x, __fmaf_rn(a.y, b.y, a.z * b.z)); }
MJ_DEV V3 fmadd(V3 a, float s, V3 c) {
  return V3{__fmaf_rn(a.x, s, c.x), __fmaf_rn(a.y, s, c.y), __fmaf_rn(a.z, s, c.z)};
}
MJ_DEV V3 fnormalize(V3 a) {
  float l2 = fdot(a, a);
  return l2 > 0.0f ? a * rsqrtf(l2) : a;
}

// Compact shading-only math (colours tolerate ~1e-6 relative error): atan on [-1, 1] as x P(x^2)
// with a degree-7 polynomial fitted by least squares on Chebyshev nodes (max error 1.7e-7 rad),
// extended to atan2 by octant symmetry; acos(x) = atan2(sqrt((1 - x)(1 + x)), x); powers and
// logarithms through the special-function unit.
MJ_DEV float atan_unit(float x) {
  float t = x * x;
  float p = -0.004831168334931135f;
  p = __fmaf_rn(p, t, 0.02475677989423275f);
  p = __fmaf_rn(p, t, -0.06021912768483162f);
  p = __fmaf_rn(p, t, 0.09967923909425735f);
  p = __fmaf_rn(p, t, -0.14040139317512512f);
  p = __fmaf_rn(p, t, 0.1997368186712265f);
  p = __fmaf_rn(p, t, -0.33332303166389465f);
  p = __fmaf_rn(p, t, 0.9999999403953552f);
  return x * p;
}
MJ_DEV float fast_atan2(float y, float x) {
  float ax = fabsf(x), ay = fabsf(y);
  float mx = fmaxf(ax, ay), mn = fminf(ax, ay);
  float r = mx > 0.0f ? atan_unit(__fdividef(mn, mx)) : 0.0f;
  if (ay > ax) r = 1.57079632679489662f - r;
  if (x < 0.0f) r = 3.14159265358979324f - r;
  return y < 0.0f ? -r : r;
}
MJ_DEV float fast_acos(float x) { return fast_atan2(sqrtf(fmaxf((1.0f - x) * (1.0f + x), 0.0f)), x); }
MJ_DEV float fast_pow(float x, float y) { return x > 0.0f ? exp2f(y * __log2f(x)) : 0.0f; }

// Row-major 3x3 matrix (MuJoCo xmat).
struct M3 {
  float m[9];
};
// R v: ((m0 v0 + m1 v1) + m2 v2) per row.
MJ_HD V3 mul(const M3& r, V3 v) {
  return V3{r.m[0] * v.x + r.m[1] * v.y + r.m[2] * v.z, r.m[3] * v.x + r.m[4] * v.y + r.m[5] * v.z,
            r.m[6] * v.x + r.m[7] * v.y + r.m[8] * v.z};
}
// R^T v.
MJ_HD V3 mul_t(const M3& r, V3 v) {
  return V3{r.m[0] * v.x + r.m[3] * v.y + r.m[6] * v.z, r.m[1] * v.x + r.m[4] * v.y + r.m[7] * v.z,
            r.m[2] * v.x + r.m[5] * v.y + r.m[8] * v.z};
}

MJ_HD float as_float(int32_t i) {
#ifdef __CUDA_ARCH__
  return __int_as_float(i);
#else
  float f;
  memcpy(&f, &i, 4);
  return f;
#endif
}
MJ_HD int32_t as_int(float f) {
#ifdef __CUDA_ARCH__
  return __float_as_int(f);
#else
  int32_t i;
  memcpy(&i, &f, 4);
  return i;
#endif
}

// sin and cos of 2*pi*t for a turn fraction t, from plain float operations only, so the value is
// identical wherever it is evaluated: quadrant reduction t = q/4 + r with |r| <= 1/8 turn, then
// Taylor polynomials of sin and cos on |theta| <= pi/4 (degree 11 and 12: truncation error below
// 1e-11, far under float rounding). Used where an angle decides geometry (soft-shadow disc
// samples, camera field of view).
MJ_HD void sincos_turns(float t, float* s, float* c) {
  float x = t * 4.0f;
  float q = floorf(x + 0.5f);
  float r = x - q;  // [-0.5, 0.5] quarter turns
  int32_t qi = ((int32_t)q) & 3;
  float th = r * 1.57079632679489662f;
  float th2 = th * th;
  // sin: th (1 - th2/6 (1 - th2/20 (1 - th2/42 (1 - th2/72 (1 - th2/110)))))
  float sp = 1.0f - th2 * (1.0f / 110.0f);
  sp = 1.0f - th2 * (1.0f / 72.0f) * sp;
  sp = 1.0f - th2 * (1.0f / 42.0f) * sp;
  sp = 1.0f - th2 * (1.0f / 20.0f) * sp;
  sp = 1.0f - th2 * (1.0f / 6.0f) * sp;
  float sn = th * sp;
  // cos: 1 - th2/2 (1 - th2/12 (1 - th2/30 (1 - th2/56 (1 - th2/90 (1 - th2/132)))))
  float cp = 1.0f - th2 * (1.0f / 132.0f);
  cp = 1.0f - th2 * (1.0f / 90.0f) * cp;
  cp = 1.0f - th2 * (1.0f / 56.0f) * cp;
  cp = 1.0f - th2 * (1.0f / 30.0f) * cp;
  cp = 1.0f - th2 * (1.0f / 12.0f) * cp;
  float cs = 1.0f - th2 * 0.5f * cp;
  if (qi == 0) {
    *s = sn;
    *c = cs;
  } else if (qi == 1) {
    *s = cs;
    *c = -sn;
  } else if (qi == 2) {
    *s = -sn;
    *c = -cs;
  } else {
    *s = -cs;
    *c = sn;
  }
}

// Counter-based random numbers: the PCG-RXS-M-XS hash of Jarzynski & Olano, "Hash Functions for
// GPU Rendering" (JCGT 2020), applied to (seed, counter). Every (pixel, sample, use) owns a
// counter, so the image is a deterministic function of the seed and of nothing else.
MJ_HD uint32_t pcg_hash(uint32_t v) {
  uint32_t state = v * 747796405u + 2891336453u;
  uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
  return (word >> 22u) ^ word;
}
MJ_HD float rand01(uint32_t seed, uint32_t counter) {
  uint32_t h = pcg_hash(seed ^ pcg_hash(counter));
  return (float)(h >> 8) * (1.0f / 16777216.0f);
}

// Relative luminance of linear Rec. 709 colour (color.py:91-93), plain arithmetic.
MJ_HD float luminance(V3 c) { return c.x * 0.2126f + c.y * 0.7152f + c.z * 0.0722f; }

// Orthonormal basis around a unit vector (Duff et al., "Building an Orthonormal Basis,
// Revisited", JCGT 2017), plain arithmetic.
MJ_HD void orthonormal_basis(V3 n, V3* t1, V3* t2) {
  float sign = n.z >= 0.0f ? 1.0f : -1.0f;
  float a = -1.0f / (sign + n.z);
  float b = n.x * n.y * a;
  *t1 = V3{1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x};
  *t2 = V3{b, sign + n.y * n.y * a, -n.y};
}

MJ_DEV float half_to_float(uint16_t h) { return __half2float(__ushort_as_half(h)); }
MJ_DEV uint16_t float_to_half(float f) { return __half_as_ushort(__float2half_rn(f)); }

template <typename T>
MJ_DEV T batched(const T* ptr, int32_t nbatch, int32_t world, int32_t row_len, int32_t index) {
  return ptr[(int64_t)(world % nbatch) * row_len + index];
}
MJ_DEV float bf(const mjpbr_f32b& a, int32_t world, int32_t row_len, int32_t index) {
  return a.ptr[(int64_t)(world % a.nbatch) * row_len + index];
}
MJ_DEV int32_t bi(const mjpbr_i32b& a, int32_t world, int32_t row_len, int32_t index) {
  return a.ptr[(int64_t)(world % a.nbatch) * row_len + index];
}
MJ_DEV V3 bv3(const mjpbr_f32b& a, int32_t world, int32_t n, int32_t index) {
  const float* p = a.ptr + ((int64_t)(world % a.nbatch) * n + index) * 3;
  return V3{p[0], p[1], p[2]};
}

}  // namespace mjpbr
