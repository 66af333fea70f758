/*
 * CPU oracle of the GB300 render path — TEST INFRASTRUCTURE ONLY.
 *
 * A plain scalar C restatement of julien-blanchon/mujoco_warp_pbr's real-time and path-traced
 * tiers and of its context-creation tables. Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline legs may load it, to check the GPU results (and, timed, as the CPU baseline); the
 * product never calls it.
 *
 * It reads the same MjpbrScene descriptor as libmjpbr (include/mjpbr.h), but with HOST pointers,
 * and it is independent of the CUDA code: no world blocks, no scene BVH (every enabled geom is
 * tested against every ray, in geom order), a brute-force or its own median-split mesh BVH.
 *
 * Arithmetic: compiled with -ffp-contract=off and without fast math, so every float operation is
 * correctly rounded and nothing is fused. Geometry (camera rays, intersections, shadow and mirror
 * rays) evaluates the same expressions in the same order as the CUDA kernels, so segmentation,
 * depth and every shadow/mirror decision are bit-identical; shading uses libm and matches the
 * GPU's colours within 1/255.
 *
 * Parity pinning: the reference's ray/primitive tests, camera rays and RNG live in the absent
 * third-party packages mujoco_warp @6c33934b and warp-lang >= 1.15; they are restated here from
 * MuJoCo's published algorithms (engine_ray.c), Woop et al. 2013 (watertight triangles) and a
 * PCG hash (Jarzynski & Olano 2020). Bit patterns of those functions are therefore "parity
 * unpinned"; results are pinned by the reference's analytic known-answer tests (tests/test_render.py,
 * tests/test_ibl.py, tests/test_effects.py of the reference), restated in tests/test_oracle_kat.py.
 *
 * Reference files followed (paths inside the reference project):
 *   camera rays           mujoco_warp_pbr/_src/camera.py:55-347
 *   traversal semantics   mujoco_warp_pbr/_src/traverse.py:195-325
 *   surface               mujoco_warp_pbr/_src/material.py:290-550, texture.py:104-233
 *   BRDF / lights / colour brdf.py:32-110, lights.py:151-198, color.py:40-119
 *   shading / pixel       render.py:67-395, kernel_inputs.py:207-231
 *   path-traced tier      pathtrace.py:64-424, brdf.py:116-191, envmap.py:433-490
 *   denoiser              denoise.py:72-248
 *   environment           envmap.py:154-303, ibl.py:40-119
 */
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/mjpbr.h"

#ifdef _OPENMP
#include <omp.h>
#endif

#define PI_F 3.14159265358979323846f
static const float MINVAL = 1.0e-15f;
static const float MAXVAL = 1.0e10f;
static const float TOL_REL = 1.0e-5f;
static const float RAY_OFFSET = 1.0e-4f;
static const float SHADOW_GAP = 1.0e-3f;
static const float UNBOUNDED = 1.0e8f;

typedef struct {
  float x, y, z;
} v3;

static inline v3 V(float x, float y, float z) {
  v3 r = {x, y, z};
  return r;
}
static inline v3 vadd(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vneg(v3 a) { return V(-a.x, -a.y, -a.z); }
static inline v3 vmul(v3 a, float s) { return V(a.x * s, a.y * s, a.z * s); }
static inline v3 vdiv(v3 a, float s) { return V(a.x / s, a.y / s, a.z / s); }
static inline v3 vcmul(v3 a, v3 b) { return V(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline float vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline v3 vcross(v3 a, v3 b) { return V(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }
static inline float vlen(v3 a) { return sqrtf(vdot(a, a)); }
static inline v3 vnorm(v3 a) {
  float l = sqrtf(vdot(a, a));
  return l > 0.0f ? vdiv(a, l) : a;
}
static inline float minf(float a, float b) { return a < b ? a : b; }
static inline float maxf(float a, float b) { return a > b ? a : b; }
static inline float clampf_(float x, float lo, float hi) { return minf(maxf(x, lo), hi); }
static inline v3 vmaxs(v3 a, float s) { return V(maxf(a.x, s), maxf(a.y, s), maxf(a.z, s)); }
static inline v3 vmins(v3 a, float s) { return V(minf(a.x, s), minf(a.y, s), minf(a.z, s)); }

/* row-major 3x3 */
static inline v3 mat_mul(const float* m, v3 v) {
  return V(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z, m[6] * v.x + m[7] * v.y + m[8] * v.z);
}
static inline v3 mat_mul_t(const float* m, v3 v) {
  return V(m[0] * v.x + m[3] * v.y + m[6] * v.z, m[1] * v.x + m[4] * v.y + m[7] * v.z, m[2] * v.x + m[5] * v.y + m[8] * v.z);
}

static inline float bf(mjpbr_f32b a, int w, int n, int i) { return a.ptr[(int64_t)(w % a.nbatch) * n + i]; }
static inline int bi(mjpbr_i32b a, int w, int n, int i) { return a.ptr[(int64_t)(w % a.nbatch) * n + i]; }
static inline v3 bv3(mjpbr_f32b a, int w, int n, int i) {
  const float* p = a.ptr + ((int64_t)(w % a.nbatch) * n + i) * 3;
  return V(p[0], p[1], p[2]);
}

/* ------------------------------------------------------------------ deterministic helpers */

/* sin and cos of 2 pi t: quadrant reduction and Taylor polynomials (see common.cuh of the library
 * for the derivation; both evaluate the same plain float expressions). */
static void sincos_turns(float t, float* s, float* c) {
  float x = t * 4.0f;
  float q = floorf(x + 0.5f);
  float r = x - q;
  int qi = ((int)q) & 3;
  float th = r * 1.57079632679489662f;
  float th2 = th * th;
  float sp = 1.0f - th2 * (1.0f / 110.0f);
  sp = 1.0f - th2 * (1.0f / 72.0f) * sp;
  sp = 1.0f - th2 * (1.0f / 42.0f) * sp;
  sp = 1.0f - th2 * (1.0f / 20.0f) * sp;
  sp = 1.0f - th2 * (1.0f / 6.0f) * sp;
  float sn = th * sp;
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

static uint32_t pcg_hash(uint32_t v) {
  uint32_t state = v * 747796405u + 2891336453u;
  uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
  return (word >> 22u) ^ word;
}
static float rand01(uint32_t seed, uint32_t counter) {
  uint32_t h = pcg_hash(seed ^ pcg_hash(counter));
  return (float)(h >> 8) * (1.0f / 16777216.0f);
}

static void orthonormal_basis(v3 n, v3* t1, v3* t2) {
  float sign = n.z >= 0.0f ? 1.0f : -1.0f;
  float a = -1.0f / (sign + n.z);
  float b = n.x * n.y * a;
  *t1 = V(1.0f + sign * n.x * n.x * a, sign * b, -sign * n.x);
  *t2 = V(b, sign + n.y * n.y * a, -n.y);
}

static float half_to_float(uint16_t h) {
  uint32_t sign = (uint32_t)(h >> 15) << 31;
  uint32_t exp = (h >> 10) & 0x1F;
  uint32_t man = h & 0x3FF;
  uint32_t bits;
  if (exp == 0) {
    if (man == 0) {
      bits = sign;
    } else {
      float f = ldexpf((float)man, -24);
      memcpy(&bits, &f, 4);
      bits |= sign;
    }
  } else if (exp == 31) {
    bits = sign | 0x7F800000u | (man << 13);
  } else {
    bits = sign | ((exp + 112) << 23) | (man << 13);
  }
  float f;
  memcpy(&f, &bits, 4);
  return f;
}

static uint16_t float_to_half(float f) {
  /* round to nearest even */
  uint32_t x;
  memcpy(&x, &f, 4);
  uint32_t sign = (x >> 16) & 0x8000u;
  uint32_t e = (x >> 23) & 0xFF;
  uint32_t m = x & 0x7FFFFFu;
  if (e == 0xFF) return (uint16_t)(sign | 0x7C00u | (m ? 0x200u : 0u));
  int exp = (int)e - 127 + 15;
  if (exp >= 31) return (uint16_t)(sign | 0x7C00u);
  if (exp <= 0) {
    if (exp < -10) return (uint16_t)sign;
    m |= 0x800000u;
    int shift = 14 - exp;
    uint32_t hm = m >> shift;
    uint32_t rem = m & ((1u << shift) - 1u);
    uint32_t halfway = 1u << (shift - 1);
    if (rem > halfway || (rem == halfway && (hm & 1u))) hm++;
    return (uint16_t)(sign | hm);
  }
  uint32_t hm = m >> 13;
  uint32_t rem = m & 0x1FFFu;
  uint16_t out = (uint16_t)(sign | ((uint32_t)exp << 10) | hm);
  if (rem > 0x1000u || (rem == 0x1000u && (hm & 1u))) out++;
  return out;
}

/* ------------------------------------------------------------------ primitives (MuJoCo) */

typedef struct {
  v3 pos;
  const float* mat;
  v3 size;
} frame_t;

static void map_local(const frame_t* g, v3 o, v3 d, v3* lo, v3* ld) {
  v3 dif = vsub(o, g->pos);
  *lo = mat_mul_t(g->mat, dif);
  *ld = mat_mul_t(g->mat, d);
}

static float ray_quad(float a, float b, float c, float* x0, float* x1) {
  float det = b * b - a * c;
  if (det < MINVAL) {
    *x0 = -1.0f;
    *x1 = -1.0f;
    return -1.0f;
  }
  det = sqrtf(det);
  *x0 = (-b - det) / a;
  *x1 = (-b + det) / a;
  if (*x0 >= 0.0f) return *x0;
  if (*x1 >= 0.0f) return *x1;
  return -1.0f;
}

static float ray_plane(const frame_t* g, v3 o, v3 d, v3* n) {
  v3 lo, ld;
  map_local(g, o, d, &lo, &ld);
  if (ld.z > -MINVAL) return -1.0f;
  float x = -lo.z / ld.z;
  if (x < 0.0f) return -1.0f;
  float p0 = lo.x + x * ld.x;
  float p1 = lo.y + x * ld.y;
  if ((g->size.x <= 0.0f || fabsf(p0) <= g->size.x) && (g->size.y <= 0.0f || fabsf(p1) <= g->size.y)) {
    *n = V(g->mat[2], g->mat[5], g->mat[8]);
    return x;
  }
  return -1.0f;
}

static float ray_sphere(const frame_t* g, v3 o, v3 d, v3* n) {
  v3 dif = vsub(o, g->pos);
  float a = vdot(d, d);
  float b = vdot(d, dif);
  float c = vdot(dif, dif) - g->size.x * g->size.x;
  float x0, x1;
  float x = ray_quad(a, b, c, &x0, &x1);
  if (x < 0.0f) return -1.0f;
  *n = vnorm(vadd(dif, vmul(d, x)));
  return x;
}

static float ray_ellipsoid(const frame_t* g, v3 o, v3 d, v3* n) {
  v3 lo, ld;
  map_local(g, o, d, &lo, &ld);
  v3 s = V(1.0f / g->size.x, 1.0f / g->size.y, 1.0f / g->size.z);
  v3 sd = vcmul(ld, s), so = vcmul(lo, s);
  float a = vdot(sd, sd), b = vdot(sd, so), c = vdot(so, so) - 1.0f;
  float x0, x1;
  float x = ray_quad(a, b, c, &x0, &x1);
  if (x < 0.0f) return -1.0f;
  v3 p = vadd(lo, vmul(ld, x));
  *n = mat_mul(g->mat, vnorm(vcmul(p, vcmul(s, s))));
  return x;
}

static float ray_capsule(const frame_t* g, v3 o, v3 d, v3* n) {
  v3 lo, ld;
  map_local(g, o, d, &lo, &ld);
  float rad = g->size.x, h = g->size.y;
  float x = -1.0f;
  int part = -1;
  float a = ld.x * ld.x + ld.y * ld.y;
  float b = ld.x * lo.x + ld.y * lo.y;
  float c = lo.x * lo.x + lo.y * lo.y - rad * rad;
  float x0, x1;
  float sol = ray_quad(a, b, c, &x0, &x1);
  if (sol >= 0.0f && fabsf(lo.z + sol * ld.z) <= h) {
    x = sol;
    part = 0;
  }
  float aa = vdot(ld, ld);
  for (int cap = 0; cap < 2; ++cap) {
    float zc = cap == 0 ? h : -h;
    v3 dif = V(lo.x, lo.y, lo.z - zc);
    float bb = vdot(ld, dif);
    float cc = vdot(dif, dif) - rad * rad;
    ray_quad(aa, bb, cc, &x0, &x1);
    float xs[2] = {x0, x1};
    for (int i = 0; i < 2; ++i) {
      float z = lo.z + xs[i] * ld.z;
      int side_ok = cap == 0 ? (z >= h) : (z <= -h);
      if (xs[i] >= 0.0f && side_ok && (x < 0.0f || xs[i] < x)) {
        x = xs[i];
        part = 1 + cap;
      }
    }
  }
  if (x < 0.0f) return -1.0f;
  v3 p = vadd(lo, vmul(ld, x));
  v3 ln = part == 0 ? vnorm(V(p.x, p.y, 0.0f)) : vnorm(V(p.x, p.y, p.z - (part == 1 ? h : -h)));
  *n = mat_mul(g->mat, ln);
  return x;
}

static float ray_cylinder(const frame_t* g, v3 o, v3 d, v3* n) {
  v3 lo, ld;
  map_local(g, o, d, &lo, &ld);
  float rad = g->size.x, h = g->size.y;
  float x = -1.0f;
  int part = -1;
  if (fabsf(ld.z) > MINVAL) {
    for (int cap = 0; cap < 2; ++cap) {
      float zc = cap == 0 ? h : -h;
      float sol = (zc - lo.z) / ld.z;
      if (sol >= 0.0f) {
        float px = lo.x + sol * ld.x, py = lo.y + sol * ld.y;
        if (px * px + py * py <= rad * rad && (x < 0.0f || sol < x)) {
          x = sol;
          part = 1 + cap;
        }
      }
    }
  }
  float a = ld.x * ld.x + ld.y * ld.y;
  float b = ld.x * lo.x + ld.y * lo.y;
  float c = lo.x * lo.x + lo.y * lo.y - rad * rad;
  float x0, x1;
  float sol = ray_quad(a, b, c, &x0, &x1);
  if (sol >= 0.0f && fabsf(lo.z + sol * ld.z) <= h && (x < 0.0f || sol < x)) {
    x = sol;
    part = 0;
  }
  if (x < 0.0f) return -1.0f;
  v3 ln;
  if (part == 0) {
    v3 p = vadd(lo, vmul(ld, x));
    ln = vnorm(V(p.x, p.y, 0.0f));
  } else {
    ln = V(0.0f, 0.0f, part == 1 ? 1.0f : -1.0f);
  }
  *n = mat_mul(g->mat, ln);
  return x;
}

static float ray_box(const frame_t* g, v3 o, v3 d, v3* n) {
  v3 lo, ld;
  map_local(g, o, d, &lo, &ld);
  float lp[3] = {lo.x, lo.y, lo.z}, lv[3] = {ld.x, ld.y, ld.z}, sz[3] = {g->size.x, g->size.y, g->size.z};
  float x = -1.0f;
  int axis = -1;
  float side_f = 0.0f;
  for (int i = 0; i < 3; ++i) {
    if (fabsf(lv[i]) > MINVAL) {
      for (int side = -1; side <= 1; side += 2) {
        float sol = ((float)side * sz[i] - lp[i]) / lv[i];
        if (sol >= 0.0f) {
          int j = i == 0 ? 1 : 0, k = i == 2 ? 1 : 2;
          if (fabsf(lp[j] + sol * lv[j]) <= sz[j] && fabsf(lp[k] + sol * lv[k]) <= sz[k] && (x < 0.0f || sol < x)) {
            x = sol;
            axis = i;
            side_f = (float)side;
          }
        }
      }
    }
  }
  if (x < 0.0f) return -1.0f;
  *n = V(g->mat[axis] * side_f, g->mat[3 + axis] * side_f, g->mat[6 + axis] * side_f);
  return x;
}

/* ------------------------------------------------------------------ triangles (Woop 2013) */

typedef struct {
  int kx, ky, kz;
  float sx, sy, sz;
  v3 o;
} woop_t;

static float comp(v3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

static woop_t woop_setup(v3 o, v3 d) {
  woop_t w;
  float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  int kx = kz == 2 ? 0 : kz + 1;
  int ky = kx == 2 ? 0 : kx + 1;
  float dd[3] = {d.x, d.y, d.z};
  if (dd[kz] < 0.0f) {
    int t = kx;
    kx = ky;
    ky = t;
  }
  w.kx = kx;
  w.ky = ky;
  w.kz = kz;
  w.sx = dd[kx] / dd[kz];
  w.sy = dd[ky] / dd[kz];
  w.sz = 1.0f / dd[kz];
  w.o = o;
  return w;
}

static float woop_hit(const woop_t* w, v3 v0, v3 v1, v3 v2, float tmax, float* bu, float* bv) {
  v3 A = vsub(v0, w->o), B = vsub(v1, w->o), C = vsub(v2, w->o);
  float az = comp(A, w->kz), bz = comp(B, w->kz), cz = comp(C, w->kz);
  float ax = comp(A, w->kx) - w->sx * az, ay = comp(A, w->ky) - w->sy * az;
  float bx = comp(B, w->kx) - w->sx * bz, by = comp(B, w->ky) - w->sy * bz;
  float cx = comp(C, w->kx) - w->sx * cz, cy = comp(C, w->ky) - w->sy * cz;
  float U = cx * by - cy * bx;
  float Vv = ax * cy - ay * cx;
  float W = bx * ay - by * ax;
  if ((U < 0.0f || Vv < 0.0f || W < 0.0f) && (U > 0.0f || Vv > 0.0f || W > 0.0f)) return -1.0f;
  float det = U + Vv + W;
  if (det == 0.0f) return -1.0f;
  float T = U * (w->sz * az) + Vv * (w->sz * bz) + W * (w->sz * cz);
  float t = T / det;
  if (!(t >= 0.0f && t < tmax)) return -1.0f;
  *bu = U / det;
  *bv = Vv / det;
  return t;
}

/* The oracle's own mesh BVH (median split, up to 4 triangles per leaf), used to make the CPU
 * baseline representative; brute force over every face stays available (oracle_set_mesh_bvh(0))
 * and both give the same closest hit. */
typedef struct {
  float lo[3], hi[3];
  int left, right; /* children, or -1 */
  int first, count; /* leaf triangles (indices into order) */
} onode_t;

typedef struct {
  onode_t* nodes;
  int* order; /* face indices */
  int nnode;
} obvh_t;

static int g_use_mesh_bvh = 1;
static obvh_t* g_mesh_bvh = NULL;
static int g_mesh_bvh_count = 0;

static int obvh_build_rec(obvh_t* b, const float* cen, const float* blo, const float* bhi, int begin, int end) {
  int idx = b->nnode++;
  onode_t* nd = &b->nodes[idx];
  for (int a = 0; a < 3; ++a) {
    nd->lo[a] = 1e30f;
    nd->hi[a] = -1e30f;
  }
  for (int i = begin; i < end; ++i) {
    int f = b->order[i];
    for (int a = 0; a < 3; ++a) {
      if (blo[f * 3 + a] < nd->lo[a]) nd->lo[a] = blo[f * 3 + a];
      if (bhi[f * 3 + a] > nd->hi[a]) nd->hi[a] = bhi[f * 3 + a];
    }
  }
  for (int a = 0; a < 3; ++a) {
    float pad = 1.0e-5f * (1.0f + maxf(fabsf(nd->lo[a]), fabsf(nd->hi[a])));
    nd->lo[a] -= pad;
    nd->hi[a] += pad;
  }
  if (end - begin <= 4) {
    nd->left = nd->right = -1;
    nd->first = begin;
    nd->count = end - begin;
    return idx;
  }
  /* median along the widest centroid axis (insertion-free: partial selection by sorting) */
  float clo[3] = {1e30f, 1e30f, 1e30f}, chi[3] = {-1e30f, -1e30f, -1e30f};
  for (int i = begin; i < end; ++i) {
    int f = b->order[i];
    for (int a = 0; a < 3; ++a) {
      if (cen[f * 3 + a] < clo[a]) clo[a] = cen[f * 3 + a];
      if (cen[f * 3 + a] > chi[a]) chi[a] = cen[f * 3 + a];
    }
  }
  int axis = 0;
  for (int a = 1; a < 3; ++a)
    if (chi[a] - clo[a] > chi[axis] - clo[axis]) axis = a;
  /* simple in-place partition around the centroid midpoint, median fallback */
  float mid = 0.5f * (clo[axis] + chi[axis]);
  int i = begin, j = end - 1;
  while (i <= j) {
    if (cen[b->order[i] * 3 + axis] < mid) {
      ++i;
    } else {
      int t = b->order[i];
      b->order[i] = b->order[j];
      b->order[j] = t;
      --j;
    }
  }
  int m = i;
  if (m == begin || m == end) m = (begin + end) / 2;
  int l = obvh_build_rec(b, cen, blo, bhi, begin, m);
  int r = obvh_build_rec(b, cen, blo, bhi, m, end);
  b->nodes[idx].left = l;
  b->nodes[idx].right = r;
  b->nodes[idx].first = 0;
  b->nodes[idx].count = 0;
  return idx;
}

static void obvh_build(const MjpbrScene* s, int mesh, int nface, obvh_t* b) {
  int vadr = s->mesh_vertadr[mesh], fadr = s->mesh_faceadr[mesh];
  float* cen = (float*)malloc(sizeof(float) * 3 * nface);
  float* blo = (float*)malloc(sizeof(float) * 3 * nface);
  float* bhi = (float*)malloc(sizeof(float) * 3 * nface);
  b->order = (int*)malloc(sizeof(int) * nface);
  b->nodes = (onode_t*)malloc(sizeof(onode_t) * 2 * nface);
  b->nnode = 0;
  for (int f = 0; f < nface; ++f) {
    const int32_t* fv = s->mesh_face + (int64_t)(fadr + f) * 3;
    for (int a = 0; a < 3; ++a) {
      float lo = 1e30f, hi = -1e30f;
      for (int k = 0; k < 3; ++k) {
        float x = s->mesh_vert[(int64_t)(vadr + fv[k]) * 3 + a];
        lo = x < lo ? x : lo;
        hi = x > hi ? x : hi;
      }
      blo[f * 3 + a] = lo;
      bhi[f * 3 + a] = hi;
      cen[f * 3 + a] = 0.5f * (lo + hi);
    }
    b->order[f] = f;
  }
  obvh_build_rec(b, cen, blo, bhi, 0, nface);
  free(cen);
  free(blo);
  free(bhi);
}

static float obox(const onode_t* n, v3 o, v3 inv, float tmax) {
  float t1x = (n->lo[0] - o.x) * inv.x, t2x = (n->hi[0] - o.x) * inv.x;
  float t1y = (n->lo[1] - o.y) * inv.y, t2y = (n->hi[1] - o.y) * inv.y;
  float t1z = (n->lo[2] - o.z) * inv.z, t2z = (n->hi[2] - o.z) * inv.z;
  float tmin = maxf(maxf(minf(t1x, t2x), minf(t1y, t2y)), minf(t1z, t2z));
  float tmx = minf(minf(maxf(t1x, t2x), maxf(t1y, t2y)), maxf(t1z, t2z));
  float entry = maxf(tmin, 0.0f);
  return (tmx >= entry && entry < tmax) ? entry : -1.0f;
}

static float rcp_safe(float x) { return 1.0f / (fabsf(x) > 1.0e-30f ? x : (x >= 0.0f ? 1.0e-30f : -1.0e-30f)); }

/* Triangle test of face f (mesh-relative) for mesh_query. */
static float face_hit(const MjpbrScene* s, int vadr, int fadr, int f, const woop_t* w, float best, float* u, float* v,
                      v3* e1o, v3* e2o) {
  const int32_t* fv = s->mesh_face + (int64_t)(fadr + f) * 3;
  const float* p0 = s->mesh_vert + (int64_t)(vadr + fv[0]) * 3;
  const float* p1 = s->mesh_vert + (int64_t)(vadr + fv[1]) * 3;
  const float* p2 = s->mesh_vert + (int64_t)(vadr + fv[2]) * 3;
  v3 v0 = V(p0[0], p0[1], p0[2]), v1 = V(p1[0], p1[1], p1[2]), v2 = V(p2[0], p2[1], p2[2]);
  *e1o = vsub(v1, v0);
  *e2o = vsub(v2, v0);
  return woop_hit(w, v0, v1, v2, best, u, v);
}

/* Closest (any_hit: first) triangle of a mesh in [0, tmax): brute force over its faces, or the
 * oracle's mesh BVH when built. */
static float mesh_query(const MjpbrScene* s, int mesh, int nface, v3 lo, v3 ld, float tmax, int cull, int any_hit,
                        v3* nl, float* bu, float* bv, int* face) {
  woop_t w = woop_setup(lo, ld);
  int vadr = s->mesh_vertadr[mesh], fadr = s->mesh_faceadr[mesh];
  float best = tmax;
  int found = -1;
  v3 e1b = V(0, 0, 0), e2b = V(0, 0, 0);
  float ub = 0.0f, vb = 0.0f;
  if (g_mesh_bvh && mesh < g_mesh_bvh_count && g_mesh_bvh[mesh].nodes) {
    const obvh_t* b = &g_mesh_bvh[mesh];
    v3 inv = V(rcp_safe(ld.x), rcp_safe(ld.y), rcp_safe(ld.z));
    int stack[64];
    float st_t[64];
    int sp = 0;
    if (obox(&b->nodes[0], lo, inv, best) >= 0.0f) {
      stack[0] = 0;
      st_t[0] = 0.0f;
      sp = 1;
    }
    while (sp > 0) {
      --sp;
      if (st_t[sp] >= best) continue;
      const onode_t* nd = &b->nodes[stack[sp]];
      if (nd->left >= 0) {
        float ta = obox(&b->nodes[nd->left], lo, inv, best), tb = obox(&b->nodes[nd->right], lo, inv, best);
        int near = nd->left, far = nd->right;
        float tn = ta, tf = tb;
        if (tb >= 0.0f && (ta < 0.0f || tb < ta)) {
          near = nd->right;
          far = nd->left;
          tn = tb;
          tf = ta;
        }
        if (tf >= 0.0f && sp < 64) {
          stack[sp] = far;
          st_t[sp++] = tf;
        }
        if (tn >= 0.0f && sp < 64) {
          stack[sp] = near;
          st_t[sp++] = tn;
        }
        continue;
      }
      for (int k = nd->first; k < nd->first + nd->count; ++k) {
        int f = b->order[k];
        float u, v;
        v3 e1, e2;
        float t = face_hit(s, vadr, fadr, f, &w, best, &u, &v, &e1, &e2);
        if (t < 0.0f) continue;
        if (!any_hit && cull && vdot(ld, vcross(e1, e2)) > 0.0f) continue;
        if (any_hit) return t;
        best = t;
        found = f;
        e1b = e1;
        e2b = e2;
        ub = u;
        vb = v;
      }
    }
    if (found < 0) return -1.0f;
    *nl = vnorm(vcross(e1b, e2b));
    *bu = ub;
    *bv = vb;
    *face = found;
    return best;
  }
  for (int f = 0; f < nface; ++f) {
    const int32_t* fv = s->mesh_face + (int64_t)(fadr + f) * 3;
    const float* p0 = s->mesh_vert + (int64_t)(vadr + fv[0]) * 3;
    const float* p1 = s->mesh_vert + (int64_t)(vadr + fv[1]) * 3;
    const float* p2 = s->mesh_vert + (int64_t)(vadr + fv[2]) * 3;
    v3 v0 = V(p0[0], p0[1], p0[2]), v1 = V(p1[0], p1[1], p1[2]), v2 = V(p2[0], p2[1], p2[2]);
    float u, v;
    float t = woop_hit(&w, v0, v1, v2, best, &u, &v);
    if (t < 0.0f) continue;
    v3 e1 = vsub(v1, v0), e2 = vsub(v2, v0);
    if (!any_hit && cull && vdot(ld, vcross(e1, e2)) > 0.0f) continue;
    if (any_hit) return t;
    best = t;
    found = f;
    e1b = e1;
    e2b = e2;
    ub = u;
    vb = v;
  }
  if (found < 0) return -1.0f;
  *nl = vnorm(vcross(e1b, e2b));
  *bu = ub;
  *bv = vb;
  *face = found;
  return best;
}

/* Height fields: MuJoCo's height-field solid (an nrow x ncol elevation grid over
 * [-size0, size0] x [-size1, size1], z = size2 * elevation, on a base at z = -size3), triangulated
 * by the oracle itself into a closed mesh and queried by brute force. The reference traces MuJoCo
 * Warp's height-field mesh (mujoco_warp_pbr/_src/traverse.py:161-164, third party). Faces, in
 * order: the top, two per cell (r, c), (r, c+1), (r+1, c+1) and (r, c), (r+1, c+1), (r+1, c),
 * cells row by row; the side walls, two per border segment p -> q of the border walked
 * counter-clockwise seen from +z from sample (0, 0) (top p, base q, top q and top p, base p,
 * base q); the base, a fan centre, base q, base p over the same segments. Outward winding.
 * Coordinates in double, rounded once to float. Set by oracle_set_hfields. */
typedef struct {
  int nvert, nface;
  float* vert;  /* (nvert, 3) */
  int32_t* face; /* (nface, 3) */
} ohf_t;

static ohf_t* g_hf = NULL;
static int g_nhf = 0;

static void hf_free(void) {
  for (int h = 0; h < g_nhf; ++h) {
    free(g_hf[h].vert);
    free(g_hf[h].face);
  }
  free(g_hf);
  g_hf = NULL;
  g_nhf = 0;
}

static void hf_build(ohf_t* o, int nr, int nc, const float* size, const float* elev) {
  int ntop = nr * nc, nring = 2 * (nr - 1) + 2 * (nc - 1);
  o->nvert = 2 * ntop + 1;
  o->nface = 2 * (nr - 1) * (nc - 1) + 3 * nring;
  o->vert = (float*)malloc(sizeof(float) * 3 * (size_t)o->nvert);
  o->face = (int32_t*)malloc(sizeof(int32_t) * 3 * (size_t)o->nface);
  for (int r = 0; r < nr; ++r) {
    for (int c = 0; c < nc; ++c) {
      double x = (double)size[0] * (2.0 * c / (nc - 1) - 1.0);
      double y = (double)size[1] * (2.0 * r / (nr - 1) - 1.0);
      float* top = o->vert + 3 * (r * nc + c);
      float* bot = o->vert + 3 * (ntop + r * nc + c);
      top[0] = bot[0] = (float)x;
      top[1] = bot[1] = (float)y;
      top[2] = (float)((double)size[2] * (double)elev[r * nc + c]);
      bot[2] = (float)(-(double)size[3]);
    }
  }
  float* centre = o->vert + 3 * (2 * ntop);
  centre[0] = 0.0f;
  centre[1] = 0.0f;
  centre[2] = (float)(-(double)size[3]);
  int32_t* f = o->face;
  for (int r = 0; r + 1 < nr; ++r) {
    for (int c = 0; c + 1 < nc; ++c) {
      int a = r * nc + c, b = r * nc + c + 1, d = (r + 1) * nc + c + 1, e = (r + 1) * nc + c;
      f[0] = a, f[1] = b, f[2] = d;
      f[3] = a, f[4] = d, f[5] = e;
      f += 6;
    }
  }
  /* border ring, counter-clockwise from +z */
  int* ring = (int*)malloc(sizeof(int) * (size_t)nring);
  int k = 0;
  for (int c = 0; c + 1 < nc; ++c) ring[k++] = c;
  for (int r = 0; r + 1 < nr; ++r) ring[k++] = r * nc + nc - 1;
  for (int c = nc - 1; c > 0; --c) ring[k++] = (nr - 1) * nc + c;
  for (int r = nr - 1; r > 0; --r) ring[k++] = r * nc;
  for (int i = 0; i < nring; ++i) {
    int p = ring[i], q = ring[(i + 1) % nring];
    f[0] = p, f[1] = q + ntop, f[2] = q;
    f[3] = p, f[4] = p + ntop, f[5] = q + ntop;
    f += 6;
  }
  for (int i = 0; i < nring; ++i) {
    int p = ring[i], q = ring[(i + 1) % nring];
    f[0] = 2 * ntop, f[1] = q + ntop, f[2] = p + ntop;
    f += 3;
  }
  free(ring);
}

/* Replaces the oracle's height fields (MuJoCo's hfield_* arrays; n = 0 clears them). Returns 0,
 * or 1 for a grid smaller than 2 x 2. */
int oracle_set_hfields(int n, const int32_t* nrow, const int32_t* ncol, const float* size, const int32_t* adr,
                       const float* data) {
  hf_free();
  if (n <= 0) return 0;
  for (int h = 0; h < n; ++h)
    if (nrow[h] < 2 || ncol[h] < 2) return 1;
  g_hf = (ohf_t*)calloc((size_t)n, sizeof(ohf_t));
  g_nhf = n;
  for (int h = 0; h < n; ++h) hf_build(&g_hf[h], nrow[h], ncol[h], size + 4 * h, data + adr[h]);
  return 0;
}

/* Copies height field h's triangulation out (for tests): counts always, arrays when not NULL. */
int oracle_hfield_mesh(int h, int* nvert, int* nface, float* vert, int32_t* face) {
  if (h < 0 || h >= g_nhf) return 1;
  *nvert = g_hf[h].nvert;
  *nface = g_hf[h].nface;
  if (vert) memcpy(vert, g_hf[h].vert, sizeof(float) * 3 * (size_t)g_hf[h].nvert);
  if (face) memcpy(face, g_hf[h].face, sizeof(int32_t) * 3 * (size_t)g_hf[h].nface);
  return 0;
}

/* Closest (any_hit: first) face of height field h in [0, tmax), brute force in face order. */
static float hfield_query(int h, v3 lo, v3 ld, float tmax, int cull, int any_hit, v3* nl, float* bu, float* bv,
                          int* face) {
  const ohf_t* o = &g_hf[h];
  woop_t w = woop_setup(lo, ld);
  float best = tmax;
  int found = -1;
  v3 e1b = V(0, 0, 0), e2b = V(0, 0, 0);
  float ub = 0.0f, vb = 0.0f;
  for (int f = 0; f < o->nface; ++f) {
    const int32_t* fv = o->face + 3 * f;
    const float* p0 = o->vert + 3 * fv[0];
    const float* p1 = o->vert + 3 * fv[1];
    const float* p2 = o->vert + 3 * fv[2];
    v3 v0 = V(p0[0], p0[1], p0[2]), v1 = V(p1[0], p1[1], p1[2]), v2 = V(p2[0], p2[1], p2[2]);
    float u, v;
    float t = woop_hit(&w, v0, v1, v2, best, &u, &v);
    if (t < 0.0f) continue;
    v3 e1 = vsub(v1, v0), e2 = vsub(v2, v0);
    if (!any_hit && cull && vdot(ld, vcross(e1, e2)) > 0.0f) continue;
    if (any_hit) return t;
    best = t;
    found = f;
    e1b = e1;
    e2b = e2;
    ub = u;
    vb = v;
  }
  if (found < 0) return -1.0f;
  *nl = vnorm(vcross(e1b, e2b));
  *bu = ub;
  *bv = vb;
  *face = found;
  return best;
}

/* ------------------------------------------------------------------ scene queries */

typedef struct {
  const MjpbrScene* s;
  const int32_t* mesh_nface; /* faces per mesh */
  int w;
} world_t;

typedef struct {
  int geom;
  float dist;
  v3 normal;
  float u, v;
  int face, mesh;
} hit_t;

static void geom_rgba(const MjpbrScene* s, int w, int g, float* rgba, int* matid_out) {
  int matid = bi(s->geom_matid, w, s->ngeom, g);
  const float* p = s->geom_rgba.ptr + ((int64_t)(w % s->geom_rgba.nbatch) * s->ngeom + g) * 4;
  for (int k = 0; k < 4; ++k) rgba[k] = p[k];
  if (matid >= 0 && rgba[0] == 0.5f && rgba[1] == 0.5f && rgba[2] == 0.5f && rgba[3] == 1.0f && s->mat_rgba.ptr) {
    const float* q = s->mat_rgba.ptr + ((int64_t)(w % s->mat_rgba.nbatch) * s->nmat + matid) * 4;
    for (int k = 0; k < 4; ++k) rgba[k] = q[k];
  }
  *matid_out = matid;
}

static void geom_frame(const world_t* W, int g, frame_t* f) {
  const MjpbrScene* s = W->s;
  const float* xp = s->geom_xpos + ((int64_t)W->w * s->ngeom + g) * 3;
  f->pos = V(xp[0], xp[1], xp[2]);
  f->mat = s->geom_xmat + ((int64_t)W->w * s->ngeom + g) * 9;
  f->size = bv3(s->geom_size, W->w, s->ngeom, g);
}

/* Distance to geom g (or -1) with world normal; mesh hit details. */
static float intersect(const world_t* W, int g, v3 o, v3 d, float max_t, int cull, int any_hit, v3* n, float* u,
                       float* v, int* face, int* mesh) {
  const MjpbrScene* s = W->s;
  frame_t f;
  geom_frame(W, g, &f);
  int type = s->geom_type[g];
  switch (type) {
    case MJPBR_GEOM_PLANE:
      return ray_plane(&f, o, d, n);
    case MJPBR_GEOM_SPHERE:
      return ray_sphere(&f, o, d, n);
    case MJPBR_GEOM_ELLIPSOID:
      return ray_ellipsoid(&f, o, d, n);
    case MJPBR_GEOM_CAPSULE:
      return ray_capsule(&f, o, d, n);
    case MJPBR_GEOM_CYLINDER:
      return ray_cylinder(&f, o, d, n);
    case MJPBR_GEOM_BOX:
      return ray_box(&f, o, d, n);
    case MJPBR_GEOM_MESH:
    case MJPBR_GEOM_SDF: {
      int mid = s->geom_dataid.ptr ? bi(s->geom_dataid, W->w, s->ngeom, g) : -1;
      if (mid < 0 || !s->mesh_vert || !W->mesh_nface) return -1.0f;
      v3 lo, ld, nl = V(0, 0, 0);
      map_local(&f, o, d, &lo, &ld);
      float t = mesh_query(s, mid, W->mesh_nface[mid], lo, ld, max_t, cull, any_hit, &nl, u, v, face);
      *n = any_hit ? V(0, 0, 0) : mat_mul(f.mat, nl);
      *mesh = mid;
      return t;
    }
    case MJPBR_GEOM_HFIELD: {
      int hid = s->geom_dataid.ptr ? bi(s->geom_dataid, W->w, s->ngeom, g) : -1;
      if (hid < 0 || hid >= g_nhf) return -1.0f;
      v3 lo, ld, nl = V(0, 0, 0);
      map_local(&f, o, d, &lo, &ld);
      float t = hfield_query(hid, lo, ld, max_t, cull, any_hit, &nl, u, v, face);
      *n = any_hit ? V(0, 0, 0) : mat_mul(f.mat, nl);
      return t;
    }
    default:
      return -1.0f;
  }
}

static int geom_visible(const world_t* W, int g) {
  float rgba[4];
  int matid;
  geom_rgba(W->s, W->w, g, rgba, &matid);
  return rgba[3] != 0.0f;
}

/* Closest hit over every enabled geom (traverse.py:280-321 without the tree: same tie-break). */
static hit_t closest(const world_t* W, v3 o, v3 d, float max_dist, int cull) {
  const MjpbrScene* s = W->s;
  hit_t h;
  h.geom = -1;
  h.dist = max_dist;
  h.normal = V(0, 0, 0);
  h.u = h.v = 0.0f;
  h.face = h.mesh = -1;
  for (int slot = 0; slot < s->nbvh_geom; ++slot) {
    int g = s->enabled_geom_ids[slot];
    if (!geom_visible(W, g)) continue;
    float cut = h.dist * (1.0f + TOL_REL) + 1.0e-7f;
    v3 n = V(0, 0, 0);
    float u = 0.0f, v = 0.0f;
    int face = -1, mesh = -1;
    float dd = intersect(W, g, o, d, cut, cull, 0, &n, &u, &v, &face, &mesh);
    if (cull && dd >= 0.0f && vdot(d, n) > 0.0f) dd = -1.0f;
    float tol = TOL_REL * maxf(h.dist, 1.0f);
    int closer = (dd < h.dist - tol) || (fabsf(dd - h.dist) <= tol && (h.geom < 0 || g > h.geom));
    if (dd >= 0.0f && closer) {
      h.dist = dd;
      h.normal = n;
      h.geom = g;
      h.u = u;
      h.v = v;
      h.face = face;
      h.mesh = mesh;
    }
  }
  return h;
}

static int occluded(const world_t* W, v3 o, v3 d, float max_dist, int cull) {
  const MjpbrScene* s = W->s;
  for (int slot = 0; slot < s->nbvh_geom; ++slot) {
    int g = s->enabled_geom_ids[slot];
    if (!geom_visible(W, g)) continue;
    v3 n = V(0, 0, 0);
    float u, v;
    int face = -1, mesh = -1;
    float dd = intersect(W, g, o, d, max_dist, cull, 1, &n, &u, &v, &face, &mesh);
    if (cull && dd >= 0.0f && vdot(d, n) > 0.0f) dd = -1.0f;
    if (dd >= 0.0f && dd < max_dist) return 1;
  }
  return 0;
}

/* ------------------------------------------------------------------ tables and textures */

static void sample_dfg(const float* lut, int n, float nov, float pr, float* dx, float* dy) {
  float fx = nov * (float)n - 0.5f, fy = pr * (float)n - 0.5f;
  float x0f = floorf(fx), y0f = floorf(fy);
  float tx = fx - x0f, ty = fy - y0f;
  int x0 = (int)x0f, y0 = (int)y0f;
  int x1 = x0 + 1, y1 = y0 + 1;
  x0 = x0 < 0 ? 0 : (x0 > n - 1 ? n - 1 : x0);
  x1 = x1 < 0 ? 0 : (x1 > n - 1 ? n - 1 : x1);
  y0 = y0 < 0 ? 0 : (y0 > n - 1 ? n - 1 : y0);
  y1 = y1 < 0 ? 0 : (y1 > n - 1 ? n - 1 : y1);
  const float *a = lut + (y0 * n + x0) * 2, *b = lut + (y0 * n + x1) * 2, *c = lut + (y1 * n + x0) * 2,
              *d = lut + (y1 * n + x1) * 2;
  float ax = a[0] + (b[0] - a[0]) * tx, ay = a[1] + (b[1] - a[1]) * tx;
  float cx = c[0] + (d[0] - c[0]) * tx, cy = c[1] + (d[1] - c[1]) * tx;
  *dx = ax + (cx - ax) * ty;
  *dy = ay + (cy - ay) * ty;
}

static void fetch_texel(const MjpbrTexture* t, const uint8_t* data, int level, int w, int x, int y, float* out) {
  int64_t idx = (int64_t)y * w + x;
  if (t->format == MJPBR_TEX_RGBA8) {
    const uint8_t* p = data + t->level_offset[level] + idx * 4;
    for (int k = 0; k < 4; ++k) out[k] = (float)p[k] * (1.0f / 255.0f);
  } else {
    const uint16_t* p = (const uint16_t*)(data + t->level_offset[level]) + idx * 4;
    for (int k = 0; k < 4; ++k) out[k] = half_to_float(p[k]);
  }
}

static int wrapi(int i, int n) {
  int r = i % n;
  return r < 0 ? r + n : r;
}
static int clampi(int i, int lo, int hi) { return i < lo ? lo : (i > hi ? hi : i); }

static void sample_level(const MjpbrTexture* t, const uint8_t* data, int level, float u, float v, int wrap_u, int wrap_v,
                         float* out) {
  int w = t->width >> level, h = t->height >> level;
  if (w < 1) w = 1;
  if (h < 1) h = 1;
  float fx = u * (float)w - 0.5f, fy = v * (float)h - 0.5f;
  float x0f = floorf(fx), y0f = floorf(fy);
  float tx = fx - x0f, ty = fy - y0f;
  int x0 = (int)x0f, y0 = (int)y0f, x1 = x0 + 1, y1 = y0 + 1;
  if (wrap_u) {
    x0 = wrapi(x0, w);
    x1 = wrapi(x1, w);
  } else {
    x0 = clampi(x0, 0, w - 1);
    x1 = clampi(x1, 0, w - 1);
  }
  if (wrap_v) {
    y0 = wrapi(y0, h);
    y1 = wrapi(y1, h);
  } else {
    y0 = clampi(y0, 0, h - 1);
    y1 = clampi(y1, 0, h - 1);
  }
  float a[4], b[4], c[4], d[4];
  fetch_texel(t, data, level, w, x0, y0, a);
  fetch_texel(t, data, level, w, x1, y0, b);
  fetch_texel(t, data, level, w, x0, y1, c);
  fetch_texel(t, data, level, w, x1, y1, d);
  for (int k = 0; k < 4; ++k) {
    float top = a[k] + (b[k] - a[k]) * tx;
    float bot = c[k] + (d[k] - c[k]) * tx;
    out[k] = top + (bot - top) * ty;
  }
}

static void sample_trilinear(const MjpbrTexture* t, const uint8_t* data, float u, float v, float lod, int wrap_u,
                             int wrap_v, float* out) {
  float l = clampf_(lod, 0.0f, (float)(t->nlevel - 1));
  float l0f = floorf(l);
  int l0 = (int)l0f;
  float f = l - l0f;
  sample_level(t, data, l0, u, v, wrap_u, wrap_v, out);
  if (f <= 0.0f || l0 + 1 >= t->nlevel) return;
  float b[4];
  sample_level(t, data, l0 + 1, u, v, wrap_u, wrap_v, b);
  for (int k = 0; k < 4; ++k) out[k] = out[k] + (b[k] - out[k]) * f;
}

static void direction_to_uv(v3 d, float yaw, float* u, float* v) {
  float phi = atan2f(d.y, d.x) - yaw;
  float uu = 0.5f + phi * (0.5f / PI_F);
  *u = uu - floorf(uu);
  *v = acosf(clampf_(d.z, -1.0f, 1.0f)) * (1.0f / PI_F);
}

static v3 rotate_yaw(v3 d, float yaw) {
  float c = cosf(yaw), s = sinf(yaw);
  return V(c * d.x - s * d.y, s * d.x + c * d.y, d.z);
}

static v3 eval_sh9(const float* sh, v3 n) {
  float x = n.x, y = n.y, z = n.z;
  float b[9] = {0.282095f,       0.488603f * y,       0.488603f * z, 0.488603f * x, 1.092548f * x * y,
                1.092548f * y * z, 0.315392f * (3.0f * z * z - 1.0f), 1.092548f * x * z, 0.546274f * (x * x - y * y)};
  v3 c = V(0, 0, 0);
  for (int k = 0; k < 9; ++k) c = vadd(c, vmul(V(sh[3 * k], sh[3 * k + 1], sh[3 * k + 2]), b[k]));
  return vmaxs(c, 0.0f);
}

static v3 sample_radiance(const MjpbrScene* s, int env, v3 d, float yaw, float lod) {
  float u, v, out[4];
  direction_to_uv(d, yaw, &u, &v);
  sample_trilinear(&s->env_radiance[env], s->env_data, u, v, maxf(lod, 0.0f), 1, 0, out);
  return V(out[0], out[1], out[2]);
}

static void stack_texel(const uint16_t* st, int w, int h, int level, int x, int y, float* out) {
  const uint16_t* p = st + (((int64_t)level * h + y) * w + x) * 4;
  for (int k = 0; k < 4; ++k) out[k] = half_to_float(p[k]);
}

static v3 sample_prefiltered(const MjpbrScene* s, int env, v3 d, float yaw, float pr) {
  int levels = s->prefilter_levels, h = s->prefilter_height, w = s->prefilter_width;
  const uint16_t* st = s->env_prefiltered + (int64_t)env * levels * h * w * 4;
  float u, v;
  direction_to_uv(d, yaw, &u, &v);
  float wz = (clampf_(pr, 0.0f, 1.0f) * ((float)levels - 1.0f) + 0.5f) / (float)levels;
  float fz = wz * (float)levels - 0.5f;
  float z0f = floorf(fz), tz = fz - z0f;
  int z0 = clampi((int)z0f, 0, levels - 1), z1 = clampi((int)z0f + 1, 0, levels - 1);
  float fx = u * (float)w - 0.5f, fy = v * (float)h - 0.5f;
  float x0f = floorf(fx), y0f = floorf(fy);
  float tx = fx - x0f, ty = fy - y0f;
  int x0 = wrapi((int)x0f, w), x1 = wrapi((int)x0f + 1, w);
  int y0 = clampi((int)y0f, 0, h - 1), y1 = clampi((int)y0f + 1, 0, h - 1);
  float r[2][4];
  for (int zz = 0; zz < 2; ++zz) {
    int z = zz == 0 ? z0 : z1;
    float a[4], b[4], c[4], dd[4];
    stack_texel(st, w, h, z, x0, y0, a);
    stack_texel(st, w, h, z, x1, y0, b);
    stack_texel(st, w, h, z, x0, y1, c);
    stack_texel(st, w, h, z, x1, y1, dd);
    for (int k = 0; k < 4; ++k) {
      float top = a[k] + (b[k] - a[k]) * tx, bot = c[k] + (dd[k] - c[k]) * tx;
      r[zz][k] = top + (bot - top) * ty;
    }
  }
  return V(r[0][0] + (r[1][0] - r[0][0]) * tz, r[0][1] + (r[1][1] - r[0][1]) * tz, r[0][2] + (r[1][2] - r[0][2]) * tz);
}

/* ------------------------------------------------------------------ BRDF, lights, colour */

typedef struct {
  v3 base_color;
  float alpha, metallic, roughness, reflectance;
  v3 emissive;
  float occlusion;
} surface_t;

typedef struct {
  float pr, alpha;
  v3 f0, energy_comp, spec_albedo, diffuse_color;
} lobes_t;

static float d_ggx(float noh, float a) {
  float a2 = a * a;
  float f = (noh * a2 - noh) * noh + 1.0f;
  return a2 / (PI_F * f * f);
}
static float v_smith(float nov, float nol, float a) {
  float a2 = a * a;
  float gv = nol * sqrtf(nov * nov * (1.0f - a2) + a2);
  float gl = nov * sqrtf(nol * nol * (1.0f - a2) + a2);
  return 0.5f / (gv + gl);
}
static v3 f_schlick(v3 f0, float f90, float voh) {
  float x = 1.0f - voh, x2 = x * x, fc = x2 * x2 * x;
  return vadd(vmul(f0, 1.0f - fc), V(f90 * fc, f90 * fc, f90 * fc));
}

static lobes_t shading_lobes(const MjpbrScene* s, const surface_t* sf, float nov) {
  lobes_t l;
  l.pr = clampf_(sf->roughness, 0.045f, 1.0f);
  l.alpha = l.pr * l.pr;
  float diel = 0.16f * sf->reflectance * sf->reflectance * (1.0f - sf->metallic);
  l.f0 = vadd(vmul(sf->base_color, sf->metallic), V(diel, diel, diel));
  float dx, dy;
  sample_dfg(s->dfg_lut, s->dfg_size, nov, l.pr, &dx, &dy);
  l.energy_comp = vadd(V(1, 1, 1), vmul(l.f0, 1.0f / maxf(dy, 1.0e-4f) - 1.0f));
  l.spec_albedo = vadd(vmul(vsub(V(1, 1, 1), l.f0), dx), vmul(l.f0, dy));
  l.diffuse_color = vcmul(vmul(sf->base_color, 1.0f - sf->metallic), vsub(V(1, 1, 1), l.spec_albedo));
  return l;
}

typedef struct {
  int type, castshadow, active;
  v3 pos, dir, diffuse, specular, attenuation;
  float intensity, range, bulbradius, cutoff, exponent;
} light_t;

static light_t fetch_light(const MjpbrScene* s, int w, int li) {
  light_t l;
  int n = s->nlight;
  l.type = bi(s->light_type, w, n, li);
  l.castshadow = bi(s->light_castshadow, w, n, li);
  l.active = bi(s->light_active, w, n, li);
  const float* xp = s->light_xpos + ((int64_t)w * n + li) * 3;
  const float* xd = s->light_xdir + ((int64_t)w * n + li) * 3;
  l.pos = V(xp[0], xp[1], xp[2]);
  l.dir = V(xd[0], xd[1], xd[2]);
  l.diffuse = bv3(s->light_diffuse, w, n, li);
  l.specular = bv3(s->light_specular, w, n, li);
  l.attenuation = bv3(s->light_attenuation, w, n, li);
  l.intensity = bf(s->light_intensity, w, n, li);
  l.range = bf(s->light_range, w, n, li);
  l.bulbradius = bf(s->light_bulbradius, w, n, li);
  l.cutoff = bf(s->light_cutoff, w, n, li);
  l.exponent = bf(s->light_exponent, w, n, li);
  return l;
}

static void eval_light(const light_t* light, int light_model, v3 point, v3* l, float* dist, v3* ds, v3* ss) {
  int physical = light_model == MJPBR_LIGHT_MODEL_PHYSICAL;
  float att = 1.0f;
  *dist = 1.0e10f;
  if (light->type == MJPBR_LIGHT_DIRECTIONAL) {
    *l = vneg(light->dir);
  } else {
    v3 to = vsub(light->pos, point);
    *dist = vlen(to);
    *l = vdiv(to, maxf(*dist, 1.0e-9f));
    float d = *dist;
    if (physical) {
      float d2 = d * d, r = maxf(light->range, 1.0e-6f);
      float factor = d2 / (r * r);
      float window = clampf_(1.0f - factor * factor, 0.0f, 1.0f);
      att = window * window / maxf(d2, 1.0e-4f);
    } else {
      att = 1.0f / maxf(light->attenuation.x + light->attenuation.y * d + light->attenuation.z * d * d, 1.0e-9f);
    }
    if (light->type == MJPBR_LIGHT_SPOT) {
      float cos_theta = vdot(vneg(*l), light->dir);
      float outer = light->cutoff * (PI_F / 180.0f);
      float cos_outer = cosf(outer);
      if (physical) {
        float cos_inner = cosf(outer * 0.75f);
        float cone = 1.0f / maxf(cos_inner - cos_outer, 1.0f / 1024.0f);
        float sc = clampf_((cos_theta - cos_outer) * cone, 0.0f, 1.0f);
        att = att * sc * sc;
      } else {
        att = cos_theta < cos_outer ? 0.0f : att * powf(maxf(cos_theta, 0.0f), light->exponent);
      }
    }
  }
  if (physical) {
    v3 sc = vmul(light->diffuse, light->intensity * att);
    *ds = sc;
    *ss = sc;
  } else {
    float k = PI_F * att;
    *ds = vmul(light->diffuse, k);
    *ss = vmul(light->specular, k);
  }
}

static v3 tonemap_pbr_neutral(v3 c) {
  const float start = 0.8f - 0.04f, desat = 0.15f;
  float x = minf(c.x, minf(c.y, c.z));
  float offset = x < 0.08f ? x - 6.25f * x * x : 0.04f;
  c = vsub(c, V(offset, offset, offset));
  float peak = maxf(c.x, maxf(c.y, c.z));
  if (peak < start) return c;
  float d = 1.0f - start;
  float new_peak = 1.0f - d * d / (peak + d - start);
  c = vmul(c, new_peak / peak);
  float g = 1.0f - 1.0f / (desat * (peak - new_peak) + 1.0f);
  return vadd(vmul(c, 1.0f - g), V(new_peak * g, new_peak * g, new_peak * g));
}

static v3 tonemap_aces(v3 c) {
  v3 v = V(0.59719f * c.x + 0.35458f * c.y + 0.04823f * c.z, 0.07600f * c.x + 0.90834f * c.y + 0.01566f * c.z,
           0.02840f * c.x + 0.13383f * c.y + 0.83777f * c.z);
  v3 num = vsub(vcmul(v, vadd(v, V(0.0245786f, 0.0245786f, 0.0245786f))), V(0.000090537f, 0.000090537f, 0.000090537f));
  v3 den = vadd(vcmul(v, vadd(vmul(v, 0.983729f), V(0.4329510f, 0.4329510f, 0.4329510f))), V(0.238081f, 0.238081f, 0.238081f));
  v = V(num.x / den.x, num.y / den.y, num.z / den.z);
  return V(1.60475f * v.x - 0.53108f * v.y - 0.07367f * v.z, -0.10208f * v.x + 1.10813f * v.y - 0.00605f * v.z,
           -0.00327f * v.x - 0.07276f * v.y + 1.07602f * v.z);
}

static v3 display_transform(v3 c, int tone) {
  c = vmaxs(c, 0.0f);
  if (tone == MJPBR_TONE_PBR_NEUTRAL) {
    c = tonemap_pbr_neutral(c);
  } else if (tone == MJPBR_TONE_ACES) {
    c = tonemap_aces(c);
  }
  return vmins(vmaxs(c, 0.0f), 1.0f);
}

static float srgb_oetf(float x) { return x <= 0.0031308f ? 12.92f * x : 1.055f * powf(x, 1.0f / 2.4f) - 0.055f; }

static uint32_t encode_display(v3 c) {
  uint32_t r = (uint32_t)(srgb_oetf(c.x) * 255.0f + 0.5f);
  uint32_t g = (uint32_t)(srgb_oetf(c.y) * 255.0f + 0.5f);
  uint32_t b = (uint32_t)(srgb_oetf(c.z) * 255.0f + 0.5f);
  return (255u << 24) | (b << 16) | (g << 8) | r;
}

/* ------------------------------------------------------------------ surface (material.py) */

static float widen_roughness(float pr, float extra) {
  pr = clampf_(pr, 0.0f, 1.0f);
  float a2 = minf(pr * pr * pr * pr + extra, 1.0f);
  return sqrtf(sqrtf(a2));
}

static v3 vertex_normal(v3 n, v3 face) {
  v3 nn = vnorm(n);
  return vdot(nn, face) < 0.8f ? face : nn;
}

static void primitive_uv(int type, v3 p, v3 ln, v3 size, float rx, float ry, int uniform, float* u, float* v,
                         float* repx, float* repy) {
  const float inv2pi = 0.5f / PI_F;
  *repx = rx;
  *repy = ry;
  if (type == MJPBR_GEOM_PLANE || type == MJPBR_GEOM_HFIELD) { /* height fields map like planes */
    float sx = size.x > 0.0f ? size.x : 1.0f, sy = size.y > 0.0f ? size.y : 1.0f;
    if (uniform) {
      *u = p.x;
      *v = -p.y;
    } else {
      *u = p.x / (2.0f * sx) + 0.5f;
      *v = 0.5f - p.y / (2.0f * sy);
    }
  } else if (type == MJPBR_GEOM_SPHERE || type == MJPBR_GEOM_ELLIPSOID) {
    v3 q = type == MJPBR_GEOM_SPHERE ? vdiv(p, size.x) : V(p.x / size.x, p.y / size.y, p.z / size.z);
    *u = atan2f(q.y, q.x) * inv2pi + 0.5f;
    *v = acosf(clampf_(q.z / maxf(vlen(q), 1.0e-9f), -1.0f, 1.0f)) * (1.0f / PI_F);
    if (uniform) {
      *repx = rx * 2.0f * PI_F * size.x;
      *repy = ry * PI_F * size.x;
    }
  } else if (type == MJPBR_GEOM_CYLINDER || type == MJPBR_GEOM_CAPSULE) {
    float h = size.y + (type == MJPBR_GEOM_CAPSULE ? size.x : 0.0f);
    *u = atan2f(p.y, p.x) * inv2pi + 0.5f;
    *v = 0.5f - p.z / (2.0f * maxf(h, 1.0e-9f));
    if (uniform) {
      *repx = rx * 2.0f * PI_F * size.x;
      *repy = ry * 2.0f * h;
    }
  } else {
    float ax = fabsf(ln.x), ay = fabsf(ln.y), az = fabsf(ln.z);
    float a, b, sa, sb;
    if (az >= ax && az >= ay) {
      a = p.x;
      b = -p.y * (ln.z >= 0.0f ? 1.0f : -1.0f);
      sa = size.x;
      sb = size.y;
    } else if (ax >= ay) {
      a = p.y * (ln.x >= 0.0f ? 1.0f : -1.0f);
      b = -p.z;
      sa = size.y;
      sb = size.z;
    } else {
      a = -p.x * (ln.y >= 0.0f ? 1.0f : -1.0f);
      b = -p.z;
      sa = size.x;
      sb = size.z;
    }
    if (uniform) {
      *u = a;
      *v = b;
    } else {
      *u = a / (2.0f * maxf(sa, 1.0e-9f)) + 0.5f;
      *v = b / (2.0f * maxf(sb, 1.0e-9f)) + 0.5f;
    }
  }
}

typedef struct {
  int has_uv;
  float u, v;
  v3 tangent, bitangent;
  float uv_per_length;
} texframe_t;

static void fetch_role(const MjpbrScene* s, int tex, const texframe_t* f, float cone, float* out) {
  const MjpbrTexture* t = &s->textures[tex];
  float texels = cone * f->uv_per_length * (float)(t->width > t->height ? t->width : t->height);
  float lod = log2f(maxf(texels, 1.0e-8f));
  sample_trilinear(t, s->tex_data, f->u, f->v, maxf(lod, 0.0f), 1, 1, out);
}

static surface_t eval_surface(const world_t* W, const hit_t* hit, v3 point, v3 dir, float footprint, v3* shading_world) {
  const MjpbrScene* s = W->s;
  const MjpbrSettings* st = &s->settings;
  int w = W->w, g = hit->geom;
  surface_t sf;
  sf.occlusion = 1.0f;
  sf.emissive = V(0, 0, 0);
  float rgba[4];
  int matid;
  geom_rgba(s, w, g, rgba, &matid);
  sf.base_color = V(rgba[0], rgba[1], rgba[2]);
  sf.alpha = rgba[3];
  sf.metallic = bf(s->geom_metallic, w, s->ngeom, g);
  sf.roughness = bf(s->geom_roughness, w, s->ngeom, g);
  sf.reflectance = bf(s->geom_reflectance, w, s->ngeom, g);
  float emission = (matid >= 0 && s->mat_emission.ptr) ? bf(s->mat_emission, w, s->nmat, matid) : 0.0f;
  frame_t fr;
  geom_frame(W, g, &fr);
  int type = s->geom_type[g];
  v3 local_dir = mat_mul_t(fr.mat, dir);
  v3 local_normal = mat_mul_t(fr.mat, hit->normal);
  if (vdot(local_normal, local_dir) > 0.0f) local_normal = vneg(local_normal);
  v3 shading = local_normal;
  float curvature = 0.0f;
  int is_mesh = type == MJPBR_GEOM_MESH || type == MJPBR_GEOM_SDF;
  int spec_aa = st->specular_aa;
  if (is_mesh && hit->mesh >= 0 && hit->face >= 0 && st->vertex_normals && s->mesh_facenormal) {
    int fadr = s->mesh_faceadr[hit->mesh] + hit->face;
    const int32_t* tri = s->mesh_facenormal + (int64_t)fadr * 3;
    int nadr = s->mesh_normaladr[hit->mesh];
    v3 nv[3];
    for (int k = 0; k < 3; ++k) {
      const float* q = s->mesh_normal + (int64_t)(nadr + tri[k]) * 3;
      nv[k] = vertex_normal(V(q[0], q[1], q[2]), local_normal);
    }
    shading = vnorm(vadd(vadd(vmul(nv[0], hit->u), vmul(nv[1], hit->v)), vmul(nv[2], 1.0f - hit->u - hit->v)));
    if (vdot(shading, local_dir) > 0.0f) shading = vneg(shading);
    if (spec_aa) {
      const int32_t* fv = s->mesh_face + (int64_t)fadr * 3;
      int vadr = s->mesh_vertadr[hit->mesh];
      const float* q0 = s->mesh_vert + (int64_t)(vadr + fv[0]) * 3;
      const float* q1 = s->mesh_vert + (int64_t)(vadr + fv[1]) * 3;
      const float* q2 = s->mesh_vert + (int64_t)(vadr + fv[2]) * 3;
      v3 p0 = V(q0[0], q0[1], q0[2]);
      float edge = sqrtf(vlen(vcross(vsub(V(q1[0], q1[1], q1[2]), p0), vsub(V(q2[0], q2[1], q2[2]), p0))));
      float spread = maxf(vlen(vsub(nv[0], nv[1])), maxf(vlen(vsub(nv[1], nv[2])), vlen(vsub(nv[2], nv[0]))));
      curvature = spread / maxf(edge, 1.0e-9f);
    }
  }
  if (spec_aa) {
    if (type == MJPBR_GEOM_SPHERE || type == MJPBR_GEOM_CAPSULE || type == MJPBR_GEOM_CYLINDER) {
      curvature = 1.0f / maxf(fr.size.x, 1.0e-9f);
    } else if (type == MJPBR_GEOM_ELLIPSOID) {
      curvature = 1.0f / maxf(minf(fr.size.x, minf(fr.size.y, fr.size.z)), 1.0e-9f);
    }
  }
  float cone = footprint / maxf(fabsf(vdot(local_normal, local_dir)), 0.05f);
  if (st->textures && matid >= 0) {
    const int32_t* texid = s->mat_texid.ptr + ((int64_t)(w % s->mat_texid.nbatch) * s->nmat + matid) * MJPBR_NTEXROLE;
    const float* rp = s->mat_texrepeat.ptr + ((int64_t)(w % s->mat_texrepeat.nbatch) * s->nmat + matid) * 2;
    int uniform = s->mat_texuniform.ptr ? bi(s->mat_texuniform, w, s->nmat, matid) != 0 : 0;
    texframe_t tf;
    tf.has_uv = 0;
    if (is_mesh) {
      int tc_adr = s->mesh_texcoordadr ? s->mesh_texcoordadr[hit->mesh] : -1;
      if (hit->mesh >= 0 && hit->face >= 0 && tc_adr >= 0 && s->mesh_facetexcoord) {
        int fadr = s->mesh_faceadr[hit->mesh] + hit->face;
        const int32_t* ti = s->mesh_facetexcoord + (int64_t)fadr * 3;
        if (ti[0] >= 0 && ti[1] >= 0 && ti[2] >= 0) {
          const float* tc = s->mesh_texcoord + (int64_t)tc_adr * 2;
          float u0 = tc[ti[0] * 2] * rp[0], v0 = tc[ti[0] * 2 + 1] * rp[1];
          float u1 = tc[ti[1] * 2] * rp[0], v1 = tc[ti[1] * 2 + 1] * rp[1];
          float u2 = tc[ti[2] * 2] * rp[0], v2 = tc[ti[2] * 2 + 1] * rp[1];
          float bw = 1.0f - hit->u - hit->v;
          tf.u = u0 * hit->u + u1 * hit->v + u2 * bw;
          tf.v = v0 * hit->u + v1 * hit->v + v2 * bw;
          int vadr = s->mesh_vertadr[hit->mesh];
          const int32_t* fv = s->mesh_face + (int64_t)fadr * 3;
          const float* q0 = s->mesh_vert + (int64_t)(vadr + fv[0]) * 3;
          const float* q1 = s->mesh_vert + (int64_t)(vadr + fv[1]) * 3;
          const float* q2 = s->mesh_vert + (int64_t)(vadr + fv[2]) * 3;
          v3 p0 = V(q0[0], q0[1], q0[2]);
          v3 e1 = vsub(V(q1[0], q1[1], q1[2]), p0), e2 = vsub(V(q2[0], q2[1], q2[2]), p0);
          float d1u = u1 - u0, d1v = v1 - v0, d2u = u2 - u0, d2v = v2 - v0;
          float det = d1u * d2v - d2u * d1v;
          float inv = 1.0f / (fabsf(det) > 1.0e-20f ? det : 1.0e-20f);
          tf.tangent = vmul(vsub(vmul(e1, d2v), vmul(e2, d1v)), inv);
          tf.bitangent = vmul(vsub(vmul(e2, d1u), vmul(e1, d2u)), inv);
          float area = vlen(vcross(e1, e2));
          tf.uv_per_length = sqrtf(fabsf(det) / maxf(area, 1.0e-20f));
          tf.has_uv = 1;
        }
      }
    } else {
      v3 local = mat_mul_t(fr.mat, vsub(point, fr.pos));
      v3 t1, t2;
      orthonormal_basis(local_normal, &t1, &t2);
      float eps = 1.0e-3f * maxf(maxf(fr.size.x, fr.size.y), maxf(fr.size.z, 1.0e-3f));
      float u0, v0, u1, v1, u2, v2, repx, repy, r1, r2;
      primitive_uv(type, local, local_normal, fr.size, rp[0], rp[1], uniform, &u0, &v0, &repx, &repy);
      primitive_uv(type, vadd(local, vmul(t1, eps)), local_normal, fr.size, rp[0], rp[1], uniform, &u1, &v1, &r1, &r2);
      primitive_uv(type, vadd(local, vmul(t2, eps)), local_normal, fr.size, rp[0], rp[1], uniform, &u2, &v2, &r1, &r2);
      float d1u = (u1 - u0 - rintf(u1 - u0)) * repx, d1v = (v1 - v0 - rintf(v1 - v0)) * repy;
      float d2u = (u2 - u0 - rintf(u2 - u0)) * repx, d2v = (v2 - v0 - rintf(v2 - v0)) * repy;
      float inv_eps = 1.0f / eps;
      float du1 = d1u * inv_eps, du2 = d2u * inv_eps, dv1 = d1v * inv_eps, dv2 = d2v * inv_eps;
      float det = du1 * dv2 - du2 * dv1;
      float inv = 1.0f / (fabsf(det) > 1.0e-20f ? det : 1.0e-20f);
      tf.tangent = vmul(vsub(vmul(t1, dv2), vmul(t2, dv1)), inv);
      tf.bitangent = vmul(vsub(vmul(t2, du1), vmul(t1, du2)), inv);
      tf.uv_per_length = sqrtf(fabsf(det));
      tf.u = u0 * repx;
      tf.v = v0 * repy;
      tf.has_uv = 1;
    }
    if (tf.has_uv) {
      float t[4];
      if (st->base_color_map) {
        int tid = texid[MJPBR_ROLE_RGB] >= 0 ? texid[MJPBR_ROLE_RGB] : texid[MJPBR_ROLE_RGBA];
        if (tid >= 0) {
          fetch_role(s, tid, &tf, cone, t);
          sf.base_color = vcmul(sf.base_color, V(t[0], t[1], t[2]));
          sf.alpha *= t[3];
        }
      }
      if (st->orm_map) {
        int tid = texid[MJPBR_ROLE_ORM];
        if (tid >= 0) {
          fetch_role(s, tid, &tf, cone, t);
          sf.occlusion = t[0];
          sf.roughness *= t[1];
          sf.metallic *= t[2];
        } else {
          tid = texid[MJPBR_ROLE_OCCLUSION];
          if (tid >= 0) {
            fetch_role(s, tid, &tf, cone, t);
            sf.occlusion = t[0];
          }
          tid = texid[MJPBR_ROLE_ROUGHNESS];
          if (tid >= 0) {
            fetch_role(s, tid, &tf, cone, t);
            sf.roughness *= t[0];
          }
          tid = texid[MJPBR_ROLE_METALLIC];
          if (tid >= 0) {
            fetch_role(s, tid, &tf, cone, t);
            sf.metallic *= t[0];
          }
        }
      }
      if (st->opacity_map) {
        int tid = texid[MJPBR_ROLE_OPACITY];
        if (tid >= 0) {
          fetch_role(s, tid, &tf, cone, t);
          sf.alpha *= t[0];
        }
      }
      if (st->emissive_map) {
        int tid = texid[MJPBR_ROLE_EMISSIVE];
        if (tid >= 0) {
          fetch_role(s, tid, &tf, cone, t);
          sf.emissive = vmul(V(t[0], t[1], t[2]), emission);
          emission = 0.0f;
        }
      }
      if (st->normal_map) {
        int tid = texid[MJPBR_ROLE_NORMAL];
        if (tid >= 0) {
          fetch_role(s, tid, &tf, cone, t);
          v3 nts = vsub(vmul(V(t[0], t[1], t[2]), 2.0f), V(1, 1, 1));
          if (spec_aa) {
            float len = clampf_(vlen(nts), 1.0e-3f, 1.0f);
            sf.roughness = widen_roughness(sf.roughness, (1.0f - len) / len);
          }
          v3 tt = vsub(tf.tangent, vmul(shading, vdot(shading, tf.tangent)));
          if (vdot(tt, tt) > 1.0e-20f) {
            tt = vnorm(tt);
            v3 bb = vcross(shading, tt);
            if (vdot(bb, tf.bitangent) > 0.0f) bb = vneg(bb);
            v3 mapped = vnorm(vadd(vadd(vmul(tt, nts.x), vmul(bb, nts.y)), vmul(shading, nts.z)));
            if (vdot(mapped, local_normal) > 0.0f) shading = mapped;
          }
        }
      }
    }
  }
  if (matid >= 0 && emission > 0.0f) sf.emissive = vmul(sf.base_color, emission);
  if (spec_aa) {
    float dn = cone * curvature;
    float kernel = minf(2.0f * 0.15f * dn * dn, 0.2f);
    sf.roughness = widen_roughness(sf.roughness, kernel);
  }
  *shading_world = vnorm(mat_mul(fr.mat, shading));
  return sf;
}

/* ------------------------------------------------------------------ real-time shading (render.py) */

typedef struct {
  world_t W;
  float exposure;
  v3 ambient;
  int env;
  float env_yaw, env_scale;
} ctx_t;

static float light_visibility(const ctx_t* c, const light_t* light, v3 point, v3 normal, v3 l, float dist, uint32_t seed,
                              int stream, int nlight, int li) {
  const MjpbrSettings* st = &c->W.s->settings;
  int cull = st->cull_backfaces;
  v3 origin = vadd(point, vmul(normal, RAY_OFFSET));
  if (light->type == MJPBR_LIGHT_DIRECTIONAL) {
    return occluded(&c->W, origin, l, UNBOUNDED, cull) ? st->shadow_light_fraction : 1.0f;
  }
  if (st->shadow_samples <= 1) {
    return occluded(&c->W, origin, l, dist - SHADOW_GAP, cull) ? st->shadow_light_fraction : 1.0f;
  }
  v3 t1, t2;
  orthonormal_basis(l, &t1, &t2);
  float visible = 0.0f;
  int ns = st->shadow_samples;
  for (int k = 0; k < ns; ++k) {
    uint32_t counter = (uint32_t)(((stream * nlight + li) * ns + k) * 2);
    float u0 = rand01(seed, counter), u1 = rand01(seed, counter + 1u);
    float r = light->bulbradius * sqrtf(u0);
    float sn, cs;
    sincos_turns(u1, &sn, &cs);
    v3 to = vsub(vadd(light->pos, vmul(vadd(vmul(t1, cs), vmul(t2, sn)), r)), origin);
    float d = vlen(to);
    if (!occluded(&c->W, origin, vdiv(to, d), d - SHADOW_GAP, cull)) visible += 1.0f;
  }
  float v = visible / (float)ns;
  return v + (1.0f - v) * st->shadow_light_fraction;
}

static v3 shade_light(const ctx_t* c, const light_t* light, const lobes_t* lb, v3 point, v3 normal, v3 view, float nov,
                      uint32_t seed, int stream, int nlight, int li) {
  const MjpbrSettings* st = &c->W.s->settings;
  v3 l, ds, ss;
  float dist;
  eval_light(light, st->light_model, point, &l, &dist, &ds, &ss);
  float nol = vdot(normal, l);
  if (nol <= 0.0f || (vdot(ds, ds) == 0.0f && vdot(ss, ss) == 0.0f)) return V(0, 0, 0);
  float vis = 1.0f;
  if (st->use_shadows && light->castshadow) vis = light_visibility(c, light, point, normal, l, dist, seed, stream, nlight, li);
  v3 h = vnorm(vadd(l, view));
  float noh = maxf(vdot(normal, h), 0.0f), loh = maxf(vdot(l, h), 0.0f);
  v3 fr = vcmul(vmul(f_schlick(lb->f0, 1.0f, loh), d_ggx(noh, lb->alpha) * v_smith(nov, nol, lb->alpha)), lb->energy_comp);
  v3 fd = vmul(lb->diffuse_color, 1.0f / PI_F);
  return vmul(vadd(vcmul(fd, ds), vcmul(fr, ss)), nol * vis);
}

static v3 shade_surface(const ctx_t* c, const surface_t* sf, v3 point, v3 normal, v3 view, v3 head_dir, uint32_t seed,
                        int stream) {
  const MjpbrScene* s = c->W.s;
  const MjpbrSettings* st = &s->settings;
  float nov = maxf(vdot(normal, view), 1.0e-4f);
  lobes_t lb = shading_lobes(s, sf, nov);
  v3 irradiance = c->ambient, prefiltered = c->ambient;
  if (st->has_env) {
    irradiance = vadd(c->ambient, vmul(eval_sh9(s->env_sh + c->env * 27, rotate_yaw(normal, -c->env_yaw)), c->env_scale));
    v3 r = vsub(view, vmul(normal, 2.0f * vdot(view, normal)));
    float a2 = lb.alpha * lb.alpha;
    v3 dominant = vnorm(vadd(vmul(vneg(r), 1.0f - a2), vmul(normal, a2)));
    v3 blurred = sample_prefiltered(s, c->env, dominant, c->env_yaw, lb.pr);
    float t = lb.pr * ((float)s->prefilter_levels - 1.0f);
    v3 spec = blurred;
    if (t < 1.0f) {
      v3 sharp = sample_radiance(s, c->env, dominant, c->env_yaw, 0.0f);
      spec = vadd(vmul(sharp, 1.0f - t), vmul(blurred, t));
    }
    prefiltered = vadd(c->ambient, vmul(spec, c->env_scale));
  }
  float ao = sf->occlusion;
  float spec_ao = clampf_(powf(nov + ao, powf(2.0f, -16.0f * lb.alpha - 1.0f)) - 1.0f + ao, 0.0f, 1.0f);
  v3 radiance = vadd(vmul(vcmul(irradiance, lb.diffuse_color), ao), vmul(vcmul(prefiltered, vcmul(lb.spec_albedo, lb.energy_comp)), spec_ao));
  for (int li = 0; li < s->nlight; ++li) {
    light_t light = fetch_light(s, c->W.w, li);
    if (!light.active) continue;
    radiance = vadd(radiance, shade_light(c, &light, &lb, point, normal, view, nov, seed, stream, s->nlight, li));
  }
  if (st->headlight_active) {
    light_t head;
    memset(&head, 0, sizeof(head));
    head.type = MJPBR_LIGHT_DIRECTIONAL;
    head.active = 1;
    head.dir = head_dir;
    head.diffuse = V(st->headlight_diffuse[0], st->headlight_diffuse[1], st->headlight_diffuse[2]);
    head.specular = V(st->headlight_specular[0], st->headlight_specular[1], st->headlight_specular[2]);
    head.attenuation = V(1, 0, 0);
    head.intensity = st->headlight_intensity / c->exposure;
    head.range = 1.0f;
    radiance = vadd(radiance, shade_light(c, &head, &lb, point, normal, view, nov, seed, stream, 1, 0));
  }
  return vadd(radiance, vdiv(sf->emissive, c->exposure));
}

static v3 background(const ctx_t* c, v3 d, float spread) {
  const MjpbrScene* s = c->W.s;
  if (s->settings.env_background) {
    float lod = log2f(maxf(spread * s->settings.inv_texel_angle, 1.0e-8f));
    return vmul(sample_radiance(s, c->env, d, c->env_yaw, lod), c->env_scale);
  }
  return vdiv(V(s->settings.background[0], s->settings.background[1], s->settings.background[2]), c->exposure);
}

static float mirror_reflectance(const ctx_t* c, int g) {
  const MjpbrScene* s = c->W.s;
  int matid = bi(s->geom_matid, c->W.w, s->ngeom, g);
  if (matid < 0 || !s->mat_reflectance.ptr) return 0.0f;
  return bf(s->mat_reflectance, c->W.w, s->nmat, matid);
}

static v3 shade_reflection(const ctx_t* c, v3 point, v3 normal, v3 dir, float footprint, float spread, v3 head_dir,
                           uint32_t seed, int stream) {
  const MjpbrScene* s = c->W.s;
  v3 r = vsub(dir, vmul(normal, 2.0f * vdot(dir, normal)));
  v3 origin = vadd(point, vmul(normal, RAY_OFFSET));
  hit_t hit = closest(&c->W, origin, r, MAXVAL, s->settings.cull_backfaces);
  if (hit.geom == -1) return background(c, r, spread);
  v3 p = vadd(origin, vmul(r, hit.dist));
  v3 n;
  surface_t sf = eval_surface(&c->W, &hit, p, r, footprint + spread * hit.dist, &n);
  return shade_surface(c, &sf, p, n, vneg(r), head_dir, seed, stream);
}

static v3 trace_pixel(const ctx_t* c, v3 origin, v3 dir, float max_dist, float footprint, float spread, v3 head_dir,
                      uint32_t seed, int stream, hit_t* first, v3* albedo, v3* gnormal) {
  const MjpbrScene* s = c->W.s;
  const MjpbrSettings* st = &s->settings;
  v3 radiance = V(0, 0, 0);
  float throughput = 1.0f, travelled = 0.0f;
  int nlayer = st->has_transparency ? st->max_layers : 1;
  for (int layer = 0; layer < nlayer; ++layer) {
    hit_t hit = closest(&c->W, origin, dir, max_dist - travelled, st->cull_backfaces);
    if (layer == 0) *first = hit;
    if (hit.geom == -1) {
      radiance = vadd(radiance, vmul(background(c, dir, spread), throughput));
      break;
    }
    v3 point = vadd(origin, vmul(dir, hit.dist));
    float cone = footprint + spread * (travelled + hit.dist);
    v3 normal;
    surface_t sf = eval_surface(&c->W, &hit, point, dir, cone, &normal);
    if (layer == 0) {
      *albedo = sf.base_color;
      *gnormal = normal;
    }
    v3 shaded = shade_surface(c, &sf, point, normal, vneg(dir), head_dir, seed, stream);
    if (st->has_reflection) {
      float mirror = mirror_reflectance(c, hit.geom);
      if (mirror > 0.0f) {
        v3 refl = shade_reflection(c, point, normal, dir, cone, spread, head_dir, seed, stream + 1);
        shaded = vadd(vmul(shaded, 1.0f - mirror), vmul(refl, mirror));
      }
    }
    if (st->has_transparency) {
      float opacity = clampf_(sf.alpha, 0.0f, 1.0f);
      radiance = vadd(radiance, vmul(shaded, throughput * opacity));
      throughput *= 1.0f - opacity;
      if (throughput < 1.0f / 255.0f) break;
      travelled += hit.dist;
      origin = vadd(point, vmul(dir, RAY_OFFSET));
    } else {
      radiance = vadd(radiance, shaded);
      break;
    }
  }
  return radiance;
}

/* Camera record derived from the model/data arrays (the library's refit writes the same values). */
typedef struct {
  v3 pos;
  const float* mat;
  int proj;
  float half_h;
  int use_intr;
  float intr[4], sensor[2];
} cam_t;

static cam_t camera(const MjpbrScene* s, int w, int c) {
  cam_t cam;
  int id = s->cam_id_map[c];
  const float* xp = s->cam_xpos + ((int64_t)w * s->ncam + id) * 3;
  cam.pos = V(xp[0], xp[1], xp[2]);
  cam.mat = s->cam_xmat + ((int64_t)w * s->ncam + id) * 9;
  cam.proj = s->cam_projection[id];
  float fovy = bf(s->cam_fovy, w, s->ncam, id);
  if (cam.proj == MJPBR_PROJ_ORTHOGRAPHIC) {
    cam.half_h = fovy * 0.5f;
  } else {
    float sn, cs;
    sincos_turns(fovy / 720.0f, &sn, &cs);
    cam.half_h = sn / cs;
  }
  cam.use_intr = s->cam_sensorsize && s->cam_sensorsize[id * 2] > 0.0f && cam.proj == MJPBR_PROJ_PERSPECTIVE;
  for (int k = 0; k < 4; ++k) cam.intr[k] = cam.use_intr && s->cam_intrinsic.ptr ? bf(s->cam_intrinsic, w, s->ncam * 4, id * 4 + k) : 0.0f;
  cam.sensor[0] = s->cam_sensorsize ? s->cam_sensorsize[id * 2] : 0.0f;
  cam.sensor[1] = s->cam_sensorsize ? s->cam_sensorsize[id * 2 + 1] : 0.0f;
  return cam;
}

static void camera_frame_ray(const cam_t* cam, int W, int H, int px, int py, int n, int sx, int sy, v3* dcam, v3* ocam) {
  int ix = px * n + sx, iy = py * n + sy;
  float u = ((float)ix + 0.5f) / (float)(W * n);
  float v = ((float)iy + 0.5f) / (float)(H * n);
  float aspect = (float)W / (float)H;
  if (cam->proj == MJPBR_PROJ_ORTHOGRAPHIC) {
    *dcam = V(0.0f, 0.0f, -1.0f);
    *ocam = V((2.0f * u - 1.0f) * (cam->half_h * aspect), (1.0f - 2.0f * v) * cam->half_h, 0.0f);
    return;
  }
  float x, y;
  if (cam->use_intr) {
    x = (u * cam->sensor[0] - 0.5f * cam->sensor[0] - cam->intr[2]) / cam->intr[0];
    y = (0.5f * cam->sensor[1] - v * cam->sensor[1] + cam->intr[3]) / cam->intr[1];
  } else {
    x = (2.0f * u - 1.0f) * (cam->half_h * aspect);
    y = (1.0f - 2.0f * v) * cam->half_h;
  }
  float len = sqrtf(x * x + y * y + 1.0f);
  *dcam = V(x / len, y / len, -1.0f / len);
  *ocam = V(0, 0, 0);
}

/* Per-pixel ray bundles (camera.py:195-330, rays.py): bilinear interpolation of the four nearest
 * bundle rays, on the image plane z = -1 when all point forward, else on the sphere. */
static void bundle_axis(int i, int n, int nb, int* x0, int* x1, float* t) {
  int64_t num = (int64_t)(2 * i + 1) * nb - n, den = 2 * (int64_t)n;
  int a = (int)((num + den) / den) - 1;
  int hi = nb - 2 > 0 ? nb - 2 : 0;
  a = a < 0 ? 0 : (a > hi ? hi : a);
  *x0 = a;
  *x1 = a + 1 < nb - 1 ? a + 1 : nb - 1;
  *t = (float)(num - (int64_t)a * den) / (float)den;
}

static v3 rvec(const float* a, int64_t i) { return V(a[i * 3], a[i * 3 + 1], a[i * 3 + 2]); }
static v3 vlerp(v3 a, v3 b, float t) { return vadd(a, vmul(vsub(b, a), t)); }

static void bundle_ray(const MjpbrScene* s, int c, int W, int H, int px, int py, int n, int sx, int sy, v3* dcam, v3* ocam) {
  int rw = s->bundle_res[c][0], rh = s->bundle_res[c][1];
  int64_t adr = s->ray_adr[c];
  int x0, x1, y0, y1;
  float tx, ty;
  bundle_axis(px * n + sx, W * n, rw, &x0, &x1, &tx);
  bundle_axis(py * n + sy, H * n, rh, &y0, &y1, &ty);
  int64_t r0 = adr + (int64_t)y0 * rw, r1 = adr + (int64_t)y1 * rw;
  v3 d00 = rvec(s->ray_direction, r0 + x0), d10 = rvec(s->ray_direction, r0 + x1);
  v3 d01 = rvec(s->ray_direction, r1 + x0), d11 = rvec(s->ray_direction, r1 + x1);
  if (vdot(d00, d00) == 0.0f || vdot(d10, d10) == 0.0f || vdot(d01, d01) == 0.0f || vdot(d11, d11) == 0.0f) {
    int64_t nearest = (ty < 0.5f ? r0 : r1) + (tx < 0.5f ? x0 : x1);
    v3 d = rvec(s->ray_direction, nearest);
    if (vdot(d, d) > 0.0f) d = vnorm(d);
    *dcam = d;
    *ocam = rvec(s->ray_origin, nearest);
    return;
  }
  v3 o00 = rvec(s->ray_origin, r0 + x0), o10 = rvec(s->ray_origin, r0 + x1);
  v3 o01 = rvec(s->ray_origin, r1 + x0), o11 = rvec(s->ray_origin, r1 + x1);
  if (d00.z < 0.0f && d10.z < 0.0f && d01.z < 0.0f && d11.z < 0.0f) {
    d00 = vmul(d00, -1.0f / d00.z);
    d10 = vmul(d10, -1.0f / d10.z);
    d01 = vmul(d01, -1.0f / d01.z);
    d11 = vmul(d11, -1.0f / d11.z);
  }
  v3 d = vlerp(vlerp(d00, d10, tx), vlerp(d01, d11, tx), ty);
  if (vdot(d, d) > 0.0f) d = vnorm(d);
  *dcam = d;
  *ocam = vlerp(vlerp(o00, o10, tx), vlerp(o01, o11, tx), ty);
}

static void bundle_step(const MjpbrScene* s, int64_t a, int64_t b, int extrapolate, float* spread, float* width) {
  v3 da = rvec(s->ray_direction, a), db = rvec(s->ray_direction, b);
  *spread = 0.0f;
  *width = 0.0f;
  if (vdot(da, da) == 0.0f || vdot(db, db) == 0.0f) return;
  da = vnorm(da);
  db = vnorm(db);
  *width = vlen(vsub(rvec(s->ray_origin, b), rvec(s->ray_origin, a)));
  if (!extrapolate)
    *spread = vlen(vsub(db, da));
  else if (da.z < 0.0f && db.z < 0.0f)
    *spread = vlen(vsub(vnorm(vadd(vmul(db, -2.0f / db.z), vmul(da, 1.0f / da.z))), db));
  else
    *spread = vlen(vsub(vnorm(vsub(vmul(db, 2.0f), da)), db));
}

/* Camera-frame ray of sub-pixel cell (sx, sy) of n x n, its maximum distance and depth axis z. */
static void primary_ray(const MjpbrScene* s, const cam_t* cam, int c, int W, int H, int px, int py, int n, int sx, int sy,
                        v3* dcam, v3* ocam, float* max_dist, float* depth_z) {
  float zfar = s->settings.zfar;
  if (s->ray_direction) {
    bundle_ray(s, c, W, H, px, py, n, sx, sy, dcam, ocam);
    *max_dist = zfar > 0.0f ? zfar : MAXVAL;
    if (vdot(*dcam, *dcam) == 0.0f) {
      *max_dist = 0.0f;
      *dcam = V(0.0f, 0.0f, -1.0f);
    }
    *depth_z = -1.0f;
    return;
  }
  camera_frame_ray(cam, W, H, px, py, n, sx, sy, dcam, ocam);
  *max_dist = zfar > 0.0f ? zfar / maxf(-dcam->z, 1.0e-6f) : MAXVAL;
  *depth_z = dcam->z;
}

static void pixel_cone(const MjpbrScene* s, const cam_t* cam, int c, int W, int H, int px, int py, float* spread, float* width) {
  if (s->ray_direction) {
    int rw = s->bundle_res[c][0], rh = s->bundle_res[c][1];
    *spread = 0.0f;
    *width = 0.0f;
    if (rw < 2) return;
    int bx = (px * rw) / W;
    int64_t b = s->ray_adr[c] + (int64_t)((py * rh) / H) * rw + bx;
    if (bx + 1 < rw)
      bundle_step(s, b, b + 1, 0, spread, width);
    else
      bundle_step(s, b - 1, b, 1, spread, width);
    float scale = (float)rw / (float)W;
    *spread *= scale;
    *width *= scale;
    return;
  }
  v3 d0, o0, d1, o1;
  camera_frame_ray(cam, W, H, px, py, 1, 0, 0, &d0, &o0);
  camera_frame_ray(cam, W, H, px, py, 1, 1, 0, &d1, &o1);
  *spread = vlen(vsub(d1, d0));
  *width = vlen(vsub(o1, o0));
}

static void write_geometry(const MjpbrScene* s, int w, int c, int pixelid, const hit_t* hit, float dcam_z) {
  if (s->render_seg[c]) {
    int32_t* o = s->seg_data + ((int64_t)w * s->seg_stride + s->seg_adr[c] + pixelid) * 2;
    o[0] = hit->geom != -1 ? hit->geom : -1;
    o[1] = hit->geom != -1 ? 5 : -1;
  }
  if (s->render_depth[c]) {
    s->depth_data[(int64_t)w * s->depth_stride + s->depth_adr[c] + pixelid] = hit->geom != -1 ? hit->dist * -dcam_z : 0.0f;
  }
}

static void render_pixel(const MjpbrScene* s, const int32_t* mesh_nface, int w, int c, int px, int py, uint32_t seed) {
  const MjpbrSettings* st = &s->settings;
  int W = s->cam_res[c][0], H = s->cam_res[c][1];
  int pixelid = py * W + px;
  cam_t cam = camera(s, w, c);
  ctx_t ctx;
  ctx.W.s = s;
  ctx.W.mesh_nface = mesh_nface;
  ctx.W.w = w;
  ctx.exposure = bf(s->exposure, w, 1, 0);
  ctx.ambient = bv3(s->ambient_radiance, w, 1, 0);
  ctx.env = 0;
  ctx.env_yaw = 0.0f;
  ctx.env_scale = 0.0f;
  if (s->nenv > 0 && s->env_id.ptr) {
    ctx.env = bi(s->env_id, w, 1, 0);
    ctx.env_yaw = bf(s->env_yaw, w, 1, 0);
    ctx.env_scale = bf(s->env_intensity, w, 1, 0);
  }
  int cull = st->cull_backfaces;
  if (!s->render_rgb[c]) {
    v3 dcam, ocam;
    float max_dist, depth_z;
    primary_ray(s, &cam, c, W, H, px, py, 1, 0, 0, &dcam, &ocam, &max_dist, &depth_z);
    hit_t hit = closest(&ctx.W, vadd(cam.pos, mat_mul(cam.mat, ocam)), mat_mul(cam.mat, dcam), max_dist, cull);
    write_geometry(s, w, c, pixelid, &hit, depth_z);
    return;
  }
  int n = st->samples_per_axis;
  float inv_n = 1.0f / (float)n;
  float spread, width;
  pixel_cone(s, &cam, c, W, H, px, py, &spread, &width);
  spread *= inv_n;
  width *= inv_n;
  v3 head_dir = vneg(V(cam.mat[2], cam.mat[5], cam.mat[8]));
  uint32_t pixel_seed = seed + (uint32_t)w * (uint32_t)s->total_rays + (uint32_t)(s->ray_adr[c] + pixelid);
  v3 display = V(0, 0, 0), hdr = V(0, 0, 0);
  for (int smp = 0; smp < n * n; ++smp) {
    v3 dcam, ocam;
    float max_dist, depth_z;
    primary_ray(s, &cam, c, W, H, px, py, n, smp % n, smp / n, &dcam, &ocam, &max_dist, &depth_z);
    v3 origin = vadd(cam.pos, mat_mul(cam.mat, ocam));
    v3 dir = mat_mul(cam.mat, dcam);
    hit_t first;
    v3 albedo = V(0, 0, 0), gnormal = V(0, 0, 0);
    v3 radiance = trace_pixel(&ctx, origin, dir, max_dist, width, spread, head_dir, pixel_seed, 2 * smp, &first, &albedo, &gnormal);
    if (smp == 0) {
      write_geometry(s, w, c, pixelid, &first, depth_z);
      if (st->render_guides && s->guide_albedo) {
        int64_t a = ((int64_t)w * s->rgb_stride + s->rgb_adr[c] + pixelid) * 3;
        v3 al = first.geom != -1 ? albedo : V(0, 0, 0), nm = first.geom != -1 ? gnormal : V(0, 0, 0);
        s->guide_albedo[a] = al.x;
        s->guide_albedo[a + 1] = al.y;
        s->guide_albedo[a + 2] = al.z;
        s->guide_normal[a] = nm.x;
        s->guide_normal[a + 1] = nm.y;
        s->guide_normal[a + 2] = nm.z;
      }
    }
    display = vadd(display, display_transform(vmul(radiance, ctx.exposure), st->tone_mapper));
    hdr = vadd(hdr, radiance);
  }
  int64_t adr = (int64_t)w * s->rgb_stride + s->rgb_adr[c] + pixelid;
  float inv_nn = inv_n * inv_n;
  if (st->render_hdr && s->hdr_data) {
    s->hdr_data[adr * 3] = hdr.x * inv_nn;
    s->hdr_data[adr * 3 + 1] = hdr.y * inv_nn;
    s->hdr_data[adr * 3 + 2] = hdr.z * inv_nn;
  }
  s->rgb_data[adr] = encode_display(vmul(display, inv_nn));
}

/* ------------------------------------------------------------------ path-traced tier (pathtrace.py) */

/* Random-number layout of pathtrace.py:64-95: path vertex (sample, depth) owns PT_SLOTS counters,
 * depth row PT_JITTER holds the sub-pixel jitter, lights past the fourth use a separate range. */
#define PT_SLOTS 16
#define PT_DEPTHS 64
#define PT_JITTER (PT_DEPTHS - 1)
#define PT_SUBPIXEL 15
#define PT_EXTRA_LIGHTS (1u << 30)

static float pt_rand(uint32_t seed, int sample, int depth, int slot) {
  return rand01(seed, (uint32_t)((sample * PT_DEPTHS + depth) * PT_SLOTS + slot));
}

static void pt_light_rand2(uint32_t seed, int sample, int depth, int nlight, int li, float* u0, float* u1) {
  if (li < 4) {
    *u0 = pt_rand(seed, sample, depth, 4 + 2 * li);
    *u1 = pt_rand(seed, sample, depth, 5 + 2 * li);
    return;
  }
  uint32_t counter = PT_EXTRA_LIGHTS + (uint32_t)(((sample * PT_DEPTHS + depth) * nlight + li) * 2);
  *u0 = rand01(seed, counter);
  *u1 = rand01(seed, counter + 1u);
}

static float lum709(v3 c) { return c.x * 0.2126f + c.y * 0.7152f + c.z * 0.0722f; }

/* brdf.py:116-191 */
static float smith_g1(float nov, float alpha) {
  float a2 = alpha * alpha;
  return 2.0f * nov / (nov + sqrtf(a2 + (1.0f - a2) * nov * nov));
}

static v3 ggx_vndf(v3 v, float alpha, float u0, float u1) {
  v3 vh = vnorm(V(alpha * v.x, alpha * v.y, v.z));
  float lensq = vh.x * vh.x + vh.y * vh.y;
  v3 t1 = V(1, 0, 0);
  if (lensq > 0.0f) t1 = vdiv(V(-vh.y, vh.x, 0.0f), sqrtf(lensq));
  v3 t2 = vcross(vh, t1);
  float r = sqrtf(u0), sn, cs;
  sincos_turns(u1, &sn, &cs);
  float p1 = r * cs, p2 = r * sn;
  float sw = 0.5f * (1.0f + vh.z);
  p2 = (1.0f - sw) * sqrtf(maxf(1.0f - p1 * p1, 0.0f)) + sw * p2;
  v3 nh = vadd(vadd(vmul(t1, p1), vmul(t2, p2)), vmul(vh, sqrtf(maxf(1.0f - p1 * p1 - p2 * p2, 0.0f))));
  return vnorm(V(alpha * nh.x, alpha * nh.y, maxf(nh.z, 0.0f)));
}

static v3 bsdf_cos(v3 diffuse_color, v3 f0, float alpha, v3 energy_comp, v3 v, v3 l) {
  float nol = l.z, nov = maxf(v.z, 1.0e-4f);
  if (nol <= 0.0f) return V(0, 0, 0);
  v3 h = vnorm(vadd(l, v));
  float noh = maxf(h.z, 0.0f), loh = maxf(vdot(l, h), 0.0f);
  v3 spec = vcmul(vmul(f_schlick(f0, 1.0f, loh), d_ggx(noh, alpha) * v_smith(nov, nol, alpha)), energy_comp);
  return vmul(vadd(vmul(diffuse_color, 1.0f / PI_F), spec), nol);
}

static float bsdf_pdf(float alpha, float p_spec, v3 v, v3 l) {
  if (l.z <= 0.0f) return 0.0f;
  float nov = maxf(v.z, 1.0e-4f);
  v3 h = vnorm(vadd(l, v));
  float pdf_spec = smith_g1(nov, alpha) * d_ggx(maxf(h.z, 0.0f), alpha) / (4.0f * nov);
  return p_spec * pdf_spec + (1.0f - p_spec) * (l.z * (1.0f / PI_F));
}

static float spec_probability(v3 diffuse_color, v3 spec_albedo) {
  float ws = lum709(spec_albedo), wd = lum709(diffuse_color);
  if (wd <= 0.0f) return 1.0f;
  return clampf_(ws / maxf(ws + wd, 1.0e-6f), 0.1f, 0.9f);
}

static v3 bsdf_sample(float alpha, float p_spec, v3 v, float u_lobe, float u0, float u1) {
  if (u_lobe < p_spec) {
    v3 h = ggx_vndf(v, alpha, u0, u1);
    return vsub(vmul(h, 2.0f * vdot(v, h)), v);
  }
  float r = sqrtf(u0), sn, cs;
  sincos_turns(u1, &sn, &cs);
  return V(r * cs, r * sn, sqrtf(maxf(1.0f - u0, 0.0f)));
}

static float power_heuristic(float a, float b) {
  float a2 = a * a;
  return a2 / maxf(a2 + b * b, 1.0e-30f);
}

static int cdf_find(const float* cdf, int n, float u) {
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    int mid = (lo + hi) / 2;
    if (cdf[mid] <= u)
      lo = mid;
    else
      hi = mid;
  }
  return lo;
}

/* envmap.py:446-490: a world direction drawn proportional to luminance x sin(theta), its pdf. */
static v3 env_sample(const MjpbrScene* s, int env, float yaw, float u0, float u1, float* pdf) {
  int h = s->cdf_height, w = s->cdf_width;
  const float* marginal = s->env_marginal + (int64_t)env * (h + 1);
  int r = cdf_find(marginal, h, u0);
  float c0 = marginal[r];
  float dv = (u0 - c0) / maxf(marginal[r + 1] - c0, 1.0e-12f);
  const float* crow = s->env_conditional + ((int64_t)env * h + r) * (w + 1);
  int c = cdf_find(crow, w, u1);
  float k0 = crow[c];
  float du = (u1 - k0) / maxf(crow[c + 1] - k0, 1.0e-12f);
  float uu = ((float)c + clampf_(du, 0.0f, 1.0f)) / (float)w;
  float vv = ((float)r + clampf_(dv, 0.0f, 1.0f)) / (float)h;
  float sp, cp, sth, cth, sy, cy;
  sincos_turns(uu - 0.5f, &sp, &cp);
  sincos_turns(vv * 0.5f, &sth, &cth);
  v3 d = V(sth * cp, sth * sp, cth);
  sincos_turns(yaw * (0.5f / PI_F), &sy, &cy);
  d = V(cy * d.x - sy * d.y, sy * d.x + cy * d.y, d.z);
  *pdf = s->env_prob[((int64_t)env * h + r) * w + c] * (float)(w * h) / (2.0f * PI_F * PI_F * maxf(sth, 1.0e-6f));
  return d;
}

static float env_pdf(const MjpbrScene* s, int env, float yaw, v3 d) {
  int h = s->cdf_height, w = s->cdf_width;
  float u, v, sn, cs;
  direction_to_uv(d, yaw, &u, &v);
  int c = (int)(u * (float)w), r = (int)(v * (float)h);
  if (c > w - 1) c = w - 1;
  if (r > h - 1) r = h - 1;
  sincos_turns(v * 0.5f, &sn, &cs);
  return s->env_prob[((int64_t)env * h + r) * w + c] * (float)(w * h) / (2.0f * PI_F * PI_F * maxf(sn, 1.0e-6f));
}

static v3 pt_environment(const ctx_t* c, v3 d) { return vmul(sample_radiance(c->W.s, c->env, d, c->env_yaw, 0.0f), c->env_scale); }

/* Next-event estimate of one light (pathtrace.py:126-160). */
static v3 pt_light(const ctx_t* c, light_t light, const lobes_t* lb, v3 point, v3 normal, v3 t1, v3 t2, v3 v, float u0,
                   float u1) {
  const MjpbrSettings* st = &c->W.s->settings;
  if (light.type != MJPBR_LIGHT_DIRECTIONAL && light.bulbradius > 0.0f) {
    v3 b1, b2;
    orthonormal_basis(vnorm(vsub(point, light.pos)), &b1, &b2);
    float r = light.bulbradius * sqrtf(u0), sn, cs;
    sincos_turns(u1, &sn, &cs);
    light.pos = vadd(light.pos, vmul(vadd(vmul(b1, cs), vmul(b2, sn)), r));
  }
  v3 l, ds, ss;
  float dist;
  eval_light(&light, st->light_model, point, &l, &dist, &ds, &ss);
  v3 ll = V(vdot(l, t1), vdot(l, t2), vdot(l, normal));
  if (ll.z <= 0.0f || (vdot(ds, ds) == 0.0f && vdot(ss, ss) == 0.0f)) return V(0, 0, 0);
  if (st->use_shadows && light.castshadow) {
    float max_t = light.type == MJPBR_LIGHT_DIRECTIONAL ? UNBOUNDED : dist - SHADOW_GAP;
    if (occluded(&c->W, vadd(point, vmul(normal, RAY_OFFSET)), l, max_t, st->cull_backfaces)) return V(0, 0, 0);
  }
  v3 zero = V(0, 0, 0);
  v3 diffuse = bsdf_cos(lb->diffuse_color, zero, lb->alpha, zero, v, ll);
  v3 specular = bsdf_cos(zero, lb->f0, lb->alpha, lb->energy_comp, v, ll);
  return vadd(vcmul(diffuse, ds), vcmul(specular, ss));
}

typedef struct {
  hit_t hit;
  v3 albedo, normal, emission, base_color;
} primary_t;

/* Radiance of one path and its first surface (pathtrace.py:200-337). */
static v3 trace_path(const ctx_t* c, v3 origin, v3 dir, float max_dist, v3 head_dir, uint32_t seed, int sample,
                     primary_t* first) {
  const MjpbrScene* s = c->W.s;
  const MjpbrSettings* st = &s->settings;
  int cull = st->cull_backfaces;
  v3 radiance = V(0, 0, 0), beta = V(1, 1, 1);
  first->hit.geom = -1;
  first->albedo = V(1, 1, 1);
  first->normal = V(0, 0, 0);
  first->emission = V(0, 0, 0);
  first->base_color = V(0, 0, 0);
  int camera_ray = 1, delta = 1, depth = 0, passes = 0;
  float pdf_prev = 0.0f;
  while (depth <= st->max_depth) {
    hit_t hit = closest(&c->W, origin, dir, max_dist, cull);
    if (camera_ray && passes == 0) first->hit = hit;
    if (hit.geom == -1) {
      if (camera_ray) {
        if (st->env_background) {
          radiance = vadd(radiance, vcmul(beta, pt_environment(c, dir)));
        } else {
          v3 bg = vdiv(V(st->background[0], st->background[1], st->background[2]), c->exposure);
          radiance = vadd(radiance, vcmul(beta, bg));
        }
      } else {
        v3 env_light = c->ambient;
        if (st->has_env) {
          float weight = 1.0f;
          if (!delta) weight = power_heuristic(pdf_prev, env_pdf(s, c->env, c->env_yaw, dir));
          env_light = vadd(env_light, vmul(pt_environment(c, dir), weight));
        }
        radiance = vadd(radiance, vcmul(beta, env_light));
      }
      break;
    }
    v3 point = vadd(origin, vmul(dir, hit.dist));
    v3 normal;
    surface_t sf = eval_surface(&c->W, &hit, point, dir, 0.0f, &normal);
    if (st->has_transparency) {
      if (pt_rand(seed, sample, depth + passes, 0) >= sf.alpha && passes < 4 * st->max_layers) {
        origin = vadd(point, vmul(dir, RAY_OFFSET));
        max_dist = max_dist - hit.dist;
        passes += 1;
        continue;
      }
    }
    radiance = vadd(radiance, vcmul(beta, vdiv(sf.emissive, c->exposure)));
    if (depth == st->max_depth) break;
    max_dist = MAXVAL;
    if (camera_ray) {
      first->albedo = sf.base_color;
      first->normal = normal;
      first->base_color = sf.base_color;
      first->emission = vdiv(sf.emissive, c->exposure);
    }
    camera_ray = 0;
    if (st->has_reflection) {
      if (pt_rand(seed, sample, depth, 1) < mirror_reflectance(c, hit.geom)) {
        dir = vsub(dir, vmul(normal, 2.0f * vdot(dir, normal)));
        origin = vadd(point, vmul(normal, RAY_OFFSET));
        delta = 1;
        depth += 1;
        continue;
      }
    }
    v3 t1, t2;
    orthonormal_basis(normal, &t1, &t2);
    v3 view = vneg(dir);
    v3 v = V(vdot(view, t1), vdot(view, t2), vdot(view, normal));
    float nov = maxf(v.z, 1.0e-4f);
    lobes_t lb = shading_lobes(s, &sf, nov);
    v3 spec_weight = vcmul(lb.spec_albedo, lb.energy_comp);
    float p_spec = spec_probability(lb.diffuse_color, spec_weight);
    if (depth == 0) first->albedo = vadd(lb.diffuse_color, spec_weight);

    v3 direct = V(0, 0, 0);
    for (int li = 0; li < s->nlight; ++li) {
      light_t light = fetch_light(s, c->W.w, li);
      if (!light.active) continue;
      float u0, u1;
      pt_light_rand2(seed, sample, depth, s->nlight, li, &u0, &u1);
      direct = vadd(direct, pt_light(c, light, &lb, point, normal, t1, t2, v, u0, u1));
    }
    if (st->headlight_active) {
      light_t head;
      memset(&head, 0, sizeof(head));
      head.type = MJPBR_LIGHT_DIRECTIONAL;
      head.active = 1;
      head.dir = head_dir;
      head.diffuse = V(st->headlight_diffuse[0], st->headlight_diffuse[1], st->headlight_diffuse[2]);
      head.specular = V(st->headlight_specular[0], st->headlight_specular[1], st->headlight_specular[2]);
      head.attenuation = V(1, 0, 0);
      head.intensity = st->headlight_intensity / c->exposure;
      head.range = 1.0f;
      direct = vadd(direct, pt_light(c, head, &lb, point, normal, t1, t2, v, 0.0f, 0.0f));
    }
    radiance = vadd(radiance, vcmul(beta, direct));

    if (st->has_env) {
      float pdf_env;
      v3 d_env = env_sample(s, c->env, c->env_yaw, pt_rand(seed, sample, depth, 2), pt_rand(seed, sample, depth, 3), &pdf_env);
      v3 le = V(vdot(d_env, t1), vdot(d_env, t2), vdot(d_env, normal));
      if (le.z > 0.0f && pdf_env > 0.0f) {
        v3 f = bsdf_cos(lb.diffuse_color, lb.f0, lb.alpha, lb.energy_comp, v, le);
        if (!occluded(&c->W, vadd(point, vmul(normal, RAY_OFFSET)), d_env, UNBOUNDED, cull)) {
          float weight = power_heuristic(pdf_env, bsdf_pdf(lb.alpha, p_spec, v, le));
          radiance = vadd(radiance, vmul(vcmul(beta, vcmul(f, pt_environment(c, d_env))), weight / pdf_env));
        }
      }
    }

    v3 l = bsdf_sample(lb.alpha, p_spec, v, pt_rand(seed, sample, depth, 12), pt_rand(seed, sample, depth, 13),
                       pt_rand(seed, sample, depth, 14));
    if (l.z <= 0.0f) break;
    float pdf = bsdf_pdf(lb.alpha, p_spec, v, l);
    if (pdf <= 0.0f) break;
    beta = vcmul(beta, vdiv(bsdf_cos(lb.diffuse_color, lb.f0, lb.alpha, lb.energy_comp, v, l), pdf));
    dir = vnorm(vadd(vadd(vmul(t1, l.x), vmul(t2, l.y)), vmul(normal, l.z)));
    origin = vadd(point, vmul(normal, RAY_OFFSET));
    pdf_prev = pdf;
    delta = 0;
    depth += 1;
    if (depth >= st->rr_depth) {
      float q = clampf_(maxf(beta.x, maxf(beta.y, beta.z)), 0.05f, 0.95f);
      if (pt_rand(seed, sample, depth, 15) >= q) break;
      beta = vdiv(beta, q);
    }
  }
  return radiance;
}

static v3 round_half3(v3 a) {
  return V(half_to_float(float_to_half(a.x)), half_to_float(float_to_half(a.y)), half_to_float(float_to_half(a.z)));
}

/* The filter's first-hit guide: normal and albedo as half floats, depth (the GPU packs the same
 * values into four 32-bit words). */
#define MIN_ALBEDO 1.0e-2f

typedef struct {
  v3 normal, albedo;
  float depth;
} guide_t;

static void store_guide(uint32_t* o, const guide_t* g) {
  o[0] = (uint32_t)float_to_half(g->normal.x) | ((uint32_t)float_to_half(g->normal.y) << 16);
  o[1] = (uint32_t)float_to_half(g->normal.z) | ((uint32_t)float_to_half(g->albedo.x) << 16);
  o[2] = (uint32_t)float_to_half(g->albedo.y) | ((uint32_t)float_to_half(g->albedo.z) << 16);
  memcpy(&o[3], &g->depth, 4);
}

static guide_t load_guide(const uint32_t* o) {
  guide_t g;
  g.normal = V(half_to_float((uint16_t)(o[0] & 0xffffu)), half_to_float((uint16_t)(o[0] >> 16)), half_to_float((uint16_t)(o[1] & 0xffffu)));
  g.albedo = V(half_to_float((uint16_t)(o[1] >> 16)), half_to_float((uint16_t)(o[2] & 0xffffu)), half_to_float((uint16_t)(o[2] >> 16)));
  memcpy(&g.depth, &o[3], 4);
  return g;
}

/* One pixel of the path-traced megakernel (pathtrace.py:340-424). */
static void render_pixel_pt(const MjpbrScene* s, const int32_t* mesh_nface, int w, int c, int px, int py, uint32_t seed) {
  const MjpbrSettings* st = &s->settings;
  int W = s->cam_res[c][0], H = s->cam_res[c][1];
  int pixelid = py * W + px;
  cam_t cam = camera(s, w, c);
  ctx_t ctx;
  ctx.W.s = s;
  ctx.W.mesh_nface = mesh_nface;
  ctx.W.w = w;
  ctx.exposure = bf(s->exposure, w, 1, 0);
  ctx.ambient = bv3(s->ambient_radiance, w, 1, 0);
  ctx.env = 0;
  ctx.env_yaw = 0.0f;
  ctx.env_scale = 0.0f;
  if (s->nenv > 0 && s->env_id.ptr) {
    ctx.env = bi(s->env_id, w, 1, 0);
    ctx.env_yaw = bf(s->env_yaw, w, 1, 0);
    ctx.env_scale = bf(s->env_intensity, w, 1, 0);
  }
  const int centre = PT_SUBPIXEL / 2;
  if (!s->render_rgb[c]) {
    v3 dcam, ocam;
    float max_dist, depth_z;
    primary_ray(s, &cam, c, W, H, px, py, PT_SUBPIXEL, centre, centre, &dcam, &ocam, &max_dist, &depth_z);
    hit_t hit = closest(&ctx.W, vadd(cam.pos, mat_mul(cam.mat, ocam)), mat_mul(cam.mat, dcam), max_dist, st->cull_backfaces);
    write_geometry(s, w, c, pixelid, &hit, depth_z);
    return;
  }
  v3 head_dir = vneg(V(cam.mat[2], cam.mat[5], cam.mat[8]));
  uint32_t pixel_seed = seed + (uint32_t)w * (uint32_t)s->total_rays + (uint32_t)(s->ray_adr[c] + pixelid);
  v3 hdr = V(0, 0, 0), albedo_sum = V(0, 0, 0), normal_sum = V(0, 0, 0), emission_sum = V(0, 0, 0);
  float first_depth = 0.0f, lum_sq = 0.0f;
  int n = st->path_samples;
  int64_t adr = (int64_t)w * s->rgb_stride + s->rgb_adr[c] + pixelid;
  for (int smp = 0; smp < n; ++smp) {
    int sx = centre, sy = centre;
    if (smp > 0) {
      sx = (int)(pt_rand(pixel_seed, smp, PT_JITTER, 0) * (float)PT_SUBPIXEL);
      sy = (int)(pt_rand(pixel_seed, smp, PT_JITTER, 1) * (float)PT_SUBPIXEL);
    }
    v3 dcam, ocam;
    float max_dist, depth_z;
    primary_ray(s, &cam, c, W, H, px, py, PT_SUBPIXEL, sx, sy, &dcam, &ocam, &max_dist, &depth_z);
    primary_t first;
    v3 radiance =
        trace_path(&ctx, vadd(cam.pos, mat_mul(cam.mat, ocam)), mat_mul(cam.mat, dcam), max_dist, head_dir, pixel_seed, smp, &first);
    if (smp == 0) {
      write_geometry(s, w, c, pixelid, &first.hit, depth_z);
      if (st->render_guides && s->guide_albedo) {
        s->guide_albedo[adr * 3] = first.base_color.x;
        s->guide_albedo[adr * 3 + 1] = first.base_color.y;
        s->guide_albedo[adr * 3 + 2] = first.base_color.z;
        s->guide_normal[adr * 3] = first.normal.x;
        s->guide_normal[adr * 3 + 1] = first.normal.y;
        s->guide_normal[adr * 3 + 2] = first.normal.z;
      }
      if (first.hit.geom != -1) first_depth = first.hit.dist * -depth_z;
    }
    hdr = vadd(hdr, radiance);
    albedo_sum = vadd(albedo_sum, first.albedo);
    normal_sum = vadd(normal_sum, first.normal);
    emission_sum = vadd(emission_sum, first.emission);
    if (st->denoise) {
      float lum = lum709(radiance) * ctx.exposure;
      lum_sq += lum * lum;
    }
  }
  float inv_n = 1.0f / (float)n;
  hdr = vmul(hdr, inv_n);
  if (st->denoise) {
    /* denoise.py Features: albedo / normal at half precision, exposed emission, depth and the
     * variance of the pixel's mean exposed luminance; then _demodulate (denoise.py:84-91). */
    s->hdr_data[adr * 3] = hdr.x;
    s->hdr_data[adr * 3 + 1] = hdr.y;
    s->hdr_data[adr * 3 + 2] = hdr.z;
    v3 em = vmul(emission_sum, ctx.exposure * inv_n);
    v3 nm = normal_sum;
    if (vdot(nm, nm) > 0.0f) nm = vnorm(nm);
    guide_t g;
    g.normal = round_half3(nm);
    g.albedo = round_half3(vmul(albedo_sum, inv_n));
    g.depth = first_depth;
    store_guide(s->aov_guide + adr * 4, &g);
    float* e = s->aov_emission + adr * 3;
    e[0] = em.x, e[1] = em.y, e[2] = em.z;
    float mean_lum = lum709(hdr) * ctx.exposure;
    float variance = maxf(lum_sq * inv_n - mean_lum * mean_lum, 0.0f) * inv_n;
    v3 c = vsub(vmul(hdr, ctx.exposure), em);
    c = V(maxf(c.x, 0.0f) / maxf(g.albedo.x, MIN_ALBEDO), maxf(c.y, 0.0f) / maxf(g.albedo.y, MIN_ALBEDO),
          maxf(c.z, 0.0f) / maxf(g.albedo.z, MIN_ALBEDO));
    float scale = 1.0f / maxf(lum709(g.albedo), MIN_ALBEDO);
    float* d = s->denoise_buffers[0] + adr * 4;
    d[0] = c.x, d[1] = c.y, d[2] = c.z, d[3] = variance * scale * scale;
    return;
  }
  if (st->render_hdr && s->hdr_data) {
    s->hdr_data[adr * 3] = hdr.x;
    s->hdr_data[adr * 3 + 1] = hdr.y;
    s->hdr_data[adr * 3 + 2] = hdr.z;
  }
  s->rgb_data[adr] = encode_display(display_transform(vmul(hdr, ctx.exposure), st->tone_mapper));
}

/* ------------------------------------------------------------------ a-trous denoiser (denoise.py) */

static float b3w(int i) { return i == 2 ? 0.375f : ((i == 1 || i == 3) ? 0.25f : 0.0625f); }

/* One filter pass over one camera image of one world (denoise.py:101-178); step 0 copies. */
static void atrous_image(const MjpbrScene* s, int64_t base, int W, int H, int step, const float* src, float* dst) {
  const MjpbrSettings* st = &s->settings;
  for (int py = 0; py < H; ++py) {
    for (int px = 0; px < W; ++px) {
      int64_t idx = base + (int64_t)py * W + px;
      guide_t g0 = load_guide(s->aov_guide + idx * 4);
      const float* s0 = src + idx * 4;
      float* o = dst + idx * 4;
      if (step == 0 || vdot(g0.normal, g0.normal) == 0.0f) {
        memcpy(o, s0, 16);
        continue;
      }
      float variance = 0.0f, variance_weight = 0.0f;
      for (int j = 0; j < 3; ++j) {
        int y = clampi(py + j - 1, 0, H - 1);
        for (int i = 0; i < 3; ++i) {
          int x = clampi(px + i - 1, 0, W - 1);
          float g = (i == 1 ? 0.5f : 0.25f) * (j == 1 ? 0.5f : 0.25f);
          variance += g * src[(base + (int64_t)y * W + x) * 4 + 3];
          variance_weight += g;
        }
      }
      float inv_sigma_l = 1.0f / (st->denoise_sigma_color * sqrtf(maxf(variance / variance_weight, 0.0f)) + 1.0e-6f);
      float l0 = lum709(V(s0[0], s0[1], s0[2]));
      float inv_sigma_a = 1.0f / st->denoise_sigma_albedo;
      float inv_sigma_z = 1.0f / maxf(st->denoise_sigma_depth * g0.depth * (float)step, 1.0e-6f);
      v3 total = V(0, 0, 0);
      float total_variance = 0.0f, weight_sum = 0.0f;
      for (int j = 0; j < 5; ++j) {
        int y = py + (j - 2) * step;
        if (y < 0 || y >= H) continue;
        for (int i = 0; i < 5; ++i) {
          int x = px + (i - 2) * step;
          if (x < 0 || x >= W) continue;
          int64_t q = base + (int64_t)y * W + x;
          const float* sq = src + q * 4;
          guide_t gq = load_guide(s->aov_guide + q * 4);
          v3 c = V(sq[0], sq[1], sq[2]);
          float wn = powf(maxf(vdot(g0.normal, gq.normal), 0.0f), st->denoise_sigma_normal);
          float distance = fabsf(gq.depth - g0.depth) * inv_sigma_z + fabsf(lum709(c) - l0) * inv_sigma_l +
                           vlen(vsub(gq.albedo, g0.albedo)) * inv_sigma_a;
          float weight = b3w(i) * b3w(j) * wn * expf(-distance);
          total = vadd(total, vmul(c, weight));
          total_variance += weight * weight * sq[3];
          weight_sum += weight;
        }
      }
      v3 c = vdiv(total, weight_sum);
      o[0] = c.x, o[1] = c.y, o[2] = c.z, o[3] = total_variance / (weight_sum * weight_sum);
    }
  }
}

/* Remodulation, tone mapping and encoding (denoise.py:181-201). */
static void finish_image(const MjpbrScene* s, int w, int64_t base, int npix, const float* src) {
  const MjpbrSettings* st = &s->settings;
  float exposure = bf(s->exposure, w, 1, 0);
  for (int64_t k = base; k < base + npix; ++k) {
    guide_t g = load_guide(s->aov_guide + k * 4);
    const float* c = src + k * 4;
    const float* e = s->aov_emission + k * 3;
    v3 exposed = V(e[0] + c[0] * maxf(g.albedo.x, MIN_ALBEDO), e[1] + c[1] * maxf(g.albedo.y, MIN_ALBEDO),
                   e[2] + c[2] * maxf(g.albedo.z, MIN_ALBEDO));
    if (st->render_hdr && s->hdr_data) {
      v3 h = vdiv(exposed, exposure);
      s->hdr_data[k * 3] = h.x, s->hdr_data[k * 3 + 1] = h.y, s->hdr_data[k * 3 + 2] = h.z;
    }
    s->rgb_data[k] = encode_display(display_transform(exposed, st->tone_mapper));
  }
}

/* ------------------------------------------------------------------ exported */

int oracle_nthreads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

static int render_worlds(const MjpbrScene* s, const int32_t* mesh_nface, uint32_t seed, int w0, int w1, int nthreads,
                         int path_traced) {
  if (!s || w0 < 0 || w1 > s->nworld || w0 > w1) return 1;
  int64_t nrow = 0;
  int row_cam[MJPBR_MAX_RENDER + 1];
  row_cam[0] = 0;
  for (int c = 0; c < s->nrender; ++c) row_cam[c + 1] = row_cam[c] + s->cam_res[c][1];
  nrow = row_cam[s->nrender];
  int64_t total = (int64_t)(w1 - w0) * nrow;
  if (g_use_mesh_bvh && s->nmesh > 0 && mesh_nface && s->mesh_vert) {
    g_mesh_bvh = (obvh_t*)calloc((size_t)s->nmesh, sizeof(obvh_t));
    g_mesh_bvh_count = s->nmesh;
    for (int m = 0; m < s->nmesh; ++m) obvh_build(s, m, mesh_nface[m], &g_mesh_bvh[m]);
  }
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4)
#endif
  for (int64_t job = 0; job < total; ++job) {
    int w = w0 + (int)(job / nrow);
    int r = (int)(job % nrow);
    int c = 0;
    while (c + 1 < s->nrender && r >= row_cam[c + 1]) ++c;
    if (!(s->render_rgb[c] || s->render_depth[c] || s->render_seg[c])) continue;
    int py = r - row_cam[c];
    for (int px = 0; px < s->cam_res[c][0]; ++px) {
      if (path_traced)
        render_pixel_pt(s, mesh_nface, w, c, px, py, seed);
      else
        render_pixel(s, mesh_nface, w, c, px, py, seed);
    }
  }
  if (g_mesh_bvh) {
    for (int m = 0; m < g_mesh_bvh_count; ++m) {
      free(g_mesh_bvh[m].nodes);
      free(g_mesh_bvh[m].order);
    }
    free(g_mesh_bvh);
    g_mesh_bvh = NULL;
    g_mesh_bvh_count = 0;
  }
  return 0;
}

/* Real-time tier of worlds [w0, w1) into the scene's (host) output buffers. mesh_nface: faces per
 * mesh (host). nthreads <= 0: all. */
int oracle_render_rt(const MjpbrScene* s, const int32_t* mesh_nface, uint32_t seed, int w0, int w1, int nthreads) {
  return render_worlds(s, mesh_nface, seed, w0, w1, nthreads, 0);
}

/* Path-traced tier of worlds [w0, w1): RGB (or, with settings.denoise, the noisy HDR and the
 * denoiser's features), depth and segmentation. */
int oracle_render_pt(const MjpbrScene* s, const int32_t* mesh_nface, uint32_t seed, int w0, int w1, int nthreads) {
  return render_worlds(s, mesh_nface, seed, w0, w1, nthreads, 1);
}

/* The a-trous denoiser over every world and RGB camera: reads denoise_buffers[0] (demodulated
 * radiance + variance, written by oracle_render_pt), aov_guide and aov_emission; ping-pongs
 * through both denoise buffers; writes rgb_data (and hdr_data with render_hdr). */
int oracle_denoise(const MjpbrScene* s, int nthreads) {
  if (!s || !s->aov_guide || !s->aov_emission || !s->denoise_buffers[0] || !s->denoise_buffers[1]) return 1;
  int passes = s->denoise_iterations;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 1)
#endif
  for (int w = 0; w < s->nworld; ++w) {
    for (int c = 0; c < s->nrender; ++c) {
      if (!s->render_rgb[c] || s->rgb_adr[c] < 0) continue;
      int W = s->cam_res[c][0], H = s->cam_res[c][1];
      int64_t base = (int64_t)w * s->rgb_stride + s->rgb_adr[c];
      int cur = 0;
      for (int i = 0; i < passes; ++i) {
        atrous_image(s, base, W, H, 1 << i, s->denoise_buffers[cur], s->denoise_buffers[1 - cur]);
        cur = 1 - cur;
      }
      finish_image(s, w, base, W * H, s->denoise_buffers[cur]);
    }
  }
  return 0;
}

/* 1: mesh queries use the oracle's own BVH (default); 0: brute force over every face. */
void oracle_set_mesh_bvh(int enable) { g_use_mesh_bvh = enable; }

/* Split-sum DFG table (size, size, 2), ibl.py:62-93. */
void oracle_dfg_lut(float* lut, int n, int nsample) {
  for (int j = 0; j < n; ++j) {
    for (int i = 0; i < n; ++i) {
      float nov = ((float)i + 0.5f) / (float)n, pr = ((float)j + 0.5f) / (float)n;
      float alpha = pr * pr;
      v3 v = V(sqrtf(1.0f - nov * nov), 0.0f, nov);
      float inv_n = 1.0f / (float)nsample;
      float x = 0.0f, y = 0.0f;
      for (int s = 0; s < nsample; ++s) {
        uint32_t bits = (uint32_t)s;
        bits = (bits << 16) | (bits >> 16);
        bits = ((bits & 0x55555555u) << 1) | ((bits & 0xAAAAAAAAu) >> 1);
        bits = ((bits & 0x33333333u) << 2) | ((bits & 0xCCCCCCCCu) >> 2);
        bits = ((bits & 0x0F0F0F0Fu) << 4) | ((bits & 0xF0F0F0F0u) >> 4);
        bits = ((bits & 0x00FF00FFu) << 8) | ((bits & 0xFF00FF00u) >> 8);
        float ux = (float)s * inv_n, uy = (float)bits * (1.0f / 4294967296.0f);
        float a2 = alpha * alpha;
        float phi = 2.0f * PI_F * ux;
        float cos2 = (1.0f - uy) / (1.0f + (a2 - 1.0f) * uy);
        float ct = sqrtf(cos2), stt = sqrtf(maxf(1.0f - cos2, 0.0f));
        v3 h = V(stt * cosf(phi), stt * sinf(phi), ct);
        float voh = vdot(v, h);
        v3 l = vsub(vmul(h, 2.0f * voh), v);
        float nol = l.z, noh = h.z;
        if (nol > 0.0f && voh > 0.0f) {
          float gv = v_smith(nov, nol, alpha) * 4.0f * voh * nol / noh;
          float fc = powf(1.0f - voh, 5.0f);
          x += gv * fc;
          y += gv;
        }
      }
      lut[(j * n + i) * 2] = x * inv_n;
      lut[(j * n + i) * 2 + 1] = y * inv_n;
    }
  }
}

/* Box-filtered mips of a texture whose level 0 is filled (host data). */
void oracle_build_mips(const MjpbrTexture* t, uint8_t* data) {
  for (int level = 1; level < t->nlevel; ++level) {
    int sw = t->width >> (level - 1), sh = t->height >> (level - 1);
    int dw = t->width >> level, dh = t->height >> level;
    if (sw < 1) sw = 1;
    if (sh < 1) sh = 1;
    if (dw < 1) dw = 1;
    if (dh < 1) dh = 1;
    for (int y = 0; y < dh; ++y) {
      for (int x = 0; x < dw; ++x) {
        int x0 = 2 * x < sw - 1 ? 2 * x : sw - 1, x1 = 2 * x + 1 < sw - 1 ? 2 * x + 1 : sw - 1;
        int y0 = 2 * y < sh - 1 ? 2 * y : sh - 1, y1 = 2 * y + 1 < sh - 1 ? 2 * y + 1 : sh - 1;
        if (t->format == MJPBR_TEX_RGBA8) {
          const uint8_t* src = data + t->level_offset[level - 1];
          uint8_t* dst = data + t->level_offset[level];
          for (int k = 0; k < 4; ++k) {
            unsigned sum = src[(y0 * sw + x0) * 4 + k] + src[(y0 * sw + x1) * 4 + k] + src[(y1 * sw + x0) * 4 + k] +
                           src[(y1 * sw + x1) * 4 + k];
            dst[(y * dw + x) * 4 + k] = (uint8_t)((sum + 2u) >> 2);
          }
        } else {
          const uint16_t* src = (const uint16_t*)(data + t->level_offset[level - 1]);
          uint16_t* dst = (uint16_t*)(data + t->level_offset[level]);
          for (int k = 0; k < 4; ++k) {
            float sum = half_to_float(src[(y0 * sw + x0) * 4 + k]) + half_to_float(src[(y0 * sw + x1) * 4 + k]) +
                        half_to_float(src[(y1 * sw + x0) * 4 + k]) + half_to_float(src[(y1 * sw + x1) * 4 + k]);
            dst[(y * dw + x) * 4 + k] = float_to_half(sum * 0.25f);
          }
        }
      }
    }
  }
}

/* GGX-prefiltered stack (levels, h, w, 4) float16 of a RGBA16F radiance texture (host data),
 * envmap.py:171-221. */
void oracle_prefilter(const MjpbrTexture* t, const uint8_t* data, int levels, int h, int w, int nsample, uint16_t* stack) {
#ifdef _OPENMP
#pragma omp parallel for collapse(2) schedule(dynamic, 8)
#endif
  for (int level = 0; level < levels; ++level) {
    for (int y = 0; y < h; ++y) {
      for (int x = 0; x < w; ++x) {
        float uu = ((float)x + 0.5f) / (float)w, vv = ((float)y + 0.5f) / (float)h;
        float phi = (uu - 0.5f) * (2.0f * PI_F), theta = vv * PI_F;
        float st = sinf(theta);
        v3 n = V(st * cosf(phi), st * sinf(phi), cosf(theta));
        float pr = (float)level / (float)(levels - 1);
        float alpha = maxf(pr * pr, 1.0e-4f);
        v3 up = fabsf(n.z) < 0.999f ? V(0, 0, 1) : V(1, 0, 0);
        v3 tt = vnorm(vcross(up, n));
        v3 bb = vcross(n, tt);
        float texel_sa = 4.0f * PI_F / (float)(t->width * t->height);
        float inv_n = 1.0f / (float)nsample;
        v3 color = V(0, 0, 0);
        float weight = 0.0f;
        for (int s = 0; s < nsample; ++s) {
          uint32_t bits = (uint32_t)s;
          bits = (bits << 16) | (bits >> 16);
          bits = ((bits & 0x55555555u) << 1) | ((bits & 0xAAAAAAAAu) >> 1);
          bits = ((bits & 0x33333333u) << 2) | ((bits & 0xCCCCCCCCu) >> 2);
          bits = ((bits & 0x0F0F0F0Fu) << 4) | ((bits & 0xF0F0F0F0u) >> 4);
          bits = ((bits & 0x00FF00FFu) << 8) | ((bits & 0xFF00FF00u) >> 8);
          float ux = (float)s * inv_n, uy = (float)bits * (1.0f / 4294967296.0f);
          float a2 = alpha * alpha;
          float ph = 2.0f * PI_F * ux;
          float cos2 = (1.0f - uy) / (1.0f + (a2 - 1.0f) * uy);
          float ct = sqrtf(cos2), stt = sqrtf(maxf(1.0f - cos2, 0.0f));
          v3 hl = V(stt * cosf(ph), stt * sinf(ph), ct);
          v3 hh = vadd(vadd(vmul(tt, hl.x), vmul(bb, hl.y)), vmul(n, hl.z));
          float noh = hl.z;
          v3 l = vsub(vmul(hh, 2.0f * noh), n);
          float nol = vdot(n, l);
          if (nol > 0.0f) {
            float pdf = d_ggx(noh, alpha) * 0.25f;
            float sa = inv_n / maxf(pdf, 1.0e-8f);
            float lod = level == 0 ? 0.0f : 0.5f * log2f(sa / texel_sa) + 1.0f;
            float u, v, c[4];
            direction_to_uv(l, 0.0f, &u, &v);
            sample_trilinear(t, data, u, v, maxf(lod, 0.0f), 1, 0, c);
            color = vadd(color, vmul(V(c[0], c[1], c[2]), nol));
            weight += nol;
          }
        }
        color = vdiv(color, maxf(weight, 1.0e-8f));
        uint16_t* o = stack + (((int64_t)level * h + y) * w + x) * 4;
        o[0] = float_to_half(color.x);
        o[1] = float_to_half(color.y);
        o[2] = float_to_half(color.z);
        o[3] = float_to_half(1.0f);
      }
    }
  }
}

void oracle_struct_layout(int64_t out[8]) {
  out[0] = (int64_t)sizeof(MjpbrScene);
  out[1] = (int64_t)sizeof(MjpbrSettings);
  out[2] = (int64_t)sizeof(MjpbrTexture);
  out[3] = (int64_t)offsetof(MjpbrScene, nrender);
  out[4] = (int64_t)offsetof(MjpbrScene, world_blocks);
  out[5] = (int64_t)offsetof(MjpbrScene, env_prefiltered);
  out[6] = (int64_t)offsetof(MjpbrScene, error_word);
  out[7] = (int64_t)offsetof(MjpbrScene, settings);
}

/* float <-> half of this file (exported for the fixtures' tests). */
uint16_t oracle_float_to_half(float f) { return float_to_half(f); }
float oracle_half_to_float(uint16_t h) { return half_to_float(h); }

/* Deterministic sincos and random numbers (exported so tests can pin them). */
void oracle_sincos_turns(float t, float* s, float* c) { sincos_turns(t, s, c); }
float oracle_rand01(uint32_t seed, uint32_t counter) { return rand01(seed, counter); }
