// Ray queries of the render kernels: ray/primitive intersection (MuJoCo's analytic tests), the
// watertight ray/triangle test, and the two-level BVH traversal over one world's block of
// records in shared memory plus the shared mesh BVHs in global memory.
//
// Reference behaviour (julien-blanchon/mujoco_warp_pbr):
//  * ordered nearest-first traversal with per-child entry distances, cut-off widened by the tie
//    tolerance, rgba.a == 0 geoms skipped, backface culling by the geometric normal, ties to the
//    higher geom id: mujoco_warp_pbr/_src/traverse.py:195-325 (_ray_aabb at :115-124);
//  * per-geom tests are MuJoCo Warp's ray_plane/sphere/ellipsoid/capsule/cylinder/box and
//    ray_mesh_with_bvh(_anyhit), called at mujoco_warp_pbr/_src/traverse.py:132-192. Those live in
//    the third-party mujoco_warp package; the functions below restate MuJoCo's published
//    algorithms (engine_ray.c: local-frame mapping, the half-b quadratic "ray_quad", the capsule
//    and cylinder side/cap decomposition, the box slab faces, the one-sided plane) and Woop,
//    Benthin and Wald, "Watertight Ray/Triangle Intersection" (JCGT 2013) for triangles.
// All of it is plain float arithmetic (see common.cuh) except the conservative box test.
#pragma once

#include "common.cuh"
#include "world_block.cuh"

namespace mjpbr {

struct Ray {
  V3 o;
  V3 d;
};

struct Hit {
  int32_t geom;  // geom id, -1 on a miss
  int32_t slot;  // slot of the geom in the world block
  float dist;
  V3 normal;     // geometric normal, world frame
  float u, v;    // barycentrics of vertex 0 and vertex 1 (meshes)
  int32_t face;  // triangle of the mesh, -1 for primitives
  int32_t mesh;  // mesh id, -1 for primitives
};

// Ray with reciprocal direction for box tests; zero direction components are replaced by
// +-1e-30 so products stay finite.
struct RayInv {
  V3 inv;
  V3 oinv;
};

MJ_HD float safe_rcp(float x) { return 1.0f / (fabsf(x) > 1.0e-30f ? x : (x >= 0.0f ? 1.0e-30f : -1.0e-30f)); }

MJ_DEV RayInv make_inv(const Ray& r) {
  RayInv ri;
  ri.inv = V3{safe_rcp(r.d.x), safe_rcp(r.d.y), safe_rcp(r.d.z)};
  ri.oinv = cmul(r.o, ri.inv);
  return ri;
}

// Entry distance (>= 0) of the ray into [lo, hi], or -1 if missed or at/after max_t. Boxes are
// padded when they are built, so rounding here never drops a box a primitive inside it is hit in.
MJ_DEV float box_entry(const RayInv& ri, float lx, float ly, float lz, float hx, float hy, float hz, float max_t) {
  float t1x = __fmaf_rn(lx, ri.inv.x, -ri.oinv.x);
  float t2x = __fmaf_rn(hx, ri.inv.x, -ri.oinv.x);
  float t1y = __fmaf_rn(ly, ri.inv.y, -ri.oinv.y);
  float t2y = __fmaf_rn(hy, ri.inv.y, -ri.oinv.y);
  float t1z = __fmaf_rn(lz, ri.inv.z, -ri.oinv.z);
  float t2z = __fmaf_rn(hz, ri.inv.z, -ri.oinv.z);
  float tmin = fmaxf(fmaxf(fminf(t1x, t2x), fminf(t1y, t2y)), fminf(t1z, t2z));
  float tmax = fminf(fminf(fmaxf(t1x, t2x), fmaxf(t1y, t2y)), fmaxf(t1z, t2z));
  float entry = fmaxf(tmin, 0.0f);
  return (tmax >= entry && entry < max_t) ? entry : -1.0f;
}

// MuJoCo's ray_quad: roots of a x^2 + 2 b x + c = 0 in x0 <= x1; returns the smaller
// non-negative one or -1.
MJ_HD float ray_quad(float a, float b, float c, float* x0, float* x1) {
  float det = b * b - a * c;
  if (det < kMinVal) {
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

// Geom frame of a world-block geom record.
struct GeomFrame {
  V3 pos;
  M3 mat;
  V3 size;
};

// Ray in the geom's local frame.
MJ_HD void map_local(const GeomFrame& g, const Ray& r, V3* lo, V3* ld) {
  V3 dif = r.o - g.pos;
  *lo = mul_t(g.mat, dif);
  *ld = mul_t(g.mat, r.d);
}

MJ_HD float ray_plane(const GeomFrame& g, const Ray& r, V3* n) {
  V3 lo, ld;
  map_local(g, r, &lo, &ld);
  if (ld.z > -kMinVal) return -1.0f;
  float x = -lo.z / ld.z;
  if (x < 0.0f) return -1.0f;
  float p0 = lo.x + x * ld.x;
  float p1 = lo.y + x * ld.y;
  if ((g.size.x <= 0.0f || fabsf(p0) <= g.size.x) && (g.size.y <= 0.0f || fabsf(p1) <= g.size.y)) {
    *n = V3{g.mat.m[2], g.mat.m[5], g.mat.m[8]};
    return x;
  }
  return -1.0f;
}

MJ_HD float ray_sphere(const GeomFrame& g, const Ray& r, V3* n) {
  V3 dif = r.o - g.pos;
  float a = dot(r.d, r.d);
  float b = dot(r.d, dif);
  float c = dot(dif, dif) - g.size.x * g.size.x;
  float x0, x1;
  float x = ray_quad(a, b, c, &x0, &x1);
  if (x < 0.0f) return -1.0f;
  *n = normalize(dif + r.d * x);
  return x;
}

MJ_HD float ray_ellipsoid(const GeomFrame& g, const Ray& r, V3* n) {
  V3 lo, ld;
  map_local(g, r, &lo, &ld);
  V3 s = V3{1.0f / g.size.x, 1.0f / g.size.y, 1.0f / g.size.z};
  V3 sd = cmul(ld, s);
  V3 so = cmul(lo, s);
  float a = dot(sd, sd);
  float b = dot(sd, so);
  float c = dot(so, so) - 1.0f;
  float x0, x1;
  float x = ray_quad(a, b, c, &x0, &x1);
  if (x < 0.0f) return -1.0f;
  V3 p = lo + ld * x;
  V3 ln = normalize(cmul(p, cmul(s, s)));
  *n = mul(g.mat, ln);
  return x;
}

// part: 0 round side, 1 top cap, 2 bottom cap.
MJ_HD float ray_capsule(const GeomFrame& g, const Ray& r, V3* n) {
  V3 lo, ld;
  map_local(g, r, &lo, &ld);
  float rad = g.size.x, h = g.size.y;
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
  float aa = dot(ld, ld);
  for (int cap = 0; cap < 2; ++cap) {
    float zc = cap == 0 ? h : -h;
    V3 dif = V3{lo.x, lo.y, lo.z - zc};
    float bb = dot(ld, dif);
    float cc = dot(dif, dif) - rad * rad;
    ray_quad(aa, bb, cc, &x0, &x1);
    float xs[2] = {x0, x1};
    for (int i = 0; i < 2; ++i) {
      float z = lo.z + xs[i] * ld.z;
      bool side_ok = cap == 0 ? (z >= h) : (z <= -h);
      if (xs[i] >= 0.0f && side_ok && (x < 0.0f || xs[i] < x)) {
        x = xs[i];
        part = 1 + cap;
      }
    }
  }
  if (x < 0.0f) return -1.0f;
  V3 p = lo + ld * x;
  V3 ln;
  if (part == 0) {
    ln = normalize(V3{p.x, p.y, 0.0f});
  } else {
    ln = normalize(V3{p.x, p.y, p.z - (part == 1 ? h : -h)});
  }
  *n = mul(g.mat, ln);
  return x;
}

MJ_HD float ray_cylinder(const GeomFrame& g, const Ray& r, V3* n) {
  V3 lo, ld;
  map_local(g, r, &lo, &ld);
  float rad = g.size.x, h = g.size.y;
  float x = -1.0f;
  int part = -1;
  // flat caps
  if (fabsf(ld.z) > kMinVal) {
    for (int cap = 0; cap < 2; ++cap) {
      float zc = cap == 0 ? h : -h;
      float sol = (zc - lo.z) / ld.z;
      if (sol >= 0.0f) {
        float px = lo.x + sol * ld.x;
        float py = lo.y + sol * ld.y;
        if (px * px + py * py <= rad * rad && (x < 0.0f || sol < x)) {
          x = sol;
          part = 1 + cap;
        }
      }
    }
  }
  // round side
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
  V3 ln;
  if (part == 0) {
    V3 p = lo + ld * x;
    ln = normalize(V3{p.x, p.y, 0.0f});
  } else {
    ln = V3{0.0f, 0.0f, part == 1 ? 1.0f : -1.0f};
  }
  *n = mul(g.mat, ln);
  return x;
}

MJ_HD float ray_box(const GeomFrame& g, const Ray& r, V3* n) {
  V3 lo, ld;
  map_local(g, r, &lo, &ld);
  float lp[3] = {lo.x, lo.y, lo.z};
  float lv[3] = {ld.x, ld.y, ld.z};
  float sz[3] = {g.size.x, g.size.y, g.size.z};
  float x = -1.0f;
  int face_axis = -1;
  float face_side = 0.0f;
  for (int i = 0; i < 3; ++i) {
    if (fabsf(lv[i]) > kMinVal) {
      for (int side = -1; side <= 1; side += 2) {
        float sol = ((float)side * sz[i] - lp[i]) / lv[i];
        if (sol >= 0.0f) {
          int j = i == 0 ? 1 : 0;
          int k = i == 2 ? 1 : 2;
          if (fabsf(lp[j] + sol * lv[j]) <= sz[j] && fabsf(lp[k] + sol * lv[k]) <= sz[k] && (x < 0.0f || sol < x)) {
            x = sol;
            face_axis = i;
            face_side = (float)side;
          }
        }
      }
    }
  }
  if (x < 0.0f) return -1.0f;
  // column face_axis of the frame, times the side
  *n = V3{g.mat.m[face_axis] * face_side, g.mat.m[3 + face_axis] * face_side, g.mat.m[6 + face_axis] * face_side};
  return x;
}

// Watertight ray/triangle test set-up (Woop et al. 2013): axis permutation and shear of one ray.
struct WoopRay {
  int kx, ky, kz;
  float sx, sy, sz;
  V3 o;
};

MJ_HD WoopRay woop_setup(V3 o, V3 d) {
  WoopRay w;
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

MJ_HD float comp(V3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

// Hit distance in [0, tmax) or -1; barycentrics of v0 (u) and v1 (v).
MJ_HD float woop_hit(const WoopRay& w, V3 v0, V3 v1, V3 v2, float tmax, float* bu, float* bv) {
  V3 A = v0 - w.o, B = v1 - w.o, C = v2 - w.o;
  float az = comp(A, w.kz), bz = comp(B, w.kz), cz = comp(C, w.kz);
  float ax = comp(A, w.kx) - w.sx * az;
  float ay = comp(A, w.ky) - w.sy * az;
  float bx = comp(B, w.kx) - w.sx * bz;
  float by = comp(B, w.ky) - w.sy * bz;
  float cx = comp(C, w.kx) - w.sx * cz;
  float cy = comp(C, w.ky) - w.sy * cz;
  float U = cx * by - cy * bx;
  float V = ax * cy - ay * cx;
  float W = bx * ay - by * ax;
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return -1.0f;
  float det = U + V + W;
  if (det == 0.0f) return -1.0f;
  float T = U * (w.sz * az) + V * (w.sz * bz) + W * (w.sz * cz);
  float t = T / det;
  if (!(t >= 0.0f && t < tmax)) return -1.0f;
  *bu = U / det;
  *bv = V / det;
  return t;
}

}  // namespace mjpbr
