// Closest-hit and any-hit queries of one world: nearest-first traversal of the world's scene BVH
// (nodes in the shared-memory copy of the world block) and, for mesh geoms, of the mesh's BVH in
// global memory in the mesh frame. Semantics follow mujoco_warp_pbr/_src/traverse.py:195-325:
// entry distances are stored with pushed children, a child whose entry is at or beyond the
// current cut-off dist * (1 + tol) + tol_abs is skipped, ties within tol go to the higher geom id,
// hits with a normal along the ray are culled when culling is on, alpha-0 geoms are skipped.
#pragma once

#include "geometry.cuh"

namespace mjpbr {

constexpr int kTlasStack = 32;
constexpr int kBlasStack = 40;

MJ_DEV GeomFrame geom_frame(const float* g) {
  GeomFrame f;
  f.pos = V3{g[0], g[1], g[2]};
  f.mat.m[0] = g[4];
  f.mat.m[1] = g[5];
  f.mat.m[2] = g[6];
  f.mat.m[3] = g[8];
  f.mat.m[4] = g[9];
  f.mat.m[5] = g[10];
  f.mat.m[6] = g[12];
  f.mat.m[7] = g[13];
  f.mat.m[8] = g[14];
  f.size = V3{g[7], g[11], g[15]};
  return f;
}

MJ_DEV float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

// Closest (or, with kAny, any) triangle of mesh `mesh` hit by the local ray in [0, tmax).
// Returns the distance or -1; on a closest hit fills the local geometric normal and barycentrics.
template <bool kAny>
__device__ __noinline__ float mesh_query(const MjpbrScene& sc, int32_t mesh, V3 lo, V3 ld, float tmax, bool cull, V3* n_local,
                        float* bu, float* bv, int32_t* face, int32_t* err) {
  const float* nodes = sc.blas_nodes + (int64_t)sc.blas_root[mesh] * kNodeFloats;
  const float* tris = sc.blas_tris + (int64_t)sc.blas_tri_base[mesh] * kTriFloats;
  WoopRay w = woop_setup(lo, ld);
  Ray lr{lo, ld};
  RayInv ri = make_inv(lr);
  int32_t st_code[kBlasStack];
  float st_t[kBlasStack];
  int sp = 0;
  float best = tmax;
  int32_t found = -1;
  V3 e1b = v3(0.0f), e2b = v3(0.0f);
  float ub = 0.0f, vb = 0.0f;
  // start from the root node's children
  st_code[0] = 0;  // node 0, count 0
  st_t[0] = 0.0f;
  sp = 1;
  while (sp > 0) {
    --sp;
    if (st_t[sp] >= best) continue;
    int32_t code = st_code[sp];
    int32_t ref = code >> 3, cnt = code & 7;
    if (cnt == 0) {
      const float* nd = nodes + (int64_t)ref * kNodeFloats;
      float4 alo = ldg4(nd), ahi = ldg4(nd + 4), blo = ldg4(nd + 8), bhi = ldg4(nd + 12);
      int32_t acnt = __float_as_int(ahi.w), bcnt = __float_as_int(bhi.w);
      float ta = acnt >= 0 ? box_entry(ri, alo.x, alo.y, alo.z, ahi.x, ahi.y, ahi.z, best) : -1.0f;
      float tb = bcnt >= 0 ? box_entry(ri, blo.x, blo.y, blo.z, bhi.x, bhi.y, bhi.z, best) : -1.0f;
      int32_t ca = (__float_as_int(alo.w) << 3) | acnt;
      int32_t cb = (__float_as_int(blo.w) << 3) | bcnt;
      int32_t cn = ca, cf = cb;
      float tn = ta, tf = tb;
      if (tb >= 0.0f && (ta < 0.0f || tb < ta)) {
        cn = cb;
        cf = ca;
        tn = tb;
        tf = ta;
      }
      if (tf >= 0.0f) {
        if (sp < kBlasStack) {
          st_code[sp] = cf;
          st_t[sp++] = tf;
        } else {
          *err |= kErrStackOverflow;
        }
      }
      if (tn >= 0.0f) {
        if (sp < kBlasStack) {
          st_code[sp] = cn;
          st_t[sp++] = tn;
        } else {
          *err |= kErrStackOverflow;
        }
      }
      continue;
    }
    for (int32_t i = ref; i < ref + cnt; ++i) {
      const float* tr = tris + (int64_t)i * kTriFloats;
      float4 a = ldg4(tr), b = ldg4(tr + 4), c = ldg4(tr + 8);
      V3 v0{a.x, a.y, a.z}, v1{b.x, b.y, b.z}, v2{c.x, c.y, c.z};
      float u, v;
      float t = woop_hit(w, v0, v1, v2, best, &u, &v);
      if (t < 0.0f) continue;
      V3 e1 = v1 - v0, e2 = v2 - v0;
      if (!kAny && cull && dot(ld, cross(e1, e2)) > 0.0f) continue;
      if (kAny) return t;
      best = t;
      found = __float_as_int(a.w);
      e1b = e1;
      e2b = e2;
      ub = u;
      vb = v;
    }
  }
  if (found < 0) return -1.0f;
  *n_local = normalize(cross(e1b, e2b));
  *bu = ub;
  *bv = vb;
  *face = found;
  return best;
}

// One geom against the ray: distance (or -1), world normal, mesh hit details.
template <bool kMesh, bool kAny>
MJ_DEV float intersect_geom(const MjpbrScene& sc, const float* g, const Ray& r, float max_t, bool cull, V3* n,
                            float* u, float* v, int32_t* face, int32_t* mesh, int32_t* err) {
  int32_t type = __float_as_int(g[3]);
  GeomFrame f = geom_frame(g);
  float d = -1.0f;
  switch (type) {
    case MJPBR_GEOM_PLANE:
      d = ray_plane(f, r, n);
      break;
    case MJPBR_GEOM_SPHERE:
      d = ray_sphere(f, r, n);
      break;
    case MJPBR_GEOM_ELLIPSOID:
      d = ray_ellipsoid(f, r, n);
      break;
    case MJPBR_GEOM_CAPSULE:
      d = ray_capsule(f, r, n);
      break;
    case MJPBR_GEOM_CYLINDER:
      d = ray_cylinder(f, r, n);
      break;
    case MJPBR_GEOM_BOX:
      d = ray_box(f, r, n);
      break;
    default:
      if (kMesh && (type == MJPBR_GEOM_MESH || type == MJPBR_GEOM_SDF)) {
        int32_t mid = __float_as_int(g[17]);
        if (mid >= 0) {
          V3 lo, ld, nl = v3(0.0f);
          map_local(f, r, &lo, &ld);
          d = mesh_query<kAny>(sc, mid, lo, ld, max_t, cull, &nl, u, v, face, err);
          *n = kAny ? v3(0.0f) : mul(f.mat, nl);
          *mesh = mid;
        }
      }
      break;
  }
  return d;
}

// Closest hit within max_dist (the reference's trace_closest).
template <bool kMesh>
__device__ __noinline__ Hit closest_hit(const MjpbrScene& sc, const float* blk, const BlockLayout& L, const Ray& r, float max_dist,
                       bool cull, int32_t* err) {
  Hit h;
  h.geom = -1;
  h.slot = -1;
  h.dist = max_dist;
  h.normal = v3(0.0f);
  h.u = 0.0f;
  h.v = 0.0f;
  h.face = -1;
  h.mesh = -1;
  RayInv ri = make_inv(r);
  int32_t st_code[kTlasStack];
  float st_t[kTlasStack];
  st_code[0] = 0;
  st_t[0] = 0.0f;
  int sp = 1;
  while (sp > 0) {
    --sp;
    float cut = h.dist * (1.0f + kRayTolRel) + kRayTolAbs;
    if (st_t[sp] >= cut) continue;
    int32_t code = st_code[sp];
    int32_t ref = code >> 3, cnt = code & 7;
    if (cnt == 0) {
      const float* nd = blk + L.node_off + ref * kNodeFloats;
      int32_t acnt = __float_as_int(nd[7]), bcnt = __float_as_int(nd[15]);
      float ta = acnt >= 0 ? box_entry(ri, nd[0], nd[1], nd[2], nd[4], nd[5], nd[6], cut) : -1.0f;
      float tb = bcnt >= 0 ? box_entry(ri, nd[8], nd[9], nd[10], nd[12], nd[13], nd[14], cut) : -1.0f;
      int32_t ca = (__float_as_int(nd[3]) << 3) | acnt;
      int32_t cb = (__float_as_int(nd[11]) << 3) | bcnt;
      int32_t cn = ca, cf = cb;
      float tn = ta, tf = tb;
      if (tb >= 0.0f && (ta < 0.0f || tb < ta)) {
        cn = cb;
        cf = ca;
        tn = tb;
        tf = ta;
      }
      if (tf >= 0.0f) {
        if (sp < kTlasStack) {
          st_code[sp] = cf;
          st_t[sp++] = tf;
        } else {
          *err |= kErrStackOverflow;
        }
      }
      if (tn >= 0.0f) {
        if (sp < kTlasStack) {
          st_code[sp] = cn;
          st_t[sp++] = tn;
        } else {
          *err |= kErrStackOverflow;
        }
      }
      continue;
    }
    for (int32_t slot = ref; slot < ref + cnt; ++slot) {
      const float* g = blk + L.geom_off + slot * kGeomFloats;
      if (__float_as_int(g[19]) & kGeomFlagSkip) continue;
      cut = h.dist * (1.0f + kRayTolRel) + kRayTolAbs;
      V3 n = v3(0.0f);
      float u = 0.0f, v = 0.0f;
      int32_t face = -1, mesh = -1;
      float d = intersect_geom<kMesh, false>(sc, g, r, cut, cull, &n, &u, &v, &face, &mesh, err);
      if (cull && d >= 0.0f && dot(r.d, n) > 0.0f) d = -1.0f;
      int32_t gi = __float_as_int(g[16]);
      float tol = kRayTolRel * fmaxf(h.dist, 1.0f);
      bool closer = (d < h.dist - tol) || (fabsf(d - h.dist) <= tol && (h.geom < 0 || gi > h.geom));
      if (d >= 0.0f && closer) {
        h.dist = d;
        h.normal = n;
        h.geom = gi;
        h.slot = slot;
        h.u = u;
        h.v = v;
        h.face = face;
        h.mesh = mesh;
      }
    }
  }
  return h;
}

// True if anything is hit before max_dist (the reference's trace_any).
template <bool kMesh>
__device__ __noinline__ bool any_hit(const MjpbrScene& sc, const float* blk, const BlockLayout& L, const Ray& r, float max_dist,
                    bool cull, int32_t* err) {
  RayInv ri = make_inv(r);
  int32_t st_code[kTlasStack];
  int sp = 1;
  st_code[0] = 0;
  while (sp > 0) {
    --sp;
    int32_t code = st_code[sp];
    int32_t ref = code >> 3, cnt = code & 7;
    if (cnt == 0) {
      const float* nd = blk + L.node_off + ref * kNodeFloats;
      int32_t acnt = __float_as_int(nd[7]), bcnt = __float_as_int(nd[15]);
      float ta = acnt >= 0 ? box_entry(ri, nd[0], nd[1], nd[2], nd[4], nd[5], nd[6], max_dist) : -1.0f;
      float tb = bcnt >= 0 ? box_entry(ri, nd[8], nd[9], nd[10], nd[12], nd[13], nd[14], max_dist) : -1.0f;
      int32_t ca = (__float_as_int(nd[3]) << 3) | acnt;
      int32_t cb = (__float_as_int(nd[11]) << 3) | bcnt;
      int32_t cn = ca, cf = cb;
      float tn = ta, tf = tb;
      if (tb >= 0.0f && (ta < 0.0f || tb < ta)) {
        cn = cb;
        cf = ca;
        tn = tb;
        tf = ta;
      }
      if (tf >= 0.0f) {
        if (sp < kTlasStack) {
          st_code[sp++] = cf;
        } else {
          *err |= kErrStackOverflow;
        }
      }
      if (tn >= 0.0f) {
        if (sp < kTlasStack) {
          st_code[sp++] = cn;
        } else {
          *err |= kErrStackOverflow;
        }
      }
      continue;
    }
    for (int32_t slot = ref; slot < ref + cnt; ++slot) {
      const float* g = blk + L.geom_off + slot * kGeomFloats;
      if (__float_as_int(g[19]) & kGeomFlagSkip) continue;
      V3 n = v3(0.0f);
      float u = 0.0f, v = 0.0f;
      int32_t face = -1, mesh = -1;
      float d = intersect_geom<kMesh, true>(sc, g, r, max_dist, cull, &n, &u, &v, &face, &mesh, err);
      if (cull && d >= 0.0f && dot(r.d, n) > 0.0f) d = -1.0f;
      if (d >= 0.0f && d < max_dist) return true;
    }
  }
  return false;
}

}  // namespace mjpbr
