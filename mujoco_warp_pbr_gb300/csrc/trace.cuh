// Closest-hit and any-hit queries of one world: nearest-first traversal of the world's scene BVH
// (nodes in the shared-memory copy of the world block) and, for mesh geoms, of the mesh's BVH in
// global memory in the mesh frame. Semantics follow mujoco_warp_pbr/_src/traverse.py:195-325:
// entry distances are stored with pushed children, a child whose entry is at or beyond the
// current cut-off dist * (1 + tol) + tol_abs is skipped, ties within tol go to the higher geom id,
// hits with a normal along the ray are culled when culling is on, alpha-0 geoms are skipped.
//
// Traversal stack: one per thread in shared memory, entry k of a thread at code[k * stride]
// (consecutive threads in consecutive words: conflict-free), shared by the scene BVH and the mesh
// BVH entered from one of its leaves (the mesh traversal pushes above the scene entries and pops
// back to them). A push that would overflow sets kErrStackOverflow instead of writing.
#pragma once

#include "geometry.cuh"
#include "opcount.cuh"

namespace mjpbr {

// Stack entries per thread of a launch: settings.stack_depth clamped to [8, kStackDepth] (0: the most).
MJ_HD int32_t stack_entries(int32_t requested) {
  return requested <= 0 ? kStackDepth : (requested < 8 ? 8 : (requested > kStackDepth ? kStackDepth : requested));
}

struct Stack {
  int32_t* code;  // (ref << 3) | count, see world_block.cuh
  float* t;       // entry distance of the pushed child
  int32_t stride;
  int32_t cap;    // entries per thread
};

// The stack of thread threadIdx.x among nthreads in shared memory at base (nthreads * cap codes,
// then nthreads * cap distances).
MJ_DEV Stack shared_stack(float* base, int32_t nthreads, int32_t cap) {
  Stack st;
  int32_t* b = reinterpret_cast<int32_t*>(base);
  st.code = b + threadIdx.x;
  st.t = reinterpret_cast<float*>(b + nthreads * cap) + threadIdx.x;
  st.stride = nthreads;
  st.cap = cap;
  return st;
}

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

MJ_DEV void push(const Stack& st, int& sp, int32_t code, float t, int32_t* err) {
  if (sp < st.cap) {
    st.code[sp * st.stride] = code;
    st.t[sp * st.stride] = t;
    ++sp;
  } else {
    *err |= kErrStackOverflow;
  }
}

// Tests both children of a node (child-bounds layout) and pushes the hit ones, far first.
MJ_DEV void expand(const Stack& st, int& sp, const RayInv& ri, float4 alo, float4 ahi, float4 blo, float4 bhi, float cut,
                   int32_t* err) {
  const int32_t acnt = __float_as_int(ahi.w), bcnt = __float_as_int(bhi.w);
  if (acnt >= 0) MJPBR_COUNT(kOpBox);
  if (bcnt >= 0) MJPBR_COUNT(kOpBox);
  const float ta = acnt >= 0 ? box_entry(ri, alo.x, alo.y, alo.z, ahi.x, ahi.y, ahi.z, cut) : -1.0f;
  const float tb = bcnt >= 0 ? box_entry(ri, blo.x, blo.y, blo.z, bhi.x, bhi.y, bhi.z, cut) : -1.0f;
  const int32_t ca = (__float_as_int(alo.w) << 3) | acnt;
  const int32_t cb = (__float_as_int(blo.w) << 3) | bcnt;
  const bool swap = tb >= 0.0f && (ta < 0.0f || tb < ta);
  const int32_t cn = swap ? cb : ca, cf = swap ? ca : cb;
  const float tn = swap ? tb : ta, tf = swap ? ta : tb;
  if (tf >= 0.0f) push(st, sp, cf, tf, err);
  if (tn >= 0.0f) push(st, sp, cn, tn, err);
}

// Closest (or, with `any`, any) triangle of mesh `mesh` hit by the local ray in [0, tmax),
// using stack entries above sp0. Returns the distance or -1; on a closest hit fills the local
// geometric normal and the barycentrics of vertices 0 and 1. Any-hit queries do not cull.
MJ_DEV float mesh_query(const MjpbrScene& sc, const Stack& st, int sp0, int32_t mesh, V3 lo, V3 ld, float tmax,
                        bool cull, bool any, V3* n_local, float* bu, float* bv, int32_t* face, int32_t* err) {
  const float* nodes = sc.blas_nodes + (int64_t)sc.blas_root[mesh] * kNodeFloats;
  const float* tris = sc.blas_tris + (int64_t)sc.blas_tri_base[mesh] * kTriFloats;
  const WoopRay w = woop_setup(lo, ld);
  const RayInv ri = make_inv(Ray{lo, ld});
  float best = tmax;
  int32_t found = -1;
  V3 nb = v3(0.0f);
  float ub = 0.0f, vb = 0.0f;
  int sp = sp0;
  push(st, sp, 0, 0.0f, err);  // the root node
  while (sp > sp0) {
    --sp;
    if (st.t[sp * st.stride] >= best) continue;
    const int32_t code = st.code[sp * st.stride];
    const int32_t ref = code >> 3, cnt = code & 7;
    if (cnt == 0) {
      const float* nd = nodes + (int64_t)ref * kNodeFloats;
      expand(st, sp, ri, ldg4(nd), ldg4(nd + 4), ldg4(nd + 8), ldg4(nd + 12), best, err);
      continue;
    }
    for (int32_t i = ref; i < ref + cnt; ++i) {
      const float* tr = tris + (int64_t)i * kTriFloats;
      const float4 a = ldg4(tr), b = ldg4(tr + 4), c = ldg4(tr + 8);
      const V3 v0{a.x, a.y, a.z}, v1{b.x, b.y, b.z}, v2{c.x, c.y, c.z};
      float u, v;
      MJPBR_COUNT(kOpTri);
      const float t = woop_hit(w, v0, v1, v2, best, &u, &v);
      if (t < 0.0f) continue;
      if (any) return t;
      const V3 ng = cross(v1 - v0, v2 - v0);
      if (cull && dot(ld, ng) > 0.0f) continue;
      best = t;
      found = __float_as_int(a.w);
      nb = ng;
      ub = u;
      vb = v;
    }
  }
  if (found < 0) return -1.0f;
  *n_local = normalize(nb);
  *bu = ub;
  *bv = vb;
  *face = found;
  return best;
}

// One geom against the ray: distance (or -1), world normal, mesh hit details. Height fields are
// traced as meshes (the reference's traverse.py:161-164 queries MuJoCo Warp's height-field mesh BVH).
template <bool kMesh>
MJ_DEV float intersect_geom(const MjpbrScene& sc, const Stack& st, int sp, const float* g, const Ray& r, float max_t,
                            bool cull, bool any, V3* n, float* u, float* v, int32_t* face, int32_t* mesh, int32_t* err) {
  const int32_t type = __float_as_int(g[3]);
  const GeomFrame f = geom_frame(g);
  float d = -1.0f;
  switch (type) {
    case MJPBR_GEOM_PLANE:
      MJPBR_COUNT(kOpPlane);
      d = ray_plane(f, r, n);
      break;
    case MJPBR_GEOM_SPHERE:
      MJPBR_COUNT(kOpSphere);
      d = ray_sphere(f, r, n);
      break;
    case MJPBR_GEOM_ELLIPSOID:
      MJPBR_COUNT(kOpEllipsoid);
      d = ray_ellipsoid(f, r, n);
      break;
    case MJPBR_GEOM_CAPSULE:
      MJPBR_COUNT(kOpCapsule);
      d = ray_capsule(f, r, n);
      break;
    case MJPBR_GEOM_CYLINDER:
      MJPBR_COUNT(kOpCylinder);
      d = ray_cylinder(f, r, n);
      break;
    case MJPBR_GEOM_BOX:
      MJPBR_COUNT(kOpBoxPrim);
      d = ray_box(f, r, n);
      break;
    default:
      if (kMesh && (type == MJPBR_GEOM_MESH || type == MJPBR_GEOM_SDF || type == MJPBR_GEOM_HFIELD)) {
        const int32_t mid = __float_as_int(g[17]);  // triangle BVH (a height field's follows the meshes')
        if (mid >= 0) {
          V3 lo, ld, nl = v3(0.0f);
          map_local(f, r, &lo, &ld);
          d = mesh_query(sc, st, sp, mid, lo, ld, max_t, cull, any, &nl, u, v, face, err);
          *n = any ? v3(0.0f) : mul(f.mat, nl);
          *mesh = mid;
        }
      }
      break;
  }
  return d;
}

// The ray query of the render kernels, one copy in the binary for every call site:
//  * any = false: closest hit within max_dist (the reference's trace_closest);
//  * any = true: the first hit found before max_dist (trace_any; hit.geom != -1 means occluded).
template <bool kMesh>
__device__ __noinline__ Hit trace_ray(const MjpbrScene& sc, const Stack& st, const float* blk, const BlockLayout& L,
                                      const Ray r, float max_dist, bool cull, bool any, int32_t* err) {
  Hit h;
  h.geom = -1;
  h.slot = -1;
  h.dist = max_dist;
  h.normal = v3(0.0f);
  h.u = 0.0f;
  h.v = 0.0f;
  h.face = -1;
  h.mesh = -1;
  if (any) {
    MJPBR_COUNT(kOpRayAny);
  } else {
    MJPBR_COUNT(kOpRayClosest);
  }
  const RayInv ri = make_inv(r);
  int sp = 0;
  push(st, sp, 0, 0.0f, err);
  while (sp > 0) {
    --sp;
    float cut = h.dist * (1.0f + kRayTolRel) + kRayTolAbs;
    if (st.t[sp * st.stride] >= cut) continue;
    const int32_t code = st.code[sp * st.stride];
    const int32_t ref = code >> 3, cnt = code & 7;
    if (cnt == 0) {
      const float4* nd = reinterpret_cast<const float4*>(blk + L.node_off + ref * kNodeFloats);
      expand(st, sp, ri, nd[0], nd[1], nd[2], nd[3], cut, err);
      continue;
    }
    for (int32_t slot = ref; slot < ref + cnt; ++slot) {
      const float* g = blk + L.geom_off + slot * kGeomFloats;
      if (__float_as_int(g[19]) & kGeomFlagSkip) continue;
      cut = h.dist * (1.0f + kRayTolRel) + kRayTolAbs;
      V3 n = v3(0.0f);
      float u = 0.0f, v = 0.0f;
      int32_t face = -1, mesh = -1;
      float d = intersect_geom<kMesh>(sc, st, sp, g, r, any ? max_dist : cut, cull, any, &n, &u, &v, &face, &mesh, err);
      if (cull && d >= 0.0f && dot(r.d, n) > 0.0f) d = -1.0f;
      const int32_t gi = __float_as_int(g[16]);
      if (any) {
        if (d >= 0.0f && d < max_dist) {
          h.geom = gi;
          h.slot = slot;
          h.dist = d;
          return h;
        }
        continue;
      }
      const float tol = kRayTolRel * fmaxf(h.dist, 1.0f);
      const bool closer = (d < h.dist - tol) || (fabsf(d - h.dist) <= tol && (h.geom < 0 || gi > h.geom));
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

// Primitive geom g (plane, sphere, ellipsoid, capsule, cylinder, box) against the ray: distance or -1,
// world normal in *n; -1 for the geoms traced through a triangle BVH.
MJ_DEV float intersect_primitive(const float* g, const Ray& r, V3* n) {
  const GeomFrame f = geom_frame(g);
  switch (__float_as_int(g[3])) {
    case MJPBR_GEOM_PLANE:
      MJPBR_COUNT(kOpPlane);
      return ray_plane(f, r, n);
    case MJPBR_GEOM_SPHERE:
      MJPBR_COUNT(kOpSphere);
      return ray_sphere(f, r, n);
    case MJPBR_GEOM_ELLIPSOID:
      MJPBR_COUNT(kOpEllipsoid);
      return ray_ellipsoid(f, r, n);
    case MJPBR_GEOM_CAPSULE:
      MJPBR_COUNT(kOpCapsule);
      return ray_capsule(f, r, n);
    case MJPBR_GEOM_CYLINDER:
      MJPBR_COUNT(kOpCylinder);
      return ray_cylinder(f, r, n);
    case MJPBR_GEOM_BOX:
      MJPBR_COUNT(kOpBoxPrim);
      return ray_box(f, r, n);
    default:
      return -1.0f;
  }
}

// Triangle BVH of geom g (a mesh's, an SDF's mesh or a height field's), -1 for none.
MJ_DEV int32_t geom_bvh(const float* g) {
  const int32_t type = __float_as_int(g[3]);
  if (type != MJPBR_GEOM_MESH && type != MJPBR_GEOM_SDF && type != MJPBR_GEOM_HFIELD) return -1;
  return __float_as_int(g[17]);
}

// Any-hit query as a resumable state machine, for persistent kernels whose lanes take a new ray
// as soon as their last one is done instead of waiting for the warp's slowest ray: any_begin sets
// up the ray, any_step advances it by one step (a scene node, one geom of a scene leaf, a mesh node
// or a mesh leaf) and returns kAnyRunning, kAnyClear (no hit before max_dist) or kAnyHit. The
// tests and their order are trace_ray's with any = true, step for step (including the op counts).
constexpr int32_t kAnyRunning = 0, kAnyClear = 1, kAnyHit = 2;

struct AnyQuery {
  Ray r;
  RayInv ri;
  float max_dist, cut;
  int32_t sp, leaf, leaf_end;
  int32_t m_base;  // the mesh traversal's stack base while a mesh is being traced, else -1
  const float* m_nodes;
  const float* m_tris;
  WoopRay m_w;
  RayInv m_ri;
};

MJ_DEV void any_begin(AnyQuery& q, const Stack& st, const Ray& r, float max_dist, int32_t* err) {
  MJPBR_COUNT(kOpRayAny);
  q.r = r;
  q.ri = make_inv(r);
  q.max_dist = max_dist;
  q.cut = max_dist * (1.0f + kRayTolRel) + kRayTolAbs;
  q.sp = 0;
  q.leaf = q.leaf_end = 0;
  q.m_base = -1;
  push(st, q.sp, 0, 0.0f, err);
}

template <bool kMesh>
MJ_DEV int32_t any_step(AnyQuery& q, const MjpbrScene& sc, const Stack& st, const float* blk, const BlockLayout& L, bool cull,
                        int32_t* err) {
  if (kMesh && q.m_base >= 0) {
    if (q.sp == q.m_base) {  // the mesh is done without a hit
      q.m_base = -1;
      return kAnyRunning;
    }
    --q.sp;
    if (st.t[q.sp * st.stride] >= q.max_dist) return kAnyRunning;
    const int32_t code = st.code[q.sp * st.stride];
    const int32_t ref = code >> 3, cnt = code & 7;
    if (cnt == 0) {
      const float* nd = q.m_nodes + (int64_t)ref * kNodeFloats;
      expand(st, q.sp, q.m_ri, ldg4(nd), ldg4(nd + 4), ldg4(nd + 8), ldg4(nd + 12), q.max_dist, err);
      return kAnyRunning;
    }
    for (int32_t i = ref; i < ref + cnt; ++i) {
      const float* tr = q.m_tris + (int64_t)i * kTriFloats;
      const float4 a = ldg4(tr), b = ldg4(tr + 4), c = ldg4(tr + 8);
      float tu, tv;
      MJPBR_COUNT(kOpTri);
      if (woop_hit(q.m_w, V3{a.x, a.y, a.z}, V3{b.x, b.y, b.z}, V3{c.x, c.y, c.z}, q.max_dist, &tu, &tv) >= 0.0f) return kAnyHit;
    }
    return kAnyRunning;
  }
  if (q.leaf < q.leaf_end) {  // the next geom of the scene leaf
    const float* g = blk + L.geom_off + (q.leaf++) * kGeomFloats;
    if (__float_as_int(g[19]) & kGeomFlagSkip) return kAnyRunning;
    const int32_t bvh = kMesh ? geom_bvh(g) : -1;
    if (bvh >= 0) {  // trace the mesh from the next steps, its entries above the scene's
      V3 lo, ld;
      map_local(geom_frame(g), q.r, &lo, &ld);
      q.m_nodes = sc.blas_nodes + (int64_t)sc.blas_root[bvh] * kNodeFloats;
      q.m_tris = sc.blas_tris + (int64_t)sc.blas_tri_base[bvh] * kTriFloats;
      q.m_w = woop_setup(lo, ld);
      q.m_ri = make_inv(Ray{lo, ld});
      q.m_base = q.sp;
      push(st, q.sp, 0, 0.0f, err);
      return kAnyRunning;
    }
    V3 n = v3(0.0f);
    float d = intersect_primitive(g, q.r, &n);
    if (cull && d >= 0.0f && dot(q.r.d, n) > 0.0f) d = -1.0f;
    return (d >= 0.0f && d < q.max_dist) ? kAnyHit : kAnyRunning;
  }
  if (q.sp == 0) return kAnyClear;
  --q.sp;
  if (st.t[q.sp * st.stride] >= q.cut) return kAnyRunning;
  const int32_t code = st.code[q.sp * st.stride];
  const int32_t ref = code >> 3, cnt = code & 7;
  if (cnt == 0) {
    const float4* nd = reinterpret_cast<const float4*>(blk + L.node_off + ref * kNodeFloats);
    expand(st, q.sp, q.ri, nd[0], nd[1], nd[2], nd[3], q.cut, err);
  } else {
    q.leaf = ref;
    q.leaf_end = ref + cnt;
  }
  return kAnyRunning;
}

// Closest-hit query as a resumable state machine (the persistent refill kernels' counterpart of
// trace_ray with any = false): closest_begin sets up the ray, closest_step advances it by one step
// and returns kAnyRunning until the query is done (kAnyClear), the best hit in q.h. The tests, their
// order and the hit selection (tolerance, tie-break to the higher geom id, culling) are
// trace_ray's, step for step.
struct ClosestQuery {
  Ray r;
  RayInv ri;
  Hit h;
  int32_t sp, leaf, leaf_end;
  int32_t m_slot, m_bvh, m_base, m_face;  // the mesh geom being traced (m_slot -1: none)
  const float* m_nodes;
  const float* m_tris;
  WoopRay m_w;
  RayInv m_ri;
  V3 m_ld, m_n;
  float m_best, m_u, m_v;
};

MJ_DEV void closest_begin(ClosestQuery& q, const Stack& st, const Ray& r, float max_dist, int32_t* err) {
  MJPBR_COUNT(kOpRayClosest);
  q.r = r;
  q.ri = make_inv(r);
  q.h.geom = -1;
  q.h.slot = -1;
  q.h.dist = max_dist;
  q.h.normal = v3(0.0f);
  q.h.u = q.h.v = 0.0f;
  q.h.face = -1;
  q.h.mesh = -1;
  q.sp = 0;
  q.leaf = q.leaf_end = 0;
  q.m_slot = -1;
  push(st, q.sp, 0, 0.0f, err);
}

// A geom's hit (d >= 0) against the best so far (trace_ray's selection).
MJ_DEV void closest_offer(ClosestQuery& q, const float* g, int32_t slot, float d, V3 n, float u, float v, int32_t face, int32_t mesh,
                          bool cull) {
  if (cull && d >= 0.0f && dot(q.r.d, n) > 0.0f) d = -1.0f;
  const int32_t gi = __float_as_int(g[16]);
  const float tol = kRayTolRel * fmaxf(q.h.dist, 1.0f);
  const bool closer = (d < q.h.dist - tol) || (fabsf(d - q.h.dist) <= tol && (q.h.geom < 0 || gi > q.h.geom));
  if (d >= 0.0f && closer) {
    q.h.dist = d;
    q.h.normal = n;
    q.h.geom = gi;
    q.h.slot = slot;
    q.h.u = u;
    q.h.v = v;
    q.h.face = face;
    q.h.mesh = mesh;
  }
}

template <bool kMesh>
MJ_DEV int32_t closest_step(ClosestQuery& q, const MjpbrScene& sc, const Stack& st, const float* blk, const BlockLayout& L, bool cull,
                            int32_t* err) {
  const bool in_mesh = kMesh && q.m_slot >= 0;
  if (!in_mesh && q.leaf < q.leaf_end) {  // the next geom of the scene leaf
    const int32_t slot = q.leaf++;
    const float* g = blk + L.geom_off + slot * kGeomFloats;
    if (__float_as_int(g[19]) & kGeomFlagSkip) return kAnyRunning;
    const int32_t bvh = kMesh ? geom_bvh(g) : -1;
    if (bvh >= 0) {  // trace the mesh from the next steps, its entries above the scene's
      V3 lo;
      map_local(geom_frame(g), q.r, &lo, &q.m_ld);
      q.m_nodes = sc.blas_nodes + (int64_t)sc.blas_root[bvh] * kNodeFloats;
      q.m_tris = sc.blas_tris + (int64_t)sc.blas_tri_base[bvh] * kTriFloats;
      q.m_w = woop_setup(lo, q.m_ld);
      q.m_ri = make_inv(Ray{lo, q.m_ld});
      q.m_best = q.h.dist * (1.0f + kRayTolRel) + kRayTolAbs;
      q.m_face = -1;
      q.m_n = v3(0.0f);
      q.m_u = q.m_v = 0.0f;
      q.m_slot = slot;
      q.m_bvh = bvh;
      q.m_base = q.sp;
      push(st, q.sp, 0, 0.0f, err);
      return kAnyRunning;
    }
    V3 n = v3(0.0f);
    const float d = intersect_primitive(g, q.r, &n);
    closest_offer(q, g, slot, d, n, 0.0f, 0.0f, -1, -1, cull);
    return kAnyRunning;
  }
  if (in_mesh && q.sp == q.m_base) {  // the mesh is done: its hit goes through the primitives' selection
    const int32_t slot = q.m_slot;
    q.m_slot = -1;
    const float* g = blk + L.geom_off + slot * kGeomFloats;
    if (q.m_face >= 0) {
      closest_offer(q, g, slot, q.m_best, mul(geom_frame(g).mat, normalize(q.m_n)), q.m_u, q.m_v, q.m_face, q.m_bvh, cull);
    }
    return kAnyRunning;
  }
  if (!in_mesh && q.sp == 0) return kAnyClear;
  // one entry of the current level's stack; scene and mesh nodes share the child-bounds layout,
  // so lanes at either level expand their node with the same instructions
  --q.sp;
  const float cut = in_mesh ? q.m_best : q.h.dist * (1.0f + kRayTolRel) + kRayTolAbs;
  if (st.t[q.sp * st.stride] >= cut) return kAnyRunning;
  const int32_t code = st.code[q.sp * st.stride];
  const int32_t ref = code >> 3, cnt = code & 7;
  if (cnt == 0) {
    const float4* nd = reinterpret_cast<const float4*>(in_mesh ? q.m_nodes + (int64_t)ref * kNodeFloats : blk + L.node_off + ref * kNodeFloats);
    RayInv ri;  // component copies: a selected reference would put the query in local memory
    ri.inv = in_mesh ? q.m_ri.inv : q.ri.inv;
    ri.oinv = in_mesh ? q.m_ri.oinv : q.ri.oinv;
    expand(st, q.sp, ri, nd[0], nd[1], nd[2], nd[3], cut, err);
    return kAnyRunning;
  }
  if (in_mesh) {
    for (int32_t i = ref; i < ref + cnt; ++i) {
      const float* tr = q.m_tris + (int64_t)i * kTriFloats;
      const float4 a = ldg4(tr), b = ldg4(tr + 4), c = ldg4(tr + 8);
      const V3 v0{a.x, a.y, a.z}, v1{b.x, b.y, b.z}, v2{c.x, c.y, c.z};
      float tu, tv;
      MJPBR_COUNT(kOpTri);
      const float t = woop_hit(q.m_w, v0, v1, v2, q.m_best, &tu, &tv);
      if (t < 0.0f) continue;
      const V3 ng = cross(v1 - v0, v2 - v0);
      if (cull && dot(q.m_ld, ng) > 0.0f) continue;
      q.m_best = t;
      q.m_face = __float_as_int(a.w);
      q.m_n = ng;
      q.m_u = tu;
      q.m_v = tv;
    }
    return kAnyRunning;
  }
  q.leaf = ref;
  q.leaf_end = ref + cnt;
  return kAnyRunning;
}

}  // namespace mjpbr
