// Surface evaluation at a hit: base colour, material, shading normal (vertex normals, normal
// maps), ORM / emissive / opacity maps with ray-cone mip selection, and specular anti-aliasing.
// Follows mujoco_warp_pbr/_src/material.py:290-503 (eval_surface) and
// mujoco_warp_pbr/_src/texture.py:104-221 (UV frames). MuJoCo Warp's primitive UV mappings
// (_texture_plane / _sphere_ellipsoid / _cylinder / _capsule / _box, third party) are restated from
// MuJoCo's texture-mapping rules: texuniform repeats per metre, otherwise across the object; +u
// runs along +x and v grows downwards (top-left UV origin).
#pragma once

#include "shading.cuh"
#include "trace.cuh"

namespace mjpbr {

constexpr float kSpecularAaVariance = 0.15f;
constexpr float kSpecularAaThreshold = 0.2f;

struct TexFrame {
  bool has_uv;
  float u, v;
  V3 tangent, bitangent;
  float uv_per_length;
};

MJ_DEV float widen_roughness(float pr, float alpha2_extra) {
  pr = clampf(pr, 0.0f, 1.0f);
  float a2 = fminf(pr * pr * pr * pr + alpha2_extra, 1.0f);
  return sqrtf(sqrtf(a2));
}

// MuJoCo Warp's vertex_normal: the vertex normal unless it is more than ~37 degrees off the face.
MJ_DEV V3 vertex_normal(V3 n, V3 face) {
  V3 nn = normalize(n);
  return dot(nn, face) < 0.8f ? face : nn;
}

// Analytic (unrepeated) UV of a primitive at a local point; *rep receives the repeat factors.
MJ_DEV void primitive_uv(int32_t type, V3 p, V3 ln, V3 size, float rx, float ry, bool uniform, float* u, float* v,
                         float* repx, float* repy) {
  *repx = rx;
  *repy = ry;
  const float inv2pi = 0.5f / kPi;
  switch (type) {
    case MJPBR_GEOM_PLANE:
    case MJPBR_GEOM_HFIELD: {  // a height field maps its texture over its x-y extent like a plane
      float sx = size.x > 0.0f ? size.x : 1.0f, sy = size.y > 0.0f ? size.y : 1.0f;
      if (uniform) {
        *u = p.x;
        *v = -p.y;
      } else {
        *u = p.x / (2.0f * sx) + 0.5f;
        *v = 0.5f - p.y / (2.0f * sy);
      }
      break;
    }
    case MJPBR_GEOM_SPHERE:
    case MJPBR_GEOM_ELLIPSOID: {
      V3 q = type == MJPBR_GEOM_SPHERE ? p / size.x : V3{p.x / size.x, p.y / size.y, p.z / size.z};
      *u = fast_atan2(q.y, q.x) * inv2pi + 0.5f;
      *v = fast_acos(clampf(q.z / fmaxf(length(q), 1.0e-9f), -1.0f, 1.0f)) * (1.0f / kPi);
      if (uniform) {
        *repx = rx * 2.0f * kPi * size.x;
        *repy = ry * kPi * size.x;
      }
      break;
    }
    case MJPBR_GEOM_CYLINDER:
    case MJPBR_GEOM_CAPSULE: {
      float h = size.y;
      *u = fast_atan2(p.y, p.x) * inv2pi + 0.5f;
      *v = 0.5f - p.z / (2.0f * fmaxf(h + (type == MJPBR_GEOM_CAPSULE ? size.x : 0.0f), 1.0e-9f));
      if (uniform) {
        *repx = rx * 2.0f * kPi * size.x;
        *repy = ry * 2.0f * (h + (type == MJPBR_GEOM_CAPSULE ? size.x : 0.0f));
      }
      break;
    }
    default: {  // box: planar mapping of the face the normal points out of
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
        *u = a / (2.0f * fmaxf(sa, 1.0e-9f)) + 0.5f;
        *v = b / (2.0f * fmaxf(sb, 1.0e-9f)) + 0.5f;
      }
      break;
    }
  }
}

MJ_DEV float wrap_delta(float d) { return d - rintf(d); }

// Tangent (dp/du), bitangent (dp/dv) and UV per length from the UV Jacobian on (t1, t2)
// (texture.py:162-176).
MJ_DEV void frame_from_uv_jacobian(V3 t1, V3 t2, float du1, float du2, float dv1, float dv2, TexFrame* f) {
  float det = du1 * dv2 - du2 * dv1;
  float inv = 1.0f / (fabsf(det) > 1.0e-20f ? det : 1.0e-20f);
  f->tangent = (t1 * dv2 - t2 * dv1) * inv;
  f->bitangent = (t2 * du1 - t1 * du2) * inv;
  f->uv_per_length = sqrtf(fabsf(det));
}

// Texture frame of a mesh hit in the mesh frame (texture.py:179-221).
MJ_DEV TexFrame mesh_triangle_frame(const MjpbrScene& s, int32_t mesh, int32_t face, float bu, float bv, float rx,
                                    float ry) {
  TexFrame f;
  f.has_uv = false;
  int32_t tc_adr = s.mesh_texcoordadr ? s.mesh_texcoordadr[mesh] : -1;
  if (tc_adr < 0 || !s.mesh_facetexcoord) return f;
  int32_t fadr = s.mesh_faceadr[mesh] + face;
  int32_t t0 = s.mesh_facetexcoord[fadr * 3], t1 = s.mesh_facetexcoord[fadr * 3 + 1],
          t2 = s.mesh_facetexcoord[fadr * 3 + 2];
  if (t0 < 0 || t1 < 0 || t2 < 0) return f;
  const float* tc = s.mesh_texcoord + (int64_t)tc_adr * 2;
  float u0 = tc[t0 * 2] * rx, v0 = tc[t0 * 2 + 1] * ry;
  float u1 = tc[t1 * 2] * rx, v1 = tc[t1 * 2 + 1] * ry;
  float u2 = tc[t2 * 2] * rx, v2 = tc[t2 * 2 + 1] * ry;
  float bw = 1.0f - bu - bv;
  f.u = u0 * bu + u1 * bv + u2 * bw;
  f.v = v0 * bu + v1 * bv + v2 * bw;
  int32_t vadr = s.mesh_vertadr[mesh];
  const int32_t* fv = s.mesh_face + (int64_t)fadr * 3;
  const float* p0p = s.mesh_vert + (int64_t)(vadr + fv[0]) * 3;
  const float* p1p = s.mesh_vert + (int64_t)(vadr + fv[1]) * 3;
  const float* p2p = s.mesh_vert + (int64_t)(vadr + fv[2]) * 3;
  V3 p0{p0p[0], p0p[1], p0p[2]};
  V3 e1 = V3{p1p[0], p1p[1], p1p[2]} - p0;
  V3 e2 = V3{p2p[0], p2p[1], p2p[2]} - p0;
  float d1u = u1 - u0, d1v = v1 - v0, d2u = u2 - u0, d2v = v2 - v0;
  float det = d1u * d2v - d2u * d1v;
  float inv = 1.0f / (fabsf(det) > 1.0e-20f ? det : 1.0e-20f);
  f.tangent = (e1 * d2v - e2 * d1v) * inv;
  f.bitangent = (e2 * d1u - e1 * d2u) * inv;
  float area = length(cross(e1, e2));
  f.uv_per_length = sqrtf(fabsf(det) / fmaxf(area, 1.0e-20f));
  f.has_uv = true;
  return f;
}

MJ_DEV float4 fetch_role(const MjpbrScene& s, int32_t tex_id, const TexFrame& f, float cone) {
  const MjpbrTexture& t = s.textures[tex_id];
  float lod = texture_lod(cone, f.uv_per_length, t);
  return sample_trilinear(t, s.tex_data, f.u, f.v, fmaxf(lod, 0.0f), true, true);
}

// Surface and viewer-facing shading normal (world frame) at a hit (material.py:301-503).
template <bool kMesh, bool kTex>
__device__ __noinline__ Surface eval_surface(const MjpbrScene& s, const float* blk, const BlockLayout& L, int32_t w, const Hit& hit,
                            int32_t slot, V3 point, V3 dir, float footprint, V3* shading_world) {
  Surface sf;
  sf.occlusion = 1.0f;
  sf.emissive = v3(0.0f);
  const float* g = blk + L.geom_off + slot * kGeomFloats;
  const int32_t gid = hit.geom;
  const int32_t type = __float_as_int(g[3]);
  const int32_t matid = __float_as_int(g[18]);
  // rgba: material colour when the geom keeps the default rgba
  const float* gp = s.geom_rgba.ptr + ((int64_t)(w % s.geom_rgba.nbatch) * s.ngeom + gid) * 4;
  float4 rgba = make_float4(gp[0], gp[1], gp[2], gp[3]);
  if (matid >= 0 && rgba.x == 0.5f && rgba.y == 0.5f && rgba.z == 0.5f && rgba.w == 1.0f && s.mat_rgba.ptr) {
    const float* mp = s.mat_rgba.ptr + ((int64_t)(w % s.mat_rgba.nbatch) * s.nmat + matid) * 4;
    rgba = make_float4(mp[0], mp[1], mp[2], mp[3]);
  }
  sf.base_color = V3{rgba.x, rgba.y, rgba.z};
  sf.alpha = rgba.w;
  sf.metallic = bf(s.geom_metallic, w, s.ngeom, gid);
  sf.roughness = bf(s.geom_roughness, w, s.ngeom, gid);
  sf.reflectance = bf(s.geom_reflectance, w, s.ngeom, gid);
  float emission = (matid >= 0 && s.mat_emission.ptr) ? bf(s.mat_emission, w, s.nmat, matid) : 0.0f;

  GeomFrame fr = geom_frame(g);
  V3 local_dir = mul_t(fr.mat, dir);
  V3 local_normal = mul_t(fr.mat, hit.normal);
  if (dot(local_normal, local_dir) > 0.0f) local_normal = -local_normal;
  V3 shading = local_normal;
  float curvature = 0.0f;
  const bool is_mesh = type == MJPBR_GEOM_MESH || type == MJPBR_GEOM_SDF;
  const bool spec_aa = s.settings.specular_aa != 0;

  if (kMesh && is_mesh && hit.mesh >= 0 && hit.face >= 0 && s.settings.vertex_normals && s.mesh_facenormal) {
    int32_t fadr = s.mesh_faceadr[hit.mesh] + hit.face;
    const int32_t* tri = s.mesh_facenormal + (int64_t)fadr * 3;
    int32_t nadr = s.mesh_normaladr[hit.mesh];
    const float* a = s.mesh_normal + (int64_t)(nadr + tri[0]) * 3;
    const float* b = s.mesh_normal + (int64_t)(nadr + tri[1]) * 3;
    const float* c = s.mesh_normal + (int64_t)(nadr + tri[2]) * 3;
    V3 n0 = vertex_normal(V3{a[0], a[1], a[2]}, local_normal);
    V3 n1 = vertex_normal(V3{b[0], b[1], b[2]}, local_normal);
    V3 n2 = vertex_normal(V3{c[0], c[1], c[2]}, local_normal);
    shading = normalize(n0 * hit.u + n1 * hit.v + n2 * (1.0f - hit.u - hit.v));
    if (dot(shading, local_dir) > 0.0f) shading = -shading;
    if (spec_aa) {
      const int32_t* fv = s.mesh_face + (int64_t)fadr * 3;
      int32_t vadr = s.mesh_vertadr[hit.mesh];
      const float* q0 = s.mesh_vert + (int64_t)(vadr + fv[0]) * 3;
      const float* q1 = s.mesh_vert + (int64_t)(vadr + fv[1]) * 3;
      const float* q2 = s.mesh_vert + (int64_t)(vadr + fv[2]) * 3;
      V3 p0{q0[0], q0[1], q0[2]};
      float edge = sqrtf(length(cross(V3{q1[0], q1[1], q1[2]} - p0, V3{q2[0], q2[1], q2[2]} - p0)));
      float spread = fmaxf(length(n0 - n1), fmaxf(length(n1 - n2), length(n2 - n0)));
      curvature = spread / fmaxf(edge, 1.0e-9f);
    }
  }
  if (spec_aa) {
    if (type == MJPBR_GEOM_SPHERE || type == MJPBR_GEOM_CAPSULE || type == MJPBR_GEOM_CYLINDER) {
      curvature = 1.0f / fmaxf(fr.size.x, 1.0e-9f);
    } else if (type == MJPBR_GEOM_ELLIPSOID) {
      curvature = 1.0f / fmaxf(fminf(fr.size.x, fminf(fr.size.y, fr.size.z)), 1.0e-9f);
    }
  }
  float cone = footprint / fmaxf(fabsf(dot(local_normal, local_dir)), 0.05f);

  if (kTex && s.settings.textures && matid >= 0) {
    int32_t mw = w % s.mat_texid.nbatch;
    const int32_t* texid = s.mat_texid.ptr + ((int64_t)mw * s.nmat + matid) * MJPBR_NTEXROLE;
    const float* rp = s.mat_texrepeat.ptr + ((int64_t)(w % s.mat_texrepeat.nbatch) * s.nmat + matid) * 2;
    bool uniform = s.mat_texuniform.ptr ? bi(s.mat_texuniform, w, s.nmat, matid) != 0 : false;
    TexFrame tf;
    tf.has_uv = false;
    if (kMesh && is_mesh) {
      if (hit.mesh >= 0 && hit.face >= 0) tf = mesh_triangle_frame(s, hit.mesh, hit.face, hit.u, hit.v, rp[0], rp[1]);
    } else {
      V3 local = mul_t(fr.mat, point - fr.pos);
      V3 t1, t2;
      orthonormal_basis(local_normal, &t1, &t2);
      float eps = 1.0e-3f * fmaxf(fmaxf(fr.size.x, fr.size.y), fmaxf(fr.size.z, 1.0e-3f));
      float u0, v0, u1, v1, u2, v2, repx, repy, r1, r2;
      primitive_uv(type, local, local_normal, fr.size, rp[0], rp[1], uniform, &u0, &v0, &repx, &repy);
      primitive_uv(type, local + t1 * eps, local_normal, fr.size, rp[0], rp[1], uniform, &u1, &v1, &r1, &r2);
      primitive_uv(type, local + t2 * eps, local_normal, fr.size, rp[0], rp[1], uniform, &u2, &v2, &r1, &r2);
      float d1u = wrap_delta(u1 - u0) * repx, d1v = wrap_delta(v1 - v0) * repy;
      float d2u = wrap_delta(u2 - u0) * repx, d2v = wrap_delta(v2 - v0) * repy;
      float inv_eps = 1.0f / eps;
      frame_from_uv_jacobian(t1, t2, d1u * inv_eps, d2u * inv_eps, d1v * inv_eps, d2v * inv_eps, &tf);
      tf.u = u0 * repx;
      tf.v = v0 * repy;
      tf.has_uv = true;
    }
    if (tf.has_uv) {
      if (s.settings.base_color_map) {
        int32_t tid = texid[MJPBR_ROLE_RGB] >= 0 ? texid[MJPBR_ROLE_RGB] : texid[MJPBR_ROLE_RGBA];
        if (tid >= 0) {
          float4 t = fetch_role(s, tid, tf, cone);
          sf.base_color = cmul(sf.base_color, V3{t.x, t.y, t.z});
          sf.alpha *= t.w;
        }
      }
      if (s.settings.orm_map) {
        int32_t tid = texid[MJPBR_ROLE_ORM];
        if (tid >= 0) {
          float4 t = fetch_role(s, tid, tf, cone);
          sf.occlusion = t.x;
          sf.roughness *= t.y;
          sf.metallic *= t.z;
        } else {
          tid = texid[MJPBR_ROLE_OCCLUSION];
          if (tid >= 0) sf.occlusion = fetch_role(s, tid, tf, cone).x;
          tid = texid[MJPBR_ROLE_ROUGHNESS];
          if (tid >= 0) sf.roughness *= fetch_role(s, tid, tf, cone).x;
          tid = texid[MJPBR_ROLE_METALLIC];
          if (tid >= 0) sf.metallic *= fetch_role(s, tid, tf, cone).x;
        }
      }
      if (s.settings.opacity_map) {
        int32_t tid = texid[MJPBR_ROLE_OPACITY];
        if (tid >= 0) sf.alpha *= fetch_role(s, tid, tf, cone).x;
      }
      if (s.settings.emissive_map) {
        int32_t tid = texid[MJPBR_ROLE_EMISSIVE];
        if (tid >= 0) {
          float4 t = fetch_role(s, tid, tf, cone);
          sf.emissive = V3{t.x, t.y, t.z} * emission;
          emission = 0.0f;
        }
      }
      if (s.settings.normal_map) {
        int32_t tid = texid[MJPBR_ROLE_NORMAL];
        if (tid >= 0) {
          float4 t = fetch_role(s, tid, tf, cone);
          V3 nts = V3{t.x, t.y, t.z} * 2.0f - v3(1.0f);
          if (spec_aa) {
            float len = clampf(length(nts), 1.0e-3f, 1.0f);
            sf.roughness = widen_roughness(sf.roughness, (1.0f - len) / len);
          }
          V3 tt = tf.tangent - shading * dot(shading, tf.tangent);
          if (length_sq(tt) > 1.0e-20f) {
            tt = normalize(tt);
            V3 bb = cross(shading, tt);
            if (dot(bb, tf.bitangent) > 0.0f) bb = -bb;
            V3 mapped = normalize(tt * nts.x + bb * nts.y + shading * nts.z);
            if (dot(mapped, local_normal) > 0.0f) shading = mapped;
          }
        }
      }
    }
  }
  if (matid >= 0 && emission > 0.0f) sf.emissive = sf.base_color * emission;
  if (spec_aa) {
    float dn = cone * curvature;
    float kernel = fminf(2.0f * kSpecularAaVariance * dn * dn, kSpecularAaThreshold);
    sf.roughness = widen_roughness(sf.roughness, kernel);
  }
  *shading_world = normalize(mul(fr.mat, shading));
  return sf;
}

}  // namespace mjpbr
