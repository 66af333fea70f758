// Pieces shared by the render kernels (real-time and path-traced tiers): camera tiles, the pixel
// of a thread, camera rays, the per-world shading context and the depth / segmentation writes.
#pragma once

#include "surface.cuh"

namespace mjpbr {

// Tiles of every rendering camera of a world, in camera order.
struct TileMap {
  int32_t w0;  // first world of the launch (launches cover at most kMaxGridWorlds worlds in grid y)
  int32_t ncam;
  int32_t tile_w, tile_h;
  int32_t tiles_x[MJPBR_MAX_RENDER];
  int32_t tile_base[MJPBR_MAX_RENDER + 1];
};

struct Pixel {
  int32_t cam;     // rendering camera
  int32_t px, py;  // pixel
  int32_t width, height;
  int32_t pixelid;  // row-major within the camera image
  const float* rec;  // camera record in the world block
};

// Camera-frame ray through sub-pixel cell (sx, sy) of a pixel divided into n x n cells (pinhole
// or orthographic; MuJoCo Warp's compute_ray restated with the image plane at z = -1).
MJ_DEV void camera_frame_ray(const Pixel& p, int32_t n, int32_t sx, int32_t sy, V3* dcam, V3* ocam) {
  const float* c = p.rec;
  int32_t ix = p.px * n + sx, iy = p.py * n + sy;
  float u = ((float)ix + 0.5f) / (float)(p.width * n);
  float v = ((float)iy + 0.5f) / (float)(p.height * n);
  int32_t proj = __float_as_int(c[3]);
  float half_h = c[13];
  float aspect = (float)p.width / (float)p.height;
  if (proj == MJPBR_PROJ_ORTHOGRAPHIC) {
    *dcam = V3{0.0f, 0.0f, -1.0f};
    *ocam = V3{(2.0f * u - 1.0f) * (half_h * aspect), (1.0f - 2.0f * v) * half_h, 0.0f};
    return;
  }
  float x, y;
  if (__float_as_int(c[14])) {
    // intrinsics: principal point offset from the sensor centre, focal lengths in sensor units
    x = (u * c[20] - 0.5f * c[20] - c[18]) / c[16];
    y = (0.5f * c[21] - v * c[21] + c[19]) / c[17];
  } else {
    x = (2.0f * u - 1.0f) * (half_h * aspect);
    y = (1.0f - 2.0f * v) * half_h;
  }
  float len = sqrtf(x * x + y * y + 1.0f);
  *dcam = V3{x / len, y / len, -1.0f / len};
  *ocam = v3(0.0f);
}

// ---------------------------------------------------------------- per-pixel ray bundles
// (camera.py:195-296): each pixel of a bundle camera has its own camera-frame ray (rays.py); a
// sub-pixel sample interpolates its four nearest bundle rays, on the image plane z = -1 when all
// four point forward (exact for pinhole bundles), else on the sphere; a zero direction is a pixel
// without a ray.

// Bundle rays x0, x1 and weight t of sample i of n along an axis of nb bundle rays: the sample
// sits at bundle coordinate (i + 0.5) nb / n - 0.5 = num / den, in integers so that t is exactly 0
// on a bundle pixel centre.
MJ_DEV void bundle_axis(int32_t i, int32_t n, int32_t nb, int32_t* x0, int32_t* x1, float* t) {
  const int64_t num = (int64_t)(2 * i + 1) * nb - n;
  const int64_t den = 2 * (int64_t)n;
  int32_t a = (int32_t)((num + den) / den) - 1;  // num + den > 0
  a = min(max(a, 0), max(nb - 2, 0));
  *x0 = a;
  *x1 = min(a + 1, nb - 1);
  *t = (float)(num - (int64_t)a * den) / (float)den;
}

MJ_DEV V3 ray_vec(const float* a, int64_t i) { return V3{a[i * 3], a[i * 3 + 1], a[i * 3 + 2]}; }
MJ_DEV V3 lerp3(V3 a, V3 b, float t) { return a + (b - a) * t; }

// Camera-frame (direction, origin) of the bundle ray through sub-pixel cell (sx, sy) of n x n.
MJ_DEV void bundle_ray(const MjpbrScene& s, const Pixel& p, int32_t n, int32_t sx, int32_t sy, V3* dcam, V3* ocam) {
  const int32_t rw = s.bundle_res[p.cam][0], rh = s.bundle_res[p.cam][1];
  const int64_t adr = s.ray_adr[p.cam];
  int32_t x0, x1, y0, y1;
  float tx, ty;
  bundle_axis(p.px * n + sx, p.width * n, rw, &x0, &x1, &tx);
  bundle_axis(p.py * n + sy, p.height * n, rh, &y0, &y1, &ty);
  const int64_t r0 = adr + (int64_t)y0 * rw, r1 = adr + (int64_t)y1 * rw;
  V3 d00 = ray_vec(s.ray_direction, r0 + x0), d10 = ray_vec(s.ray_direction, r0 + x1);
  V3 d01 = ray_vec(s.ray_direction, r1 + x0), d11 = ray_vec(s.ray_direction, r1 + x1);
  if (length_sq(d00) == 0.0f || length_sq(d10) == 0.0f || length_sq(d01) == 0.0f || length_sq(d11) == 0.0f) {
    // next to a pixel without a ray: the nearest bundle ray, no interpolation
    const int64_t nearest = (ty < 0.5f ? r0 : r1) + (tx < 0.5f ? x0 : x1);
    V3 d = ray_vec(s.ray_direction, nearest);
    if (length_sq(d) > 0.0f) d = normalize(d);
    *dcam = d;
    *ocam = ray_vec(s.ray_origin, nearest);
    return;
  }
  const V3 o00 = ray_vec(s.ray_origin, r0 + x0), o10 = ray_vec(s.ray_origin, r0 + x1);
  const V3 o01 = ray_vec(s.ray_origin, r1 + x0), o11 = ray_vec(s.ray_origin, r1 + x1);
  if (d00.z < 0.0f && d10.z < 0.0f && d01.z < 0.0f && d11.z < 0.0f) {
    d00 = d00 * (-1.0f / d00.z);
    d10 = d10 * (-1.0f / d10.z);
    d01 = d01 * (-1.0f / d01.z);
    d11 = d11 * (-1.0f / d11.z);
  }
  V3 d = lerp3(lerp3(d00, d10, tx), lerp3(d01, d11, tx), ty);
  if (length_sq(d) > 0.0f) d = normalize(d);
  *dcam = d;
  *ocam = lerp3(lerp3(o00, o10, tx), lerp3(o01, o11, tx), ty);
}

// (angle, distance) between bundle rays a and b, or between b and its linear extrapolation.
MJ_DEV void bundle_step(const MjpbrScene& s, int64_t a, int64_t b, bool extrapolate, float* spread, float* width) {
  V3 da = ray_vec(s.ray_direction, a), db = ray_vec(s.ray_direction, b);
  *spread = 0.0f;
  *width = 0.0f;
  if (length_sq(da) == 0.0f || length_sq(db) == 0.0f) return;
  da = normalize(da);
  db = normalize(db);
  *width = length(ray_vec(s.ray_origin, b) - ray_vec(s.ray_origin, a));
  if (!extrapolate) {
    *spread = length(db - da);
  } else if (da.z < 0.0f && db.z < 0.0f) {
    *spread = length(normalize(db * (-2.0f / db.z) + da * (1.0f / da.z)) - db);
  } else {
    *spread = length(normalize(db * 2.0f - da) - db);
  }
}

// Camera-frame ray of sub-pixel cell (sx, sy) of n x n (camera.py:300-330): direction, origin,
// the maximum hit distance (zfar: planar for projections, along the ray for bundles; 0 for a
// bundle pixel without a ray) and the z of the depth axis (depth = distance * -depth_z).
MJ_DEV void primary_ray(const MjpbrScene& s, const Pixel& p, int32_t n, int32_t sx, int32_t sy, V3* dcam, V3* ocam,
                        float* max_dist, float* depth_z) {
  const float zfar = s.settings.zfar;
  if (s.ray_direction) {
    bundle_ray(s, p, n, sx, sy, dcam, ocam);
    *max_dist = zfar > 0.0f ? zfar : kMaxVal;
    if (length_sq(*dcam) == 0.0f) {
      *max_dist = 0.0f;
      *dcam = V3{0.0f, 0.0f, -1.0f};
    }
    *depth_z = -1.0f;
    return;
  }
  camera_frame_ray(p, n, sx, sy, dcam, ocam);
  *max_dist = zfar > 0.0f ? zfar / fmaxf(-dcam->z, 1.0e-6f) : kMaxVal;
  *depth_z = dcam->z;
}

// Angular spread and width (orthographic origins) of one pixel, the ray-cone parameters
// (camera.py:322-347): the difference to the next pixel's ray along x (for bundles, to the next
// bundle ray, or the extrapolation of the previous one in the last column).
MJ_DEV void pixel_cone(const MjpbrScene& s, const Pixel& p, float* spread, float* width) {
  if (s.ray_direction) {
    const int32_t rw = s.bundle_res[p.cam][0], rh = s.bundle_res[p.cam][1];
    *spread = 0.0f;
    *width = 0.0f;
    if (rw < 2) return;
    const int32_t bx = (p.px * rw) / p.width;
    const int64_t b = s.ray_adr[p.cam] + (int64_t)((p.py * rh) / p.height) * rw + bx;
    if (bx + 1 < rw) {
      bundle_step(s, b, b + 1, false, spread, width);
    } else {
      bundle_step(s, b - 1, b, true, spread, width);
    }
    const float scale = (float)rw / (float)p.width;
    *spread *= scale;
    *width *= scale;
    return;
  }
  V3 d0, o0, d1, o1;
  camera_frame_ray(p, 1, 0, 0, &d0, &o0);
  camera_frame_ray(p, 1, 1, 0, &d1, &o1);
  *spread = length(d1 - d0);
  *width = length(o1 - o0);
}

MJ_DEV M3 cam_mat(const float* c) {
  M3 m;
#pragma unroll
  for (int k = 0; k < 9; ++k) m.m[k] = c[4 + k];
  return m;
}

struct RtCtx {
  const MjpbrScene* s;
  const float* blk;
  BlockLayout L;
  int32_t w;
  float exposure;
  V3 ambient;
  int32_t env;
  float env_yaw, env_scale;
  int32_t err;
  Stack st;
};

// MuJoCo reflectance of a slot's material (material.py:543-550), 0 without a material.
MJ_DEV float mirror_reflectance(const RtCtx& c, int32_t slot) {
  int32_t matid = __float_as_int(c.blk[c.L.geom_off + slot * kGeomFloats + 18]);
  if (matid < 0 || !c.s->mat_reflectance.ptr) return 0.0f;
  return bf(c.s->mat_reflectance, c.w, c.s->nmat, matid);
}

// MuJoCo's headlight (lights.py:120-131): directional along the view, no shadow, its illuminance
// display-relative (divided by the world's exposure).
MJ_DEV Light make_headlight(const MjpbrSettings& st, V3 head_dir, float exposure) {
  Light light;
  light.type = MJPBR_LIGHT_DIRECTIONAL;
  light.castshadow = false;
  light.active = true;
  light.dir = head_dir;
  light.diffuse = V3{st.headlight_diffuse[0], st.headlight_diffuse[1], st.headlight_diffuse[2]};
  light.specular = V3{st.headlight_specular[0], st.headlight_specular[1], st.headlight_specular[2]};
  light.attenuation = V3{1.0f, 0.0f, 0.0f};
  light.intensity = st.headlight_intensity / exposure;
  light.range = 1.0f;
  light.bulbradius = 0.0f;
  light.cutoff = 0.0f;
  light.exponent = 0.0f;
  light.pos = v3(0.0f);
  return light;
}

MJ_DEV void write_geometry(const MjpbrScene& s, int32_t w, const Pixel& p, const Hit& hit, float dcam_z) {
  if (s.render_seg[p.cam]) {
    int32_t* o = s.seg_data + ((int64_t)w * s.seg_stride + s.seg_adr[p.cam] + p.pixelid) * 2;
    int2 v = hit.geom != -1 ? make_int2(hit.geom, 5) : make_int2(-1, -1);  // mjOBJ_GEOM
    *reinterpret_cast<int2*>(o) = v;
  }
  if (s.render_depth[p.cam]) {
    s.depth_data[(int64_t)w * s.depth_stride + s.depth_adr[p.cam] + p.pixelid] =
        hit.geom != -1 ? hit.dist * -dcam_z : 0.0f;
  }
}

// Copies world w's block (written by mjpbr_refit_bvh) into shared memory; the caller synchronises.
MJ_DEV void stage_world_block(const MjpbrScene& s, int32_t w, float* blk, int32_t nthreads) {
  const float4* src = reinterpret_cast<const float4*>(s.world_blocks + (int64_t)w * s.world_block_floats);
  float4* dst = reinterpret_cast<float4*>(blk);
  const int32_t n4 = s.world_block_floats >> 2;
  for (int32_t i = threadIdx.x; i < n4; i += nthreads) dst[i] = __ldg(src + i);
}

// The world block a CTA reads: world w's block staged into shared memory at smem (kStaged; the
// caller synchronises before reading), or the block in global memory itself when it does not fit
// in shared memory beside the traversal stacks.
template <bool kStaged>
MJ_DEV const float* world_block_of(const MjpbrScene& s, int32_t w, float* smem, int32_t nthreads) {
  if constexpr (kStaged) {
    stage_world_block(s, w, smem, nthreads);
    return smem;
  } else {
    return s.world_blocks + (int64_t)w * s.world_block_floats;
  }
}

// Per-world shading constants of a context.
MJ_DEV void init_ctx(RtCtx& c, const MjpbrScene& s, const float* blk, const BlockLayout& L, int32_t w, bool tex) {
  c.s = &s;
  c.blk = blk;
  c.L = L;
  c.w = w;
  c.err = 0;
  c.exposure = bf(s.exposure, w, 1, 0);
  c.ambient = bv3(s.ambient_radiance, w, 1, 0);
  c.env = 0;
  c.env_yaw = 0.0f;
  c.env_scale = 0.0f;
  if (tex && s.nenv > 0) {
    c.env = bi(s.env_id, w, 1, 0);
    c.env_yaw = bf(s.env_yaw, w, 1, 0);
    c.env_scale = bf(s.env_intensity, w, 1, 0);
  }
}

}  // namespace mjpbr
