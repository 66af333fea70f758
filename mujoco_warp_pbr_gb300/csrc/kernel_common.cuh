// Pieces shared by the render kernels (real-time and path-traced tiers): camera tiles, the pixel
// of a thread, camera rays, the per-world shading context and the depth / segmentation writes.
#pragma once

#include "surface.cuh"

namespace mjpbr {

// Tiles of every rendering camera of a world, in camera order.
struct TileMap {
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
