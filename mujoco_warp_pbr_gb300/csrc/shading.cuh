// Shading of the render kernels: Filament's BRDF, punctual lights, tone mapping and sRGB
// encoding, software-filtered textures (bilinear / trilinear with the CUDA texture unit's
// addressing conventions, exact float weights), the DFG table and the environment lookups.
//
// Reference formulas (julien-blanchon/mujoco_warp_pbr):
//   BRDF            mujoco_warp_pbr/_src/brdf.py:32-110
//   lobes           mujoco_warp_pbr/_src/material.py:506-550
//   lights          mujoco_warp_pbr/_src/lights.py:151-198
//   colour          mujoco_warp_pbr/_src/color.py:40-119
//   environment     mujoco_warp_pbr/_src/envmap.py:154-168,252-303
//   DFG lookup      mujoco_warp_pbr/_src/ibl.py:117-119
//   texture LOD     mujoco_warp_pbr/_src/texture.py:225-233
#pragma once

#include "common.cuh"
#include "world_block.cuh"

namespace mjpbr {

constexpr float kMinPerceptualRoughness = 0.045f;

// ---------------------------------------------------------------- BRDF (Filament)

MJ_DEV float d_ggx(float noh, float alpha) {
  float a2 = alpha * alpha;
  float f = (noh * a2 - noh) * noh + 1.0f;
  return a2 / (kPi * f * f);
}

MJ_DEV float v_smith_ggx_correlated(float nov, float nol, float alpha) {
  float a2 = alpha * alpha;
  float gv = nol * sqrtf(nov * nov * (1.0f - a2) + a2);
  float gl = nov * sqrtf(nol * nol * (1.0f - a2) + a2);
  return 0.5f / (gv + gl);
}

MJ_DEV V3 f_schlick(V3 f0, float f90, float voh) {
  float x = 1.0f - voh;
  float x2 = x * x;
  float fc = x2 * x2 * x;
  return f0 * (1.0f - fc) + v3(f90 * fc);
}

MJ_DEV V3 specular_lobe(V3 f0, float alpha, float noh, float nov, float nol, float loh) {
  return f_schlick(f0, 1.0f, loh) * (d_ggx(noh, alpha) * v_smith_ggx_correlated(nov, nol, alpha));
}

struct Surface {
  V3 base_color;
  float alpha;
  float metallic;
  float roughness;  // perceptual
  float reflectance;
  V3 emissive;
  float occlusion;
};

struct Lobes {
  float pr;     // clamped perceptual roughness
  float alpha;  // pr^2
  V3 f0;
  V3 energy_comp;
  V3 spec_albedo;
  V3 diffuse_color;
};

// ---------------------------------------------------------------- filtered table lookups

// Bilinear sample of a (h, w, 2) float table at normalised (x, y) with clamp addressing and
// texel-centre coordinates (x * w - 0.5), as a CLAMP / LINEAR CUDA texture with exact weights.
MJ_DEV void sample_dfg(const float* lut, int32_t n, float nov, float pr, float* dx, float* dy) {
  float fx = nov * (float)n - 0.5f;
  float fy = pr * (float)n - 0.5f;
  float x0f = floorf(fx), y0f = floorf(fy);
  float tx = fx - x0f, ty = fy - y0f;
  int x0 = (int)x0f, y0 = (int)y0f;
  int x1 = min(max(x0 + 1, 0), n - 1), y1 = min(max(y0 + 1, 0), n - 1);
  x0 = min(max(x0, 0), n - 1);
  y0 = min(max(y0, 0), n - 1);
  float2 a = __ldg(reinterpret_cast<const float2*>(lut) + (y0 * n + x0));
  float2 b = __ldg(reinterpret_cast<const float2*>(lut) + (y0 * n + x1));
  float2 c = __ldg(reinterpret_cast<const float2*>(lut) + (y1 * n + x0));
  float2 d = __ldg(reinterpret_cast<const float2*>(lut) + (y1 * n + x1));
  float ax = a.x + (b.x - a.x) * tx, ay = a.y + (b.y - a.y) * tx;
  float cx = c.x + (d.x - c.x) * tx, cy = c.y + (d.y - c.y) * tx;
  *dx = ax + (cx - ax) * ty;
  *dy = ay + (cy - ay) * ty;
}

MJ_DEV Lobes shading_lobes(const float* dfg, int32_t dfg_size, const Surface& s, float nov) {
  Lobes l;
  l.pr = clampf(s.roughness, kMinPerceptualRoughness, 1.0f);
  l.alpha = l.pr * l.pr;
  float diel = 0.16f * s.reflectance * s.reflectance * (1.0f - s.metallic);
  l.f0 = s.base_color * s.metallic + v3(diel);
  float dx, dy;
  sample_dfg(dfg, dfg_size, nov, l.pr, &dx, &dy);
  l.energy_comp = v3(1.0f) + l.f0 * (1.0f / fmaxf(dy, 1.0e-4f) - 1.0f);
  l.spec_albedo = (v3(1.0f) - l.f0) * dx + l.f0 * dy;
  l.diffuse_color = cmul(s.base_color * (1.0f - s.metallic), v3(1.0f) - l.spec_albedo);
  return l;
}

// ---------------------------------------------------------------- lights

struct Light {
  int32_t type;
  bool castshadow;
  bool active;
  V3 pos, dir, diffuse, specular, attenuation;
  float intensity, range, bulbradius, cutoff, exponent;
};

MJ_DEV Light load_light(const float* p) {
  Light l;
  l.pos = V3{p[0], p[1], p[2]};
  l.type = __float_as_int(p[3]);
  l.dir = V3{p[4], p[5], p[6]};
  int32_t flags = __float_as_int(p[7]);
  l.castshadow = (flags & kLightFlagCastShadow) != 0;
  l.active = (flags & kLightFlagActive) != 0;
  l.diffuse = V3{p[8], p[9], p[10]};
  l.intensity = p[11];
  l.specular = V3{p[12], p[13], p[14]};
  l.range = p[15];
  l.attenuation = V3{p[16], p[17], p[18]};
  l.bulbradius = p[19];
  l.cutoff = p[20];
  l.exponent = p[21];
  return l;
}

// Direction to the light (plain arithmetic: it feeds shadow rays), distance and the diffuse /
// specular radiance scales (zero: the light does not reach the point).
MJ_DEV void eval_light(const Light& light, int32_t light_model, V3 point, V3* l, float* dist, V3* dscale,
                       V3* sscale) {
  bool physical = light_model == MJPBR_LIGHT_MODEL_PHYSICAL;
  float att = 1.0f;
  *dist = 1.0e10f;
  if (light.type == MJPBR_LIGHT_DIRECTIONAL) {
    *l = -light.dir;
  } else {
    V3 to = light.pos - point;
    *dist = length(to);
    *l = to / fmaxf(*dist, 1.0e-9f);
    float d = *dist;
    if (physical) {
      float d2 = d * d;
      float r = fmaxf(light.range, 1.0e-6f);
      float factor = d2 / (r * r);
      float window = clampf(1.0f - factor * factor, 0.0f, 1.0f);
      att = window * window / fmaxf(d2, 1.0e-4f);
    } else {
      att = 1.0f / fmaxf(light.attenuation.x + light.attenuation.y * d + light.attenuation.z * d * d, 1.0e-9f);
    }
    if (light.type == MJPBR_LIGHT_SPOT) {
      float cos_theta = dot(-*l, light.dir);
      float outer = light.cutoff * (kPi / 180.0f);
      float cos_outer = __cosf(outer);
      if (physical) {
        float cos_inner = __cosf(outer * 0.75f);
        float cone_scale = 1.0f / fmaxf(cos_inner - cos_outer, 1.0f / 1024.0f);
        float s = clampf((cos_theta - cos_outer) * cone_scale, 0.0f, 1.0f);
        att = att * s * s;
      } else {
        att = cos_theta < cos_outer ? 0.0f : att * fast_pow(fmaxf(cos_theta, 0.0f), light.exponent);
      }
    }
  }
  if (physical) {
    V3 s = light.diffuse * (light.intensity * att);
    *dscale = s;
    *sscale = s;
  } else {
    float k = kPi * att;
    *dscale = light.diffuse * k;
    *sscale = light.specular * k;
  }
}

// ---------------------------------------------------------------- colour


MJ_DEV V3 tonemap_pbr_neutral(V3 c) {
  const float start = 0.8f - 0.04f;
  const float desat = 0.15f;
  float x = fminf(c.x, fminf(c.y, c.z));
  float offset = x < 0.08f ? x - 6.25f * x * x : 0.04f;
  c = c - v3(offset);
  float peak = fmaxf(c.x, fmaxf(c.y, c.z));
  if (peak < start) return c;
  float d = 1.0f - start;
  float new_peak = 1.0f - d * d / (peak + d - start);
  c = c * (new_peak / peak);
  float g = 1.0f - 1.0f / (desat * (peak - new_peak) + 1.0f);
  return c * (1.0f - g) + v3(new_peak * g);
}

MJ_DEV V3 tonemap_aces(V3 c) {
  V3 v = V3{0.59719f * c.x + 0.35458f * c.y + 0.04823f * c.z, 0.07600f * c.x + 0.90834f * c.y + 0.01566f * c.z,
            0.02840f * c.x + 0.13383f * c.y + 0.83777f * c.z};
  V3 num = cmul(v, v + v3(0.0245786f)) - v3(0.000090537f);
  V3 den = cmul(v, v * 0.983729f + v3(0.4329510f)) + v3(0.238081f);
  v = V3{num.x / den.x, num.y / den.y, num.z / den.z};
  return V3{1.60475f * v.x - 0.53108f * v.y - 0.07367f * v.z, -0.10208f * v.x + 1.10813f * v.y - 0.00605f * v.z,
            -0.00327f * v.x - 0.07276f * v.y + 1.07602f * v.z};
}

// Exposed linear HDR -> tone-mapped linear [0, 1] (averaged over sub-pixel samples, then encoded).
MJ_DEV V3 display_transform(V3 c, int32_t tone_mapper) {
  c = vmax(c, v3(0.0f));
  if (tone_mapper == MJPBR_TONE_PBR_NEUTRAL) {
    c = tonemap_pbr_neutral(c);
  } else if (tone_mapper == MJPBR_TONE_ACES) {
    c = tonemap_aces(c);
  }
  return vmin(vmax(c, v3(0.0f)), v3(1.0f));
}

MJ_DEV float srgb_oetf(float x) { return x <= 0.0031308f ? 12.92f * x : 1.055f * fast_pow(x, 1.0f / 2.4f) - 0.055f; }

// Display-linear [0, 1] -> 8-bit sRGB RGBA packed with R in the low byte (round half up).
MJ_DEV uint32_t encode_display(V3 c) {
  uint32_t r = (uint32_t)(srgb_oetf(c.x) * 255.0f + 0.5f);
  uint32_t g = (uint32_t)(srgb_oetf(c.y) * 255.0f + 0.5f);
  uint32_t b = (uint32_t)(srgb_oetf(c.z) * 255.0f + 0.5f);
  return (255u << 24) | (b << 16) | (g << 8) | r;
}

// ---------------------------------------------------------------- textures

MJ_DEV float4 fetch_texel(const MjpbrTexture& t, const uint8_t* data, int level, int w, int x, int y) {
  int64_t idx = (int64_t)y * w + x;
  if (t.format == MJPBR_TEX_RGBA8) {
    uchar4 c = __ldg(reinterpret_cast<const uchar4*>(data + t.level_offset[level]) + idx);
    return make_float4(c.x * (1.0f / 255.0f), c.y * (1.0f / 255.0f), c.z * (1.0f / 255.0f), c.w * (1.0f / 255.0f));
  }
  uint2 raw = __ldg(reinterpret_cast<const uint2*>(data + t.level_offset[level]) + idx);
  __half2 lo = *reinterpret_cast<__half2*>(&raw.x);
  __half2 hi = *reinterpret_cast<__half2*>(&raw.y);
  float2 a = __half22float2(lo), b = __half22float2(hi);
  return make_float4(a.x, a.y, b.x, b.y);
}

MJ_DEV int wrap_index(int i, int n) {
  int r = i % n;
  return r < 0 ? r + n : r;
}

MJ_DEV float4 lerp4(float4 a, float4 b, float t) {
  return make_float4(a.x + (b.x - a.x) * t, a.y + (b.y - a.y) * t, a.z + (b.z - a.z) * t, a.w + (b.w - a.w) * t);
}

// Bilinear sample of one level; wrap_u / wrap_v select WRAP (else CLAMP) addressing.
MJ_DEV float4 sample_level(const MjpbrTexture& t, const uint8_t* data, int level, float u, float v, bool wrap_u,
                           bool wrap_v) {
  int w = max(t.width >> level, 1), h = max(t.height >> level, 1);
  float fx = u * (float)w - 0.5f, fy = v * (float)h - 0.5f;
  float x0f = floorf(fx), y0f = floorf(fy);
  float tx = fx - x0f, ty = fy - y0f;
  int x0 = (int)x0f, y0 = (int)y0f, x1 = x0 + 1, y1 = y0 + 1;
  if (wrap_u) {
    x0 = wrap_index(x0, w);
    x1 = wrap_index(x1, w);
  } else {
    x0 = min(max(x0, 0), w - 1);
    x1 = min(max(x1, 0), w - 1);
  }
  if (wrap_v) {
    y0 = wrap_index(y0, h);
    y1 = wrap_index(y1, h);
  } else {
    y0 = min(max(y0, 0), h - 1);
    y1 = min(max(y1, 0), h - 1);
  }
  float4 a = fetch_texel(t, data, level, w, x0, y0);
  float4 b = fetch_texel(t, data, level, w, x1, y0);
  float4 c = fetch_texel(t, data, level, w, x0, y1);
  float4 d = fetch_texel(t, data, level, w, x1, y1);
  return lerp4(lerp4(a, b, tx), lerp4(c, d, tx), ty);
}

// Trilinear sample at level of detail lod (clamped to the chain).
static __device__ __noinline__ float4 sample_trilinear(const MjpbrTexture& t, const uint8_t* data, float u, float v, float lod, bool wrap_u,
                               bool wrap_v) {
  float l = clampf(lod, 0.0f, (float)(t.nlevel - 1));
  float l0f = floorf(l);
  int l0 = (int)l0f;
  float f = l - l0f;
  float4 a = sample_level(t, data, l0, u, v, wrap_u, wrap_v);
  if (f <= 0.0f || l0 + 1 >= t.nlevel) return a;
  float4 b = sample_level(t, data, l0 + 1, u, v, wrap_u, wrap_v);
  return lerp4(a, b, f);
}

// Mip level of a ray-cone footprint (texture.py:225-228).
MJ_DEV float texture_lod(float footprint, float uv_per_length, const MjpbrTexture& t) {
  float texels = footprint * uv_per_length * (float)max(t.width, t.height);
  return __log2f(fmaxf(texels, 1.0e-8f));
}

// ---------------------------------------------------------------- environment

// Equirect coordinates of a world direction (row 0 = +z, centre column = +x), yaw about +z.
MJ_DEV void direction_to_uv(V3 d, float yaw, float* u, float* v) {
  float phi = fast_atan2(d.y, d.x) - yaw;
  float uu = 0.5f + phi * (0.5f / kPi);
  *u = uu - floorf(uu);
  *v = fast_acos(clampf(d.z, -1.0f, 1.0f)) * (1.0f / kPi);
}

MJ_DEV V3 rotate_yaw(V3 d, float yaw) {
  float c = __cosf(yaw), s = __sinf(yaw);
  return V3{c * d.x - s * d.y, s * d.x + c * d.y, d.z};
}

MJ_DEV V3 eval_sh9(const float* sh, V3 n) {
  float x = n.x, y = n.y, z = n.z;
  float b[9] = {0.282095f,
                0.488603f * y,
                0.488603f * z,
                0.488603f * x,
                1.092548f * x * y,
                1.092548f * y * z,
                0.315392f * (3.0f * z * z - 1.0f),
                1.092548f * x * z,
                0.546274f * (x * x - y * y)};
  V3 c = v3(0.0f);
#pragma unroll
  for (int k = 0; k < 9; ++k) c = c + V3{__ldg(sh + 3 * k), __ldg(sh + 3 * k + 1), __ldg(sh + 3 * k + 2)} * b[k];
  return vmax(c, v3(0.0f));
}

MJ_DEV V3 sample_radiance(const MjpbrTexture& t, const uint8_t* data, V3 d, float yaw, float lod) {
  float u, v;
  direction_to_uv(d, yaw, &u, &v);
  float4 c = sample_trilinear(t, data, u, v, fmaxf(lod, 0.0f), true, false);
  return V3{c.x, c.y, c.z};
}

MJ_DEV float4 stack_texel(const uint16_t* stack, int w, int h, int level, int x, int y) {
  uint2 raw = __ldg(reinterpret_cast<const uint2*>(stack) + ((int64_t)(level * h + y) * w + x));
  __half2 lo = *reinterpret_cast<__half2*>(&raw.x);
  __half2 hi = *reinterpret_cast<__half2*>(&raw.y);
  float2 a = __half22float2(lo), b = __half22float2(hi);
  return make_float4(a.x, a.y, b.x, b.y);
}

// Trilinear lookup of the prefiltered stack (u WRAP, v CLAMP, roughness axis CLAMP), a 3D texture
// sampled at w = (pr (levels - 1) + 0.5) / levels.
static __device__ __noinline__ V3 sample_prefiltered(const uint16_t* stack, int levels, int h, int w, V3 d, float yaw, float pr) {
  float u, v;
  direction_to_uv(d, yaw, &u, &v);
  float wz = (clampf(pr, 0.0f, 1.0f) * ((float)levels - 1.0f) + 0.5f) / (float)levels;
  float fz = wz * (float)levels - 0.5f;
  float z0f = floorf(fz);
  float tz = fz - z0f;
  int z0 = min(max((int)z0f, 0), levels - 1), z1 = min(max((int)z0f + 1, 0), levels - 1);
  float fx = u * (float)w - 0.5f, fy = v * (float)h - 0.5f;
  float x0f = floorf(fx), y0f = floorf(fy);
  float tx = fx - x0f, ty = fy - y0f;
  int x0 = wrap_index((int)x0f, w), x1 = wrap_index((int)x0f + 1, w);
  int y0 = min(max((int)y0f, 0), h - 1), y1 = min(max((int)y0f + 1, 0), h - 1);
  float4 r0 = lerp4(lerp4(stack_texel(stack, w, h, z0, x0, y0), stack_texel(stack, w, h, z0, x1, y0), tx),
                    lerp4(stack_texel(stack, w, h, z0, x0, y1), stack_texel(stack, w, h, z0, x1, y1), tx), ty);
  float4 r1 = lerp4(lerp4(stack_texel(stack, w, h, z1, x0, y0), stack_texel(stack, w, h, z1, x1, y0), tx),
                    lerp4(stack_texel(stack, w, h, z1, x0, y1), stack_texel(stack, w, h, z1, x1, y1), tx), ty);
  float4 c = lerp4(r0, r1, tz);
  return V3{c.x, c.y, c.z};
}

}  // namespace mjpbr
