// Pixel-local pieces of the edge-avoiding a-trous denoiser (mujoco_warp_pbr/_src/denoise.py): the
// packed first-hit guide (normal and albedo at half precision, as the reference's vec3h feature
// arrays, and the depth), demodulation of the noisy radiance by the albedo and its remodulation.
#pragma once

#include "common.cuh"

namespace mjpbr {

// Albedo floor of the demodulation (dark albedos would amplify noise).
constexpr float kMinAlbedo = 1.0e-2f;

struct Guide {
  V3 normal, albedo;
  float depth;
};

MJ_DEV uint4 pack_guide(V3 n, V3 a, float depth) {
  uint4 g;
  g.x = (uint32_t)float_to_half(n.x) | ((uint32_t)float_to_half(n.y) << 16);
  g.y = (uint32_t)float_to_half(n.z) | ((uint32_t)float_to_half(a.x) << 16);
  g.z = (uint32_t)float_to_half(a.y) | ((uint32_t)float_to_half(a.z) << 16);
  g.w = __float_as_uint(depth);
  return g;
}

MJ_DEV Guide unpack_guide(uint4 g) {
  Guide r;
  r.normal = V3{half_to_float((uint16_t)(g.x & 0xffffu)), half_to_float((uint16_t)(g.x >> 16)), half_to_float((uint16_t)(g.y & 0xffffu))};
  r.albedo = V3{half_to_float((uint16_t)(g.y >> 16)), half_to_float((uint16_t)(g.z & 0xffffu)), half_to_float((uint16_t)(g.z >> 16))};
  r.depth = __uint_as_float(g.w);
  return r;
}

// Demodulated exposed radiance (emission removed, divided by the albedo) and the variance of its
// luminance (denoise.py:84-91).
MJ_DEV float4 demodulate(V3 hdr, float exposure, V3 emission, V3 albedo, float variance) {
  V3 c = hdr * exposure - emission;
  c = V3{fmaxf(c.x, 0.0f) / fmaxf(albedo.x, kMinAlbedo), fmaxf(c.y, 0.0f) / fmaxf(albedo.y, kMinAlbedo),
         fmaxf(c.z, 0.0f) / fmaxf(albedo.z, kMinAlbedo)};
  float scale = 1.0f / fmaxf(luminance(albedo), kMinAlbedo);
  return make_float4(c.x, c.y, c.z, variance * scale * scale);
}

// Exposed radiance of a filtered demodulated pixel (denoise.py:181-201).
MJ_DEV V3 remodulate(float4 s, V3 emission, V3 albedo) {
  return emission + V3{s.x * fmaxf(albedo.x, kMinAlbedo), s.y * fmaxf(albedo.y, kMinAlbedo), s.z * fmaxf(albedo.z, kMinAlbedo)};
}

}  // namespace mjpbr
