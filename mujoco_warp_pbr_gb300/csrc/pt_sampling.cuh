// Sampling of the path-traced tier: GGX visible-normal and cosine lobes, their pdfs and the
// BSDF x cosine (mujoco_warp_pbr/_src/brdf.py:116-191), environment importance sampling over the
// luminance * sin(theta) CDF tables (mujoco_warp_pbr/_src/envmap.py:433-490), the power
// heuristic, and the random-number layout (mujoco_warp_pbr/_src/pathtrace.py:64-95).
//
// Everything that decides where a path goes (sampled directions, probabilities of lobes and
// Russian roulette, beta) is plain float arithmetic with the deterministic sincos_turns, so the
// scalar oracle takes the same decisions bit for bit.
#pragma once

#include "shading.cuh"

namespace mjpbr {

// The BSDF evaluation and pdf are called from several places of the bounce loop (each light's
// sample, the environment sample, the continuation); one out-of-line copy keeps the loop's code
// small (the path kernel is bound by instruction fetch when everything is inlined).
#ifdef MJPBR_PT_INLINE
#define MJPBR_PT_CALL static __device__ __forceinline__
#else
#define MJPBR_PT_CALL static __device__ __noinline__
#endif

// Random-number layout: path vertex (sample, depth) owns kSlots consecutive counters; depth row
// kJitterDepth holds the sub-pixel jitter. Slots: 0 alpha, 1 mirror, 2-3 environment, 4-11 the
// light samples of lights 0-3, 12-14 BSDF, 15 Russian roulette; further lights draw from a
// separate counter range from kExtraLights.
constexpr int32_t kSlots = 16;
constexpr int32_t kDepths = 64;
constexpr int32_t kJitterDepth = kDepths - 1;
constexpr int32_t kSlotLights = 4;
constexpr int32_t kSlottedLights = 4;
constexpr uint32_t kExtraLights = 1u << 30;
constexpr int32_t kSubpixel = 15;
constexpr float kRrMin = 0.05f;
constexpr float kRrMax = 0.95f;

MJ_HD float pt_rand(uint32_t seed, int32_t sample, int32_t depth, int32_t slot) {
  return rand01(seed, (uint32_t)((sample * kDepths + depth) * kSlots + slot));
}

MJ_HD void light_rand2(uint32_t seed, int32_t sample, int32_t depth, int32_t nlight, int32_t li, float* u0, float* u1) {
  if (li < kSlottedLights) {
    int32_t slot = kSlotLights + 2 * li;
    *u0 = pt_rand(seed, sample, depth, slot);
    *u1 = pt_rand(seed, sample, depth, slot + 1);
    return;
  }
  uint32_t counter = kExtraLights + (uint32_t)(((sample * kDepths + depth) * nlight + li) * 2);
  *u0 = rand01(seed, counter);
  *u1 = rand01(seed, counter + 1u);
}

MJ_HD float smith_g1(float nov, float alpha) {
  float a2 = alpha * alpha;
  return 2.0f * nov / (nov + sqrtf(a2 + (1.0f - a2) * nov * nov));
}

// Half vector distributed as GGX's visible normals for view v (Heitz 2018), local frame +z = n.
MJ_HD V3 sample_ggx_vndf(V3 v, float alpha, float u0, float u1) {
  V3 vh = normalize(V3{alpha * v.x, alpha * v.y, v.z});
  float lensq = vh.x * vh.x + vh.y * vh.y;
  V3 t1 = V3{1.0f, 0.0f, 0.0f};
  if (lensq > 0.0f) t1 = V3{-vh.y, vh.x, 0.0f} / sqrtf(lensq);
  V3 t2 = cross(vh, t1);
  float r = sqrtf(u0);
  float sn, cs;
  sincos_turns(u1, &sn, &cs);
  float p1 = r * cs;
  float p2 = r * sn;
  float s = 0.5f * (1.0f + vh.z);
  p2 = (1.0f - s) * sqrtf(fmaxf(1.0f - p1 * p1, 0.0f)) + s * p2;
  V3 nh = t1 * p1 + t2 * p2 + vh * sqrtf(fmaxf(1.0f - p1 * p1 - p2 * p2, 0.0f));
  return normalize(V3{alpha * nh.x, alpha * nh.y, fmaxf(nh.z, 0.0f)});
}

// BRDF x cos(theta_l) for local view v and light l (diffuse already (1 - E) weighted).
MJPBR_PT_CALL V3 eval_bsdf_cos(V3 diffuse_color, V3 f0, float alpha, V3 energy_comp, V3 v, V3 l) {
  float nol = l.z;
  float nov = fmaxf(v.z, 1.0e-4f);
  if (nol <= 0.0f) return v3(0.0f);
  V3 h = normalize(l + v);
  float noh = fmaxf(h.z, 0.0f), loh = fmaxf(dot(l, h), 0.0f);
  // specular_lobe with plain arithmetic
  float a2 = alpha * alpha;
  float fd = (noh * a2 - noh) * noh + 1.0f;
  float D = a2 / (kPi * fd * fd);
  float gv = nol * sqrtf(nov * nov * (1.0f - a2) + a2);
  float gl = nov * sqrtf(nol * nol * (1.0f - a2) + a2);
  float Vis = 0.5f / (gv + gl);
  float x = 1.0f - loh;
  float x2 = x * x;
  float fc = x2 * x2 * x;
  V3 F = f0 * (1.0f - fc) + v3(fc);
  V3 spec = cmul(F * (D * Vis), energy_comp);
  return (diffuse_color * (1.0f / kPi) + spec) * nol;
}

// Solid-angle pdf of sample_bsdf: mixture of GGX VNDF and cosine-weighted hemisphere.
MJPBR_PT_CALL float pdf_bsdf(float alpha, float p_spec, V3 v, V3 l) {
  if (l.z <= 0.0f) return 0.0f;
  float nov = fmaxf(v.z, 1.0e-4f);
  V3 h = normalize(l + v);
  float noh = fmaxf(h.z, 0.0f);
  float a2 = alpha * alpha;
  float fd = (noh * a2 - noh) * noh + 1.0f;
  float D = a2 / (kPi * fd * fd);
  float pdf_spec = smith_g1(nov, alpha) * D / (4.0f * nov);
  float pdf_diff = l.z * (1.0f / kPi);
  return p_spec * pdf_spec + (1.0f - p_spec) * pdf_diff;
}

// Probability of sampling the specular lobe, from the lobes' albedo luminance.
MJ_HD float specular_probability(V3 diffuse_color, V3 spec_albedo) {
  float ws = luminance(spec_albedo);
  float wd = luminance(diffuse_color);
  if (wd <= 0.0f) return 1.0f;
  return clampf(ws / fmaxf(ws + wd, 1.0e-6f), 0.1f, 0.9f);
}

// Local light direction drawn from the mixture (may fall below the horizon: then rejected).
MJ_HD V3 sample_bsdf(float alpha, float p_spec, V3 v, float u_lobe, float u0, float u1) {
  if (u_lobe < p_spec) {
    V3 h = sample_ggx_vndf(v, alpha, u0, u1);
    return h * (2.0f * dot(v, h)) - v;
  }
  float r = sqrtf(u0);
  float sn, cs;
  sincos_turns(u1, &sn, &cs);
  return V3{r * cs, r * sn, sqrtf(fmaxf(1.0f - u0, 0.0f))};
}

MJ_HD float power_heuristic(float a, float b) {
  float a2 = a * a;
  return a2 / fmaxf(a2 + b * b, 1.0e-30f);
}

// Equirect direction of (u, v) (row 0 = +z, centre column = +x), deterministic sincos.
MJ_HD V3 uv_to_direction_exact(float u, float v) {
  float sp, cp, st, ct;
  sincos_turns(u - 0.5f, &sp, &cp);
  sincos_turns(v * 0.5f, &st, &ct);
  return V3{st * cp, st * sp, ct};
}

MJ_HD V3 rotate_yaw_exact(V3 d, float yaw) {
  float s, c;
  sincos_turns(yaw * (0.5f / kPi), &s, &c);
  return V3{c * d.x - s * d.y, s * d.x + c * d.y, d.z};
}

// Largest i in [0, n) with cdf[i] <= u.
MJ_HD int32_t cdf_search(const float* cdf, int32_t n, float u) {
  int32_t lo = 0, hi = n;
  while (hi - lo > 1) {
    int32_t mid = (lo + hi) / 2;
    if (cdf[mid] <= u) {
      lo = mid;
    } else {
      hi = mid;
    }
  }
  return lo;
}

// World direction drawn proportional to the environment's luminance, and its solid-angle pdf.
MJ_HD V3 env_sample_direction(const float* marginal, const float* conditional, const float* prob, int32_t h, int32_t w,
                              float yaw, float u0, float u1, float* pdf) {
  int32_t r = cdf_search(marginal, h, u0);
  float c0 = marginal[r];
  float dv = (u0 - c0) / fmaxf(marginal[r + 1] - c0, 1.0e-12f);
  const float* crow = conditional + (int64_t)r * (w + 1);
  int32_t c = cdf_search(crow, w, u1);
  float k0 = crow[c];
  float du = (u1 - k0) / fmaxf(crow[c + 1] - k0, 1.0e-12f);
  float uu = ((float)c + clampf(du, 0.0f, 1.0f)) / (float)w;
  float vv = ((float)r + clampf(dv, 0.0f, 1.0f)) / (float)h;
  V3 d = rotate_yaw_exact(uv_to_direction_exact(uu, vv), yaw);
  float st, ct;
  sincos_turns(vv * 0.5f, &st, &ct);
  float sin_theta = fmaxf(st, 1.0e-6f);
  *pdf = prob[(int64_t)r * w + c] * (float)(w * h) / (2.0f * kPi * kPi * sin_theta);
  return d;
}

}  // namespace mjpbr
