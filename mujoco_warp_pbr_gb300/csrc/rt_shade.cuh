// Real-time tier shading shared by the megakernel (render_rt.cu) and the staged wavefront
// (render_wave.cu): direct lights with their shadow visibility, split-sum ambient from the
// environment, and the background of missed rays (mujoco_warp_pbr/_src/render.py:81-239).
//
// How a light's shadow visibility is obtained is a policy (`Vis::visibility`): the megakernel
// traces the shadow rays where it needs them; the wavefront traces them in a separate kernel and
// reads the counts back. Both go through the same ray set-up (shadow_setup / shadow_ray) and the
// same count -> fraction rule (visible_fraction), so the two give bit-identical images.
#pragma once

#include "kernel_common.cuh"

namespace mjpbr {

constexpr float kMinTexels = 1.0e-8f;

// Rays a light's visibility takes: one towards a directional light or with hard shadows,
// settings.shadow_samples towards the disc of a point / spot light's bulb.
MJ_DEV int32_t shadow_ray_count(const Light& light, int32_t shadow_samples) {
  return (light.type == MJPBR_LIGHT_DIRECTIONAL || shadow_samples <= 1) ? 1 : shadow_samples;
}

// Whether shade_light asks for the visibility of `light` at a point with shading normal `normal`,
// and its direction / distance when it does (the same eval_light call as the shading).
MJ_DEV bool shadow_setup(const MjpbrSettings& st, const Light& light, V3 point, V3 normal, V3* l, float* dist) {
  V3 ds, ss;
  eval_light(light, st.light_model, point, l, dist, &ds, &ss);
  const float nol = dot(normal, *l);
  if (nol <= 0.0f || (length_sq(ds) == 0.0f && length_sq(ss) == 0.0f)) return false;
  return st.use_shadows && light.castshadow;
}

// Shadow ray k of a light's visibility from origin (render.py:81-127): towards a directional
// light, the light centre (hard shadows), or a point of the bulb disc drawn with the counter-based
// generator (counter ((stream * nlight + li) * ns + k) * 2).
MJ_DEV void shadow_ray(const Light& light, int32_t ns, V3 origin, V3 l, float dist, uint32_t seed, int32_t stream,
                       int32_t nlight, int32_t li, int32_t k, V3* dir, float* max_dist) {
  if (light.type == MJPBR_LIGHT_DIRECTIONAL) {
    *dir = l;
    *max_dist = kUnboundedShadow;
    return;
  }
  if (ns <= 1) {
    *dir = l;
    *max_dist = dist - kShadowGap;
    return;
  }
  V3 t1, t2;
  orthonormal_basis(l, &t1, &t2);
  const uint32_t counter = (uint32_t)(((stream * nlight + li) * ns + k) * 2);
  const float u0 = rand01(seed, counter), u1 = rand01(seed, counter + 1u);
  const float r = light.bulbradius * sqrtf(u0);
  float sn, cs;
  sincos_turns(u1, &sn, &cs);
  const V3 to = light.pos + (t1 * cs + t2 * sn) * r - origin;
  const float d = length(to);
  *dir = to / d;
  *max_dist = d - kShadowGap;
}

// Fraction of the light reaching the point from the number of unoccluded shadow rays.
MJ_DEV float visible_fraction(const Light& light, int32_t ns, int32_t visible, float shadow_light_fraction) {
  if (light.type == MJPBR_LIGHT_DIRECTIONAL || ns <= 1) return visible > 0 ? 1.0f : shadow_light_fraction;
  const float v = (float)visible / (float)ns;
  return v + (1.0f - v) * shadow_light_fraction;
}

template <bool kTex, class Vis>
struct RtShade {
  static MJ_DEV V3 shade_light(RtCtx& c, Vis& vis, const Light& light, const Lobes& lb, V3 point, V3 normal, V3 view,
                               float nov, uint32_t seed, int32_t stream, int32_t nlight, int32_t li) {
    const MjpbrSettings& st = c.s->settings;
    V3 l, ds, ss;
    float dist;
    MJPBR_COUNT(kOpLight);
    eval_light(light, st.light_model, point, &l, &dist, &ds, &ss);
    float nol = dot(normal, l);
    if (nol <= 0.0f || (length_sq(ds) == 0.0f && length_sq(ss) == 0.0f)) return v3(0.0f);
    float v = 1.0f;
    if (st.use_shadows && light.castshadow) v = vis.visibility(c, light, point, normal, l, dist, seed, stream, nlight, li);
    V3 h = fnormalize(l + view);
    float noh = fmaxf(fdot(normal, h), 0.0f);
    float loh = fmaxf(fdot(l, h), 0.0f);
    V3 fr = cmul(specular_lobe(lb.f0, lb.alpha, noh, nov, nol, loh), lb.energy_comp);
    V3 fd = lb.diffuse_color * (1.0f / kPi);
    return (cmul(fd, ds) + cmul(fr, ss)) * (nol * v);
  }

  // Outgoing radiance towards view, before exposure (render.py:184-239).
  static MJ_DEV V3 shade_surface(RtCtx& c, Vis& vis, const Surface& sf, V3 point, V3 normal, V3 view, V3 head_dir,
                                 uint32_t seed, int32_t stream) {
    const MjpbrScene& s = *c.s;
    const MjpbrSettings& st = s.settings;
    float nov = fmaxf(fdot(normal, view), 1.0e-4f);
    MJPBR_COUNT(kOpShade);
    Lobes lb = shading_lobes(s.dfg_lut, s.dfg_size, sf, nov);
    V3 irradiance = c.ambient, prefiltered = c.ambient;
    if (kTex && st.has_env) {
      MJPBR_COUNT(kOpEnv);
      irradiance = c.ambient + eval_sh9(s.env_sh + c.env * 27, rotate_yaw(normal, -c.env_yaw)) * c.env_scale;
      V3 r = view - normal * (2.0f * fdot(view, normal));
      float a2 = lb.alpha * lb.alpha;
      V3 dominant = fnormalize(-r * (1.0f - a2) + normal * a2);
      const uint16_t* stack = s.env_prefiltered +
                              (int64_t)c.env * s.prefilter_levels * s.prefilter_height * s.prefilter_width * 4;
      V3 blurred = sample_prefiltered(stack, s.prefilter_levels, s.prefilter_height, s.prefilter_width, dominant,
                                      c.env_yaw, lb.pr);
      float t = lb.pr * ((float)s.prefilter_levels - 1.0f);
      V3 spec = blurred;
      if (t < 1.0f) {
        V3 sharp = sample_radiance(s.env_radiance[c.env], s.env_data, dominant, c.env_yaw, 0.0f);
        spec = sharp * (1.0f - t) + blurred * t;
      }
      prefiltered = c.ambient + spec * c.env_scale;
    }
    float ao = sf.occlusion;
    float spec_ao = clampf(powf(nov + ao, exp2f(-16.0f * lb.alpha - 1.0f)) - 1.0f + ao, 0.0f, 1.0f);
    V3 radiance = cmul(irradiance, lb.diffuse_color) * ao + cmul(prefiltered, cmul(lb.spec_albedo, lb.energy_comp)) * spec_ao;
    // MuJoCo lights, then the headlight (a directional light along the view, no shadow, its
    // illuminance display-relative), through one shade_light call site.
    const int32_t nl = c.L.nlight + (st.headlight_active ? 1 : 0);
#pragma unroll 1
    for (int32_t li = 0; li < nl; ++li) {
      Light light;
      int32_t count = c.L.nlight, index = li;
      if (li < c.L.nlight) {
        light = load_light(c.blk + c.L.light_off + li * kLightFloats);
        if (!light.active) continue;
      } else {
        light = make_headlight(st, head_dir, c.exposure);
        count = 1;
        index = 0;
      }
      radiance += shade_light(c, vis, light, lb, point, normal, view, nov, seed, stream, count, index);
    }
    return radiance + sf.emissive / c.exposure;
  }

  static MJ_DEV V3 background(RtCtx& c, V3 d, float spread) {
    const MjpbrScene& s = *c.s;
    if (kTex && s.settings.env_background) {
      MJPBR_COUNT(kOpBackground);
      float lod = log2f(fmaxf(spread * s.settings.inv_texel_angle, kMinTexels));
      return sample_radiance(s.env_radiance[c.env], s.env_data, d, c.env_yaw, lod) * c.env_scale;
    }
    return V3{s.settings.background[0], s.settings.background[1], s.settings.background[2]} / c.exposure;
  }
};

// Mirror ray of a surface (render.py:249-274): from the point offset along the shading normal,
// the view direction reflected about it.
MJ_DEV void mirror_ray(V3 point, V3 normal, V3 dir, V3* origin, V3* reflected) {
  *reflected = dir - normal * (2.0f * dot(dir, normal));
  *origin = point + normal * kRayOffset;
}

}  // namespace mjpbr
