// One bounce of the path tracer (mujoco_warp_pbr/_src/pathtrace.py:200-338) after its closest hit
// is known, shared by the persistent path kernel (pathtrace.cu) and the staged wavefront
// (pt_wave.cu): the miss (background / environment with MIS), the surface, stochastic alpha
// pass-through, emission, the mirror lobe, next-event estimation of every light and of the
// environment, BSDF sampling and Russian roulette.
//
// How the shadow rays of next-event estimation are answered is a policy (`Nee`): the persistent
// kernel traces each one where it is asked; the wavefront records the unshadowed contribution and
// the ray, traces all of a stage's shadow rays in a separate kernel and adds the contributions
// afterwards in the same order. Both add exactly the same terms in the same order, so the images
// are bit-identical.
#pragma once

#include "denoise_common.cuh"
#include "kernel_common.cuh"
#include "pt_sampling.cuh"

namespace mjpbr {

struct PathState {
  V3 o, d, beta, radiance;
  float max_dist, pdf_prev;
  int32_t depth, passes, sample;
  bool camera_ray, delta;
  // first surface of the path (denoiser features, guides)
  V3 albedo, normal, emission, base_color;
  float dcam_z;
};

struct PixelAcc {
  V3 hdr, albedo, normal, emission;
  float lum_sq, first_depth;
  V3 guide_albedo, guide_normal;
};

// The terms of one light's next-event estimate before its shadow test.
struct LightQuery {
  V3 l;           // direction to the (jittered) light
  V3 ll;          // l in the shading frame (t1, t2, n)
  V3 ds, ss;      // diffuse / specular radiance scales
  float max_t;    // shadow ray length
  bool shadowed;  // the light casts shadows: the estimate needs a shadow ray
};

template <bool kMesh, bool kTex>
struct PtCore {
  static __device__ __noinline__ V3 environment(const RtCtx& c, V3 d) {
    const MjpbrScene& s = *c.s;
    MJPBR_COUNT(kOpBackground);
    return sample_radiance(s.env_radiance[c.env], s.env_data, d, c.env_yaw, 0.0f) * c.env_scale;
  }

  // Solid-angle pdf of env_sample_direction for a world direction (envmap.py:478-490).
  static MJ_DEV float env_direction_pdf(const RtCtx& c, V3 d) {
    const MjpbrScene& s = *c.s;
    const int32_t h = s.cdf_height, w = s.cdf_width;
    float u, v;
    direction_to_uv(d, c.env_yaw, &u, &v);
    int32_t col = min((int32_t)(u * (float)w), w - 1);
    int32_t row = min((int32_t)(v * (float)h), h - 1);
    float sn, cs;
    sincos_turns(v * 0.5f, &sn, &cs);
    float sin_theta = fmaxf(sn, 1.0e-6f);
    return s.env_prob[((int64_t)c.env * h + row) * w + col] * (float)(w * h) / (2.0f * kPi * kPi * sin_theta);
  }

  // One punctual light (its bulb disc jittered by u0, u1 for soft shadows) seen from the point:
  // false when it does not reach it (behind the surface, outside its cone or range).
  // out of line: one copy of the light-sampling code in the bounce loop (1 % faster measured)
  static __device__ __noinline__ bool light_query(RtCtx& c, Light light, V3 point, V3 normal, V3 t1, V3 t2, float u0, float u1,
                                                  LightQuery* q) {
    const MjpbrSettings& st = c.s->settings;
    if (light.type != MJPBR_LIGHT_DIRECTIONAL && light.bulbradius > 0.0f) {
      V3 b1, b2;
      orthonormal_basis(normalize(point - light.pos), &b1, &b2);
      float r = light.bulbradius * sqrtf(u0);
      float sn, cs;
      sincos_turns(u1, &sn, &cs);
      light.pos = light.pos + (b1 * cs + b2 * sn) * r;
    }
    float dist;
    MJPBR_COUNT(kOpPtLight);
    eval_light(light, st.light_model, point, &q->l, &dist, &q->ds, &q->ss);
    q->ll = V3{dot(q->l, t1), dot(q->l, t2), dot(q->l, normal)};
    if (q->ll.z <= 0.0f || (length_sq(q->ds) == 0.0f && length_sq(q->ss) == 0.0f)) return false;
    q->shadowed = st.use_shadows && light.castshadow;
    q->max_t = light.type == MJPBR_LIGHT_DIRECTIONAL ? kUnboundedShadow : dist - kShadowGap;
    return true;
  }

  // The unshadowed next-event estimate of a light that reaches the point.
  static MJ_DEV V3 light_contribution(const Lobes& lb, V3 v, const LightQuery& q) {
    V3 diffuse = eval_bsdf_cos(lb.diffuse_color, v3(0.0f), lb.alpha, v3(0.0f), v, q.ll);
    V3 specular = eval_bsdf_cos(v3(0.0f), lb.f0, lb.alpha, lb.energy_comp, v, q.ll);
    return cmul(diffuse, q.ds) + cmul(specular, q.ss);
  }

  // The bounce after its closest hit (pathtrace.py:230-337); true when the path has ended.
  template <class Nee>
  static MJ_DEV bool surface(RtCtx& c, Nee& nee, PathState& ps, const Hit& hit, uint32_t seed, V3 head_dir) {
    const MjpbrScene& s = *c.s;
    const MjpbrSettings& st = s.settings;
    if (hit.geom == -1) {
      if (ps.camera_ray) {
        V3 bg = (kTex && st.env_background)
                    ? environment(c, ps.d)
                    : V3{st.background[0], st.background[1], st.background[2]} / c.exposure;
        ps.radiance += cmul(ps.beta, bg);
      } else {
        V3 env_light = c.ambient;
        if (kTex && st.has_env) {
          float weight = 1.0f;
          if (!ps.delta) weight = power_heuristic(ps.pdf_prev, env_direction_pdf(c, ps.d));
          env_light = env_light + environment(c, ps.d) * weight;
        }
        ps.radiance += cmul(ps.beta, env_light);
      }
      return true;
    }
    const V3 point = ps.o + ps.d * hit.dist;
    V3 normal;
    MJPBR_COUNT(kOpPtVertex);
    Surface sf = eval_surface<kMesh, kTex>(s, c.blk, c.L, c.w, hit, hit.slot, point, ps.d, 0.0f, &normal);
    if (st.has_transparency) {
      if (pt_rand(seed, ps.sample, ps.depth + ps.passes, 0) >= sf.alpha && ps.passes < 4 * st.max_layers) {
        ps.o = point + ps.d * kRayOffset;
        ps.max_dist = ps.max_dist - hit.dist;
        ps.passes += 1;
        return false;
      }
    }
    ps.radiance += cmul(ps.beta, sf.emissive / c.exposure);
    if (ps.depth == st.max_depth) return true;
    ps.max_dist = kMaxVal;
    if (ps.camera_ray) {
      ps.albedo = sf.base_color;
      ps.normal = normal;
      ps.base_color = sf.base_color;
      ps.emission = sf.emissive / c.exposure;
    }
    const bool camera_ray = ps.camera_ray;
    ps.camera_ray = false;
    if (st.has_reflection) {
      const float mirror = mirror_reflectance(c, hit.slot);
      if (pt_rand(seed, ps.sample, ps.depth, 1) < mirror) {
        ps.d = ps.d - normal * (2.0f * dot(ps.d, normal));
        ps.o = point + normal * kRayOffset;
        ps.delta = true;
        ps.depth += 1;
        return ps.depth > st.max_depth;
      }
    }
    V3 t1, t2;
    orthonormal_basis(normal, &t1, &t2);
    const V3 view = -ps.d;
    const V3 v{dot(view, t1), dot(view, t2), dot(view, normal)};
    const float nov = fmaxf(v.z, 1.0e-4f);
    const Lobes lb = shading_lobes(s.dfg_lut, s.dfg_size, sf, nov);
    const V3 spec_weight = cmul(lb.spec_albedo, lb.energy_comp);
    const float p_spec = specular_probability(lb.diffuse_color, spec_weight);
    if (ps.depth == 0 && camera_ray) ps.albedo = lb.diffuse_color + spec_weight;

    // next-event estimation: MuJoCo lights (slots 0 .. nlight - 1), then the headlight (slot
    // nlight: no shadow, display-relative), then the environment
    const V3 origin = point + normal * kRayOffset;
    nee.begin(ps, origin);
    const int32_t nl = c.L.nlight + (st.headlight_active ? 1 : 0);
#pragma unroll 1
    for (int32_t li = 0; li < nl; ++li) {
      Light light;
      float u0 = 0.0f, u1 = 0.0f;
      if (li < c.L.nlight) {
        light = load_light(c.blk + c.L.light_off + li * kLightFloats);
        if (!light.active) continue;
        light_rand2(seed, ps.sample, ps.depth, c.L.nlight, li, &u0, &u1);
      } else {
        light = make_headlight(st, head_dir, c.exposure);
      }
      LightQuery q;
      if (!light_query(c, light, point, normal, t1, t2, u0, u1, &q)) {
        nee.none(li);
        continue;
      }
      nee.light(c, li, q.shadowed, origin, q.l, q.max_t, [&] { return light_contribution(lb, v, q); });
    }
    nee.lights_done(ps);

    if (kTex && st.has_env) {
      float pdf_env;
      MJPBR_COUNT(kOpPtEnvSample);
      const int32_t h = s.cdf_height, w = s.cdf_width;
      V3 d_env = env_sample_direction(s.env_marginal + (int64_t)c.env * (h + 1), s.env_conditional + (int64_t)c.env * h * (w + 1),
                                      s.env_prob + (int64_t)c.env * h * w, h, w, c.env_yaw,
                                      pt_rand(seed, ps.sample, ps.depth, 2), pt_rand(seed, ps.sample, ps.depth, 3), &pdf_env);
      V3 le{dot(d_env, t1), dot(d_env, t2), dot(d_env, normal)};
      if (le.z > 0.0f && pdf_env > 0.0f) {
        V3 f = eval_bsdf_cos(lb.diffuse_color, lb.f0, lb.alpha, lb.energy_comp, v, le);
        const V3 beta = ps.beta;
        nee.env(c, ps, origin, d_env, [&] {
          float weight = power_heuristic(pdf_env, pdf_bsdf(lb.alpha, p_spec, v, le));
          return cmul(beta, cmul(f, environment(c, d_env))) * (weight / pdf_env);
        });
      }
    }

    // continue the path by sampling the BSDF
    const V3 l = sample_bsdf(lb.alpha, p_spec, v, pt_rand(seed, ps.sample, ps.depth, 12), pt_rand(seed, ps.sample, ps.depth, 13),
                             pt_rand(seed, ps.sample, ps.depth, 14));
    if (l.z <= 0.0f) return true;
    const float pdf = pdf_bsdf(lb.alpha, p_spec, v, l);
    if (pdf <= 0.0f) return true;
    ps.beta = cmul(ps.beta, eval_bsdf_cos(lb.diffuse_color, lb.f0, lb.alpha, lb.energy_comp, v, l) / pdf);
    ps.d = normalize(t1 * l.x + t2 * l.y + normal * l.z);
    ps.o = point + normal * kRayOffset;
    ps.pdf_prev = pdf;
    ps.delta = false;
    ps.depth += 1;
    if (ps.depth >= st.rr_depth) {
      float q = clampf(fmaxf(ps.beta.x, fmaxf(ps.beta.y, ps.beta.z)), kRrMin, kRrMax);
      if (pt_rand(seed, ps.sample, ps.depth, 15) >= q) return true;
      ps.beta = ps.beta / q;
    }
    return ps.depth > st.max_depth;
  }
};

// Sample `sample` of a pixel: sample 0 through the centre of the 15 x 15 sub-pixel grid, the others
// at a jittered cell (pathtrace.py:362-378).
MJ_DEV void start_sample(PathState& ps, const MjpbrScene& s, const Pixel& p, uint32_t seed, const M3& R, V3 cpos,
                         int32_t sample) {
  int32_t sx = kSubpixel / 2, sy = kSubpixel / 2;
  if (sample > 0) {
    sx = (int32_t)(pt_rand(seed, sample, kJitterDepth, 0) * (float)kSubpixel);
    sy = (int32_t)(pt_rand(seed, sample, kJitterDepth, 1) * (float)kSubpixel);
  }
  V3 dcam, ocam;
  primary_ray(s, p, kSubpixel, sx, sy, &dcam, &ocam, &ps.max_dist, &ps.dcam_z);
  ps.o = cpos + mul(R, ocam);
  ps.d = mul(R, dcam);
  ps.beta = v3(1.0f);
  ps.radiance = v3(0.0f);
  ps.pdf_prev = 0.0f;
  ps.depth = 0;
  ps.passes = 0;
  ps.sample = sample;
  ps.camera_ray = true;
  ps.delta = true;
  ps.albedo = v3(1.0f);
  ps.normal = v3(0.0f);
  ps.emission = v3(0.0f);
  ps.base_color = v3(0.0f);
}

MJ_DEV void clear_pixel(PixelAcc& acc) {
  acc.hdr = acc.albedo = acc.normal = acc.emission = v3(0.0f);
  acc.lum_sq = 0.0f;
  acc.first_depth = 0.0f;
  acc.guide_albedo = acc.guide_normal = v3(0.0f);
}

// Adds a finished sample to its pixel (samples in order).
MJ_DEV void add_sample(PixelAcc& acc, const PathState& ps, bool denoise, float exposure) {
  acc.hdr += ps.radiance;
  acc.albedo += ps.albedo;
  acc.normal += ps.normal;
  acc.emission += ps.emission;
  if (ps.sample == 0) {
    acc.guide_albedo = ps.base_color;
    acc.guide_normal = ps.normal;
  }
  if (denoise) {
    float lum = luminance(ps.radiance) * exposure;
    acc.lum_sq += lum * lum;
  }
}

// Writes a finished pixel (address adr in the output rows): the display colour, or with the
// denoiser the noisy HDR and the filter's inputs (pathtrace.py:381-421).
MJ_DEV void write_pixel(const MjpbrScene& s, const RtCtx& c, int64_t adr, const PixelAcc& acc, int32_t nsample) {
  const MjpbrSettings& st = s.settings;
  const float inv_n = 1.0f / (float)nsample;
  const V3 hdr = acc.hdr * inv_n;
  if (st.render_guides && s.guide_albedo) {
    s.guide_albedo[adr * 3] = acc.guide_albedo.x;
    s.guide_albedo[adr * 3 + 1] = acc.guide_albedo.y;
    s.guide_albedo[adr * 3 + 2] = acc.guide_albedo.z;
    s.guide_normal[adr * 3] = acc.guide_normal.x;
    s.guide_normal[adr * 3 + 1] = acc.guide_normal.y;
    s.guide_normal[adr * 3 + 2] = acc.guide_normal.z;
  }
  if (st.denoise) {
    // noisy HDR, the filter's guide (normal and albedo at half precision), the exposed first-hit
    // emission and the demodulated radiance the first filter pass reads
    s.hdr_data[adr * 3] = hdr.x;
    s.hdr_data[adr * 3 + 1] = hdr.y;
    s.hdr_data[adr * 3 + 2] = hdr.z;
    const V3 em = acc.emission * (c.exposure * inv_n);
    V3 nm = acc.normal;
    if (length_sq(nm) > 0.0f) nm = normalize(nm);
    const uint4 g = pack_guide(nm, acc.albedo * inv_n, acc.first_depth);
    reinterpret_cast<uint4*>(s.aov_guide)[adr] = g;
    float* e = s.aov_emission + adr * 3;
    e[0] = em.x;
    e[1] = em.y;
    e[2] = em.z;
    const float mean_lum = luminance(hdr) * c.exposure;
    const float variance = fmaxf(acc.lum_sq * inv_n - mean_lum * mean_lum, 0.0f) * inv_n;
    reinterpret_cast<float4*>(s.denoise_buffers[0])[adr] = demodulate(hdr, c.exposure, em, unpack_guide(g).albedo, variance);
  } else {
    if (st.render_hdr && s.hdr_data) {
      s.hdr_data[adr * 3] = hdr.x;
      s.hdr_data[adr * 3 + 1] = hdr.y;
      s.hdr_data[adr * 3 + 2] = hdr.z;
    }
    s.rgb_data[adr] = encode_display(display_transform(hdr * c.exposure, st.tone_mapper));
  }
}

}  // namespace mjpbr
