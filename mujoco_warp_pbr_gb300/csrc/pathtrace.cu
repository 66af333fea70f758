// Path-traced tier (mujoco_warp_pbr/_src/pathtrace.py:64-438): unidirectional path tracing with
// next-event estimation of every light (bulb discs for soft shadows) and the headlight, the
// environment importance-sampled and combined with BSDF sampling by multiple importance sampling
// (power heuristic), a stochastic perfect-mirror lobe for MuJoCo reflectance, stochastic alpha
// pass-through, Russian roulette after rr_depth bounces, sample 0 through the pixel centre and the
// others jittered on a 15 x 15 sub-pixel grid, and the denoiser's features.
//
// Execution: a persistent kernel. Each CTA pulls 32 x 32-pixel tiles (one world, one camera) from
// a global counter, copies the tile's world block into shared memory, and its warps pull pixels
// from the tile with one aggregated atomic per warp (__ballot_sync over the lanes that need work,
// each lane's slot from the population count of the lanes below it). A lane runs one bounce per
// loop iteration; when its path ends it starts the pixel's next sample, and when the pixel's last
// sample ends it writes the pixel and takes another, so lanes with short paths keep working while
// others finish long ones. Each pixel's samples are accumulated by one lane in sample order: the
// image is a deterministic function of the seed.
#include "abi_internal.h"
#include "kernel_common.cuh"
#include "pt_sampling.cuh"
#include "denoise_common.cuh"

namespace mjpbr {
namespace {

constexpr int kThreads = 256;
constexpr int kTile = 32;
constexpr int kTilePixels = kTile * kTile;

struct PtTiles {
  int32_t ncam;
  int32_t tiles_x[MJPBR_MAX_RENDER];
  int32_t tile_base[MJPBR_MAX_RENDER + 1];  // per world
  int32_t tiles_per_world;
  int32_t total;
};

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

template <bool kMesh, bool kTex>
struct Pt {
  static MJ_DEV Hit trace(RtCtx& c, V3 o, V3 d, float max_dist, bool any) {
    return trace_ray<kMesh>(*c.s, c.st, c.blk, c.L, Ray{o, d}, max_dist, c.s->settings.cull_backfaces != 0, any, &c.err);
  }

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

  // Next-event estimate of one punctual light (its bulb disc for soft shadows).
  // out of line: one copy of the light-sampling code in the bounce loop (1 % faster measured)
  static __device__ __noinline__ V3 light_sample(RtCtx& c, Light light, const Lobes& lb, V3 point, V3 normal, V3 t1, V3 t2, V3 v, float u0,
                                float u1) {
    const MjpbrSettings& st = c.s->settings;
    if (light.type != MJPBR_LIGHT_DIRECTIONAL && light.bulbradius > 0.0f) {
      V3 b1, b2;
      orthonormal_basis(normalize(point - light.pos), &b1, &b2);
      float r = light.bulbradius * sqrtf(u0);
      float sn, cs;
      sincos_turns(u1, &sn, &cs);
      light.pos = light.pos + (b1 * cs + b2 * sn) * r;
    }
    V3 l, ds, ss;
    float dist;
    MJPBR_COUNT(kOpPtLight);
    eval_light(light, st.light_model, point, &l, &dist, &ds, &ss);
    V3 ll{dot(l, t1), dot(l, t2), dot(l, normal)};
    if (ll.z <= 0.0f || (length_sq(ds) == 0.0f && length_sq(ss) == 0.0f)) return v3(0.0f);
    if (st.use_shadows && light.castshadow) {
      float max_t = light.type == MJPBR_LIGHT_DIRECTIONAL ? kUnboundedShadow : dist - kShadowGap;
      if (trace(c, point + normal * kRayOffset, l, max_t, true).geom != -1) return v3(0.0f);
    }
    V3 diffuse = eval_bsdf_cos(lb.diffuse_color, v3(0.0f), lb.alpha, v3(0.0f), v, ll);
    V3 specular = eval_bsdf_cos(v3(0.0f), lb.f0, lb.alpha, lb.energy_comp, v, ll);
    return cmul(diffuse, ds) + cmul(specular, ss);
  }

  // One iteration of the bounce loop (pathtrace.py:230-337); true when the path has ended.
  static MJ_DEV bool bounce(RtCtx& c, PathState& ps, PixelAcc& acc, const Pixel& p, uint32_t seed, V3 head_dir) {
    const MjpbrScene& s = *c.s;
    const MjpbrSettings& st = s.settings;
    if (ps.depth > st.max_depth) return true;
    Hit hit = trace(c, ps.o, ps.d, ps.max_dist, false);
    if (ps.camera_ray && ps.passes == 0 && ps.sample == 0) {
      write_geometry(s, c.w, p, hit, ps.dcam_z);
      if (hit.geom != -1) acc.first_depth = hit.dist * -ps.dcam_z;
    }
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

    // next-event estimation: MuJoCo lights, then the headlight (no shadow, display-relative)
    const int32_t nl = c.L.nlight + (st.headlight_active ? 1 : 0);
    V3 direct = v3(0.0f);
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
      direct += light_sample(c, light, lb, point, normal, t1, t2, v, u0, u1);
    }
    ps.radiance += cmul(ps.beta, direct);

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
        if (trace(c, point + normal * kRayOffset, d_env, kUnboundedShadow, true).geom == -1) {
          float weight = power_heuristic(pdf_env, pdf_bsdf(lb.alpha, p_spec, v, le));
          ps.radiance += cmul(ps.beta, cmul(f, environment(c, d_env))) * (weight / pdf_env);
        }
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

template <bool kMesh, bool kTex>
__global__ void __launch_bounds__(kThreads, 2) pt_kernel(const __grid_constant__ MjpbrScene s, uint32_t seed,
                                                         const __grid_constant__ PtTiles tm) {
  extern __shared__ __align__(16) float smem[];
  __shared__ int32_t s_tile, s_next;
  float* blk = smem;
  const BlockLayout L = block_layout(s.nbvh_geom, s.nnode, s.nlight, s.nrender);
  const MjpbrSettings& st = s.settings;
  const int lane = threadIdx.x & 31;
  const unsigned full = 0xffffffffu;
  RtCtx c;
  {
    int32_t* stack_base = reinterpret_cast<int32_t*>(smem + s.world_block_floats);
    c.st.code = stack_base + threadIdx.x;
    c.st.t = reinterpret_cast<float*>(stack_base + kThreads * kStackDepth) + threadIdx.x;
    c.st.stride = kThreads;
  }
  int32_t err = 0;
  for (;;) {
    if (threadIdx.x == 0) s_tile = atomicAdd(s.work_counter, 1);
    __syncthreads();
    const int32_t tile = s_tile;
    if (tile >= tm.total) break;
    const int32_t w = tile / tm.tiles_per_world;
    const int32_t lt = tile - w * tm.tiles_per_world;
    int32_t cam = 0;
    while (cam + 1 < tm.ncam && lt >= tm.tile_base[cam + 1]) ++cam;
    const int32_t t = lt - tm.tile_base[cam];
    const int32_t tx = t % tm.tiles_x[cam], ty = t / tm.tiles_x[cam];
    stage_world_block(s, w, blk, kThreads);
    if (threadIdx.x == 0) s_next = 0;
    __syncthreads();
    init_ctx(c, s, blk, L, w, kTex);

    Pixel p;
    p.cam = cam;
    p.width = s.cam_res[cam][0];
    p.height = s.cam_res[cam][1];
    p.rec = blk + L.cam_off + cam * kCamFloats;
    const M3 R = cam_mat(p.rec);
    const V3 cpos{p.rec[0], p.rec[1], p.rec[2]};
    const V3 head_dir = -V3{R.m[2], R.m[5], R.m[8]};
    const bool want_rgb = s.render_rgb[cam] != 0;
    const int32_t nsample = st.path_samples;

    PathState ps;
    PixelAcc acc;
    uint32_t pixel_seed = 0;
    bool has_pixel = false, exhausted = false;
    for (;;) {
      const bool want = !has_pixel && !exhausted;
      const unsigned need = __ballot_sync(full, want);
      if (need) {
        const int leader = __ffs(need) - 1;
        int32_t base = 0;
        if (lane == leader) base = atomicAdd(&s_next, __popc(need));
        base = __shfl_sync(full, base, leader);
        if (want) {
          const int32_t idx = base + __popc(need & ((1u << lane) - 1u));
          if (idx >= kTilePixels) {
            exhausted = true;
          } else {
            p.px = tx * kTile + (idx % kTile);
            p.py = ty * kTile + (idx / kTile);
            if (p.px < p.width && p.py < p.height) {
              p.pixelid = p.py * p.width + p.px;
              if (!want_rgb) {
                // depth / segmentation only: the centre of the 15 x 15 grid
                V3 dcam, ocam;
                float max_dist, depth_z;
                primary_ray(s, p, kSubpixel, kSubpixel / 2, kSubpixel / 2, &dcam, &ocam, &max_dist, &depth_z);
                Hit hit = Pt<kMesh, kTex>::trace(c, cpos + mul(R, ocam), mul(R, dcam), max_dist, false);
                write_geometry(s, w, p, hit, depth_z);
              } else {
                pixel_seed = seed + (uint32_t)w * (uint32_t)s.total_rays + (uint32_t)(s.ray_adr[cam] + p.pixelid);
                acc.hdr = acc.albedo = acc.normal = acc.emission = v3(0.0f);
                acc.lum_sq = 0.0f;
                acc.first_depth = 0.0f;
                acc.guide_albedo = acc.guide_normal = v3(0.0f);
                start_sample(ps, s, p, pixel_seed, R, cpos, 0);
                has_pixel = true;
              }
            }
          }
        }
      }
      if (__all_sync(full, exhausted && !has_pixel)) break;
      if (!has_pixel) continue;
      if (!Pt<kMesh, kTex>::bounce(c, ps, acc, p, pixel_seed, head_dir)) continue;
      // the path ended: accumulate the sample
      acc.hdr += ps.radiance;
      acc.albedo += ps.albedo;
      acc.normal += ps.normal;
      acc.emission += ps.emission;
      if (ps.sample == 0) {
        acc.guide_albedo = ps.base_color;
        acc.guide_normal = ps.normal;
      }
      if (st.denoise) {
        float lum = luminance(ps.radiance) * c.exposure;
        acc.lum_sq += lum * lum;
      }
      if (ps.sample + 1 < nsample) {
        start_sample(ps, s, p, pixel_seed, R, cpos, ps.sample + 1);
        continue;
      }
      // the pixel's last sample: write it
      has_pixel = false;
      const float inv_n = 1.0f / (float)nsample;
      const V3 hdr = acc.hdr * inv_n;
      const int64_t adr = (int64_t)w * s.rgb_stride + s.rgb_adr[cam] + p.pixelid;
      if (st.render_guides && s.guide_albedo) {
        s.guide_albedo[adr * 3] = acc.guide_albedo.x;
        s.guide_albedo[adr * 3 + 1] = acc.guide_albedo.y;
        s.guide_albedo[adr * 3 + 2] = acc.guide_albedo.z;
        s.guide_normal[adr * 3] = acc.guide_normal.x;
        s.guide_normal[adr * 3 + 1] = acc.guide_normal.y;
        s.guide_normal[adr * 3 + 2] = acc.guide_normal.z;
      }
      if (st.denoise) {
        // noisy HDR, the filter's guide (normal and albedo at half precision), the exposed
        // first-hit emission and the demodulated radiance the first filter pass reads
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
    err |= c.err;
    __syncthreads();  // every lane done with this tile's block before the next one is staged
  }
  if (err && s.error_word) atomicOr(s.error_word, err);
}

template <bool kMesh, bool kTex>
int launch_variant(const MjpbrScene& s, uint32_t seed, const PtTiles& tm, cudaStream_t stream) {
  size_t smem = (size_t)s.world_block_floats * sizeof(float) + (size_t)kThreads * kStackDepth * 8;
  auto kern = pt_kernel<kMesh, kTex>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return set_error(MJPBR_ERR_CUDA, "path tracer: %zu bytes of shared memory: %s", smem, cudaGetErrorString(e));
  int grid = std::min(tm.total, device_sm_count() * 2);
  e = cudaMemsetAsync(s.work_counter, 0, 4 * sizeof(int32_t), stream);
  if (e != cudaSuccess) return set_error(MJPBR_ERR_CUDA, "path tracer: work counter: %s", cudaGetErrorString(e));
  kern<<<grid, kThreads, smem, stream>>>(s, seed, tm);
  return check_launch("pt_kernel");
}

}  // namespace

int render_pt_launch(const MjpbrScene& s, uint32_t seed, cudaStream_t stream) {
  if (!s.work_counter) return set_error(MJPBR_ERR_ARG, "the path tracer needs the work_counter scratch");
  if (s.settings.path_samples < 1 || s.settings.max_depth < 0) return set_error(MJPBR_ERR_ARG, "bad path-tracer settings");
  if (s.settings.denoise && (!s.hdr_data || !s.aov_guide || !s.aov_emission || !s.denoise_buffers[0])) {
    return set_error(MJPBR_ERR_ARG, "denoise needs the hdr, guide, emission and denoise buffers");
  }
  PtTiles tm;
  tm.ncam = s.nrender;
  tm.tile_base[0] = 0;
  for (int32_t c = 0; c < s.nrender; ++c) {
    int32_t W = s.cam_res[c][0], H = s.cam_res[c][1];
    bool any = s.render_rgb[c] || s.render_depth[c] || s.render_seg[c];
    tm.tiles_x[c] = (W + kTile - 1) / kTile;
    int32_t ty = (H + kTile - 1) / kTile;
    tm.tile_base[c + 1] = tm.tile_base[c] + (any ? tm.tiles_x[c] * ty : 0);
  }
  tm.tiles_per_world = tm.tile_base[s.nrender];
  tm.total = tm.tiles_per_world * s.nworld;
  if (tm.total == 0) return MJPBR_OK;
  bool mesh = s.nmesh + s.nhfield > 0 && s.blas_root != nullptr;
  bool tex = s.settings.textures || s.settings.has_env || s.settings.env_background;
  if (mesh && tex) return launch_variant<true, true>(s, seed, tm, stream);
  if (mesh) return launch_variant<true, false>(s, seed, tm, stream);
  if (tex) return launch_variant<false, true>(s, seed, tm, stream);
  return launch_variant<false, false>(s, seed, tm, stream);
}

}  // namespace mjpbr

#ifdef MJPBR_COUNT_OPS
namespace mjpbr {
// Counting build only: this unit's copy of the counter array pointer (set by mjpbr_count_set).
int pt_count_set(void* counts) { return cudaMemcpyToSymbol(g_op_counts, &counts, sizeof(counts)) == cudaSuccess ? 0 : 1; }
}  // namespace mjpbr
#endif
