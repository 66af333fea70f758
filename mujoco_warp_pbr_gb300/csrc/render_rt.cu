// Real-time tier megakernel (mujoco_warp_pbr/_src/render.py:78-427 and camera.py:113-347).
//
// Work decomposition: one CTA of 256 threads per (world, camera tile). A tile is 32x8 pixels
// (RenderOrder.ROW: a warp covers 32 pixels of one row) or 16x16 pixels made of 8x4 warp tiles
// (RenderOrder.TILED). The CTA copies its world's block (BVH nodes, geom/light/camera records,
// written by mjpbr_refit_bvh) into shared memory once; every thread then renders one pixel:
// N x N supersamples, each a primary ray, surface evaluation, split-sum ambient, direct lights
// with (soft) shadow rays, one optional mirror ray and translucent layers, tone mapped per sample,
// averaged and sRGB-encoded. Depth, segmentation and guides come from the first sample.
//
// Pixels are addressed by camera and row-major pixel id; the random numbers of a pixel are keyed
// by that id, so every thread order renders identical images.
#include <algorithm>
#include <climits>

#include "abi_internal.h"
#include "rt_shade.cuh"

namespace mjpbr {
namespace {

constexpr int kThreads = 256;
// Resident CTAs per SM the register allocation targets (the register / occupancy trade-off).
#ifndef MJPBR_RT_MIN_BLOCKS
#define MJPBR_RT_MIN_BLOCKS 2
#endif
constexpr float kMinThroughput = 1.0f / 255.0f;

// Shadow visibility of the megakernel: the shadow rays are traced where the shading asks.
template <bool kMesh>
struct TracedVis {
  MJ_DEV float visibility(RtCtx& c, const Light& light, V3 point, V3 normal, V3 l, float dist, uint32_t seed, int32_t stream,
                          int32_t nlight, int32_t li) {
    const MjpbrSettings& st = c.s->settings;
    const V3 origin = point + normal * kRayOffset;
    const int32_t nray = shadow_ray_count(light, st.shadow_samples);
    const bool cull = st.cull_backfaces != 0;
    int32_t visible = 0;
    for (int32_t k = 0; k < nray; ++k) {
      Ray r;
      float max_dist;
      r.o = origin;
      shadow_ray(light, st.shadow_samples, origin, l, dist, seed, stream, nlight, li, k, &r.d, &max_dist);
      if (trace_ray<kMesh>(*c.s, c.st, c.blk, c.L, r, max_dist, cull, true, &c.err).geom == -1) ++visible;
    }
    return visible_fraction(light, st.shadow_samples, visible, st.shadow_light_fraction);
  }
};

template <bool kMesh, bool kTex>
struct Rt {
  using Shade = RtShade<kTex, TracedVis<kMesh>>;

  static MJ_DEV V3 shade_surface(RtCtx& c, const Surface& sf, V3 point, V3 normal, V3 view, V3 head_dir, uint32_t seed,
                                 int32_t stream) {
    TracedVis<kMesh> vis;
    return Shade::shade_surface(c, vis, sf, point, normal, view, head_dir, seed, stream);
  }

  static MJ_DEV V3 background(RtCtx& c, V3 d, float spread) { return Shade::background(c, d, spread); }

  // Radiance along a camera ray, its first hit, and that surface's base colour and normal
  // (render.py:242-341). Translucent layers and the one-bounce mirror ray of each layer are
  // segments of a single loop, so the closest-hit / surface / shading code exists once in the
  // kernel: layer i adds shaded_i (1 - m_i) w_i and schedules its mirror segment with weight
  // m_i w_i (w_i = throughput_i * opacity_i), whose surface is shaded without further mirrors.
  static MJ_DEV V3 trace_pixel(RtCtx& c, V3 origin, V3 dir, float max_dist, float footprint, float spread, V3 head_dir,
                               uint32_t seed, int32_t stream, Hit* first, V3* albedo, V3* gnormal) {
    const MjpbrScene& s = *c.s;
    const MjpbrSettings& st = s.settings;
    const bool cull = st.cull_backfaces != 0;
    const int32_t nlayer = st.has_transparency ? st.max_layers : 1;
    V3 radiance = v3(0.0f);
    float throughput = 1.0f, travelled = 0.0f;
    int32_t layer = 0;
    // primary continuation (next translucent layer)
    V3 po = origin;
    bool have_primary = true;
    // current segment
    V3 so = origin, sd = dir;
    float smax = max_dist, sweight = 1.0f, sfoot = footprint;
    bool mirror_seg = false;
#pragma unroll 1
    for (int32_t iter = 0; iter < 2 * nlayer; ++iter) {
      Ray ray{so, sd};
      Hit hit = trace_ray<kMesh>(s, c.st, c.blk, c.L, ray, smax, cull, false, &c.err);
      if (!mirror_seg && layer == 0) *first = hit;
      bool cont = false;
      if (hit.geom == -1) {
        radiance += background(c, sd, spread) * (mirror_seg ? sweight : throughput);
        if (mirror_seg) cont = have_primary;
      } else {
        V3 point = so + sd * hit.dist;
        float cone = mirror_seg ? sfoot + spread * hit.dist : footprint + spread * (travelled + hit.dist);
        V3 normal;
        Surface sf = eval_surface<kMesh, kTex>(s, c.blk, c.L, c.w, hit, hit.slot, point, sd, cone, &normal);
        if (!mirror_seg && layer == 0) {
          *albedo = sf.base_color;
          *gnormal = normal;
        }
        V3 shaded = shade_surface(c, sf, point, normal, -sd, head_dir, seed, mirror_seg ? stream + 1 : stream);
        if (mirror_seg) {
          radiance += shaded * sweight;
          cont = have_primary;
        } else {
          float mirror = st.has_reflection ? mirror_reflectance(c, hit.slot) : 0.0f;
          float opacity = st.has_transparency ? clampf(sf.alpha, 0.0f, 1.0f) : 1.0f;
          float w = throughput * opacity;
          radiance += shaded * ((1.0f - mirror) * w);
          have_primary = false;
          if (st.has_transparency) {
            throughput *= 1.0f - opacity;
            if (throughput >= kMinThroughput && layer + 1 < nlayer) {
              travelled += hit.dist;
              po = point + sd * kRayOffset;
              have_primary = true;
            }
          }
          if (mirror > 0.0f) {
            // the mirror segment of this layer, then the next layer (if any)
            V3 r;
            mirror_ray(point, normal, sd, &so, &r);
            sd = r;
            smax = kMaxVal;
            sweight = mirror * w;
            sfoot = cone;
            mirror_seg = true;
            if (have_primary) ++layer;
            continue;
          }
          if (have_primary) ++layer;
          cont = have_primary;
        }
      }
      if (!cont) break;
      // next primary layer
      so = po;
      sd = dir;
      smax = max_dist - travelled;
      mirror_seg = false;
      have_primary = true;
    }
    return radiance;
  }
};

// Renders pixel p of world w (render.py:343-395) from the world block blk: N x N supersamples,
// depth / segmentation / guides from the first one, tone mapped per sample, averaged and encoded.
template <bool kMesh, bool kTex>
MJ_DEV void render_pixel(const MjpbrScene& s, uint32_t seed, const float* blk, const BlockLayout& L, int32_t w, Pixel& p,
                         const Stack& stack) {
  const int32_t cam = p.cam;
  p.pixelid = p.py * p.width + p.px;
  p.rec = blk + L.cam_off + cam * kCamFloats;
  const bool want_rgb = s.render_rgb[cam] != 0;
  const MjpbrSettings& st = s.settings;
  RtCtx c;
  c.st = stack;
  init_ctx(c, s, blk, L, w, kTex);
  const M3 R = cam_mat(p.rec);
  const V3 cpos{p.rec[0], p.rec[1], p.rec[2]};
  const bool cull = st.cull_backfaces != 0;

  if (!want_rgb) {
    V3 dcam, ocam;
    float max_dist, depth_z;
    primary_ray(s, p, 1, 0, 0, &dcam, &ocam, &max_dist, &depth_z);
    Ray ray{cpos + mul(R, ocam), mul(R, dcam)};
    Hit hit = trace_ray<kMesh>(s, c.st, blk, L, ray, max_dist, cull, false, &c.err);
    write_geometry(s, w, p, hit, depth_z);
    if (c.err && s.error_word) atomicOr(s.error_word, c.err);
    return;
  }

  const int32_t n = st.samples_per_axis;
  const float inv_n = 1.0f / (float)n;
  float pixel_spread, pixel_width;
  pixel_cone(s, p, &pixel_spread, &pixel_width);
  const float spread = pixel_spread * inv_n, width = pixel_width * inv_n;
  const V3 head_dir = -V3{R.m[2], R.m[5], R.m[8]};
  const uint32_t pixel_seed = seed + (uint32_t)w * (uint32_t)s.total_rays + (uint32_t)(s.ray_adr[cam] + p.pixelid);

  V3 display = v3(0.0f), hdr = v3(0.0f);
  for (int32_t smp = 0; smp < n * n; ++smp) {
    V3 dcam, ocam;
    float max_dist, depth_z;
    primary_ray(s, p, n, smp % n, smp / n, &dcam, &ocam, &max_dist, &depth_z);
    V3 origin = cpos + mul(R, ocam);
    V3 dir = mul(R, dcam);
    Hit first;
    V3 albedo = v3(0.0f), gnormal = v3(0.0f);
    V3 radiance = Rt<kMesh, kTex>::trace_pixel(c, origin, dir, max_dist, width, spread, head_dir, pixel_seed, 2 * smp,
                                               &first, &albedo, &gnormal);
    if (smp == 0) {
      write_geometry(s, w, p, first, depth_z);
      if (st.render_guides && s.guide_albedo) {
        int64_t a = ((int64_t)w * s.rgb_stride + s.rgb_adr[cam] + p.pixelid) * 3;
        V3 al = first.geom != -1 ? albedo : v3(0.0f), nm = first.geom != -1 ? gnormal : v3(0.0f);
        s.guide_albedo[a] = al.x;
        s.guide_albedo[a + 1] = al.y;
        s.guide_albedo[a + 2] = al.z;
        s.guide_normal[a] = nm.x;
        s.guide_normal[a + 1] = nm.y;
        s.guide_normal[a + 2] = nm.z;
      }
    }
    display += display_transform(radiance * c.exposure, st.tone_mapper);
    hdr += radiance;
  }
  const int64_t adr = (int64_t)w * s.rgb_stride + s.rgb_adr[cam] + p.pixelid;
  const float inv_nn = inv_n * inv_n;
  if (st.render_hdr && s.hdr_data) {
    s.hdr_data[adr * 3] = hdr.x * inv_nn;
    s.hdr_data[adr * 3 + 1] = hdr.y * inv_nn;
    s.hdr_data[adr * 3 + 2] = hdr.z * inv_nn;
  }
  s.rgb_data[adr] = encode_display(display * inv_nn);
  if (c.err && s.error_word) atomicOr(s.error_word, c.err);
}

// Four consecutive lanes render the 2 x 2 supersamples of one pixel (sample = lane & 3): the
// samples of a pixel are nearly the same ray, so a warp's lanes stay on one code path far more
// often than with 32 pixels per warp (5 % faster on the mesh / IBL workload). The pixel's first lane
// sums the four results in sample order (warp shuffles), which are the sums of render_pixel's
// sequential loop, so the images are identical. Every lane of the warp must make the call;
// `valid` false marks lanes past the image edge.
template <bool kMesh, bool kTex>
MJ_DEV void render_pixel_lanes(const MjpbrScene& s, uint32_t seed, const float* blk, const BlockLayout& L, int32_t w,
                               Pixel& p, bool valid, int32_t smp, const Stack& stack) {
  const int32_t cam = p.cam;
  const MjpbrSettings& st = s.settings;
  RtCtx c;
  c.st = stack;
  init_ctx(c, s, blk, L, w, kTex);
  V3 display = v3(0.0f), hdr = v3(0.0f);
  if (valid) {
    p.pixelid = p.py * p.width + p.px;
    p.rec = blk + L.cam_off + cam * kCamFloats;
    const M3 R = cam_mat(p.rec);
    const V3 cpos{p.rec[0], p.rec[1], p.rec[2]};
    const int32_t n = 2;
    const float inv_n = 1.0f / (float)n;
    float pixel_spread, pixel_width;
    pixel_cone(s, p, &pixel_spread, &pixel_width);
    const float spread = pixel_spread * inv_n, width = pixel_width * inv_n;
    const V3 head_dir = -V3{R.m[2], R.m[5], R.m[8]};
    const uint32_t pixel_seed = seed + (uint32_t)w * (uint32_t)s.total_rays + (uint32_t)(s.ray_adr[cam] + p.pixelid);
    V3 dcam, ocam;
    float max_dist, depth_z;
    primary_ray(s, p, n, smp % n, smp / n, &dcam, &ocam, &max_dist, &depth_z);
    V3 origin = cpos + mul(R, ocam);
    V3 dir = mul(R, dcam);
    Hit first;
    V3 albedo = v3(0.0f), gnormal = v3(0.0f);
    V3 radiance = Rt<kMesh, kTex>::trace_pixel(c, origin, dir, max_dist, width, spread, head_dir, pixel_seed, 2 * smp,
                                               &first, &albedo, &gnormal);
    if (smp == 0) {
      write_geometry(s, w, p, first, depth_z);
      if (st.render_guides && s.guide_albedo) {
        int64_t a = ((int64_t)w * s.rgb_stride + s.rgb_adr[cam] + p.pixelid) * 3;
        V3 al = first.geom != -1 ? albedo : v3(0.0f), nm = first.geom != -1 ? gnormal : v3(0.0f);
        s.guide_albedo[a] = al.x;
        s.guide_albedo[a + 1] = al.y;
        s.guide_albedo[a + 2] = al.z;
        s.guide_normal[a] = nm.x;
        s.guide_normal[a + 1] = nm.y;
        s.guide_normal[a + 2] = nm.z;
      }
    }
    display = v3(0.0f) + display_transform(radiance * c.exposure, st.tone_mapper);
    hdr = v3(0.0f) + radiance;
  }
  const unsigned full = 0xffffffffu;
  V3 sd = display, sh = hdr;
#pragma unroll
  for (int k = 1; k < 4; ++k) {
    sd += V3{__shfl_down_sync(full, display.x, k), __shfl_down_sync(full, display.y, k), __shfl_down_sync(full, display.z, k)};
    sh += V3{__shfl_down_sync(full, hdr.x, k), __shfl_down_sync(full, hdr.y, k), __shfl_down_sync(full, hdr.z, k)};
  }
  if (valid && smp == 0) {
    const int64_t adr = (int64_t)w * s.rgb_stride + s.rgb_adr[cam] + p.pixelid;
    const float inv_nn = 0.25f;
    if (st.render_hdr && s.hdr_data) {
      s.hdr_data[adr * 3] = sh.x * inv_nn;
      s.hdr_data[adr * 3 + 1] = sh.y * inv_nn;
      s.hdr_data[adr * 3 + 2] = sh.z * inv_nn;
    }
    s.rgb_data[adr] = encode_display(sd * inv_nn);
  }
  if (c.err && s.error_word) atomicOr(s.error_word, c.err);
}

MJ_DEV Stack thread_stack(const MjpbrScene& s, float* stacks) {
  return shared_stack(stacks, kThreads, stack_entries(s.settings.stack_depth));
}

// Grid schedule: one CTA per (camera tile, world); the hardware scheduler balances the CTAs.
template <bool kMesh, bool kTex, bool kStaged>
__global__ void __launch_bounds__(kThreads, MJPBR_RT_MIN_BLOCKS) rt_kernel(const __grid_constant__ MjpbrScene s, uint32_t seed,
                                                                           const __grid_constant__ TileMap tm) {
  extern __shared__ __align__(16) float smem[];
  const int32_t w = tm.w0 + blockIdx.y;
  const float* blk = world_block_of<kStaged>(s, w, smem, kThreads);
  __syncthreads();
  float* const stack_base = smem + (kStaged ? s.world_block_floats : 0);
  const BlockLayout L = block_layout(s.nbvh_geom, s.nnode, s.nlight, s.nrender);
  const int32_t tile = blockIdx.x;
  int32_t cam = 0;
  while (cam + 1 < tm.ncam && tile >= tm.tile_base[cam + 1]) ++cam;
  const int32_t t = tile - tm.tile_base[cam];
  const int32_t tx = t % tm.tiles_x[cam], ty = t / tm.tiles_x[cam];
  Pixel p;
  p.cam = cam;
  p.width = s.cam_res[cam][0];
  p.height = s.cam_res[cam][1];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (s.settings.samples_per_axis == 2 && s.render_rgb[cam] != 0) {
    // sample lanes: 4 passes of 64 pixels, each warp a 4 x 2 pixel block (ROW tiles of 32 x 8 in
    // passes of 2 rows, TILED tiles of 16 x 16 in 8 x 8 quadrants)
    const Stack st = thread_stack(s, stack_base);
    const bool row = s.settings.render_order == MJPBR_ORDER_ROW;
    const int32_t smp = lane & 3, pix = lane >> 2;
#pragma unroll 1
    for (int q = 0; q < 4; ++q) {
      Pixel pp = p;
      if (row) {
        pp.px = tx * 32 + warp * 4 + (pix & 3);
        pp.py = ty * 8 + q * 2 + (pix >> 2);
      } else {
        pp.px = tx * 16 + (q & 1) * 8 + (warp & 1) * 4 + (pix & 3);
        pp.py = ty * 16 + (q >> 1) * 8 + (warp >> 1) * 2 + (pix >> 2);
      }
      const bool valid = pp.px < pp.width && pp.py < pp.height;
      render_pixel_lanes<kMesh, kTex>(s, seed, blk, L, w, pp, valid, smp, st);
    }
    return;
  }
  if (s.settings.render_order == MJPBR_ORDER_ROW) {
    p.px = tx * 32 + lane;
    p.py = ty * 8 + warp;
  } else {
    p.px = tx * 16 + (warp & 1) * 8 + (lane & 7);
    p.py = ty * 16 + (warp >> 1) * 4 + (lane >> 3);
  }
  if (p.px >= p.width || p.py >= p.height) return;
  render_pixel<kMesh, kTex>(s, seed, blk, L, w, p, thread_stack(s, stack_base));
}

// Work items of the queue schedule: runs of `per_item` warp tiles (8 x 4 pixels) of one camera
// image of one world, world-major.
struct QueueMap {
  int32_t ncam;
  int32_t per_item;                         // warp tiles per item
  int32_t wtiles_x[MJPBR_MAX_RENDER];       // warp tiles per row of each camera
  int32_t wtiles[MJPBR_MAX_RENDER];         // warp tiles of each camera
  int32_t item_base[MJPBR_MAX_RENDER + 1];  // first item of each camera within a world
  int32_t items_per_world;
  int32_t total;
};

// Queue schedule: a persistent launch (resident CTAs only) whose warps pull work items from a
// device counter. Each warp keeps its own copy of the current item's world block in shared
// memory (re-staged only when the world changes), so warps never wait for one another: uneven
// cameras, enable masks and per-pixel costs balance at warp granularity.
template <bool kMesh, bool kTex>
__global__ void __launch_bounds__(kThreads, MJPBR_RT_MIN_BLOCKS) rt_queue_kernel(const __grid_constant__ MjpbrScene s, uint32_t seed,
                                                                                 const __grid_constant__ QueueMap qm) {
  extern __shared__ __align__(16) float smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned full = 0xffffffffu;
  float* blk = smem + warp * s.world_block_floats;
  const Stack stack = thread_stack(s, smem + (kThreads / 32) * s.world_block_floats);
  const BlockLayout L = block_layout(s.nbvh_geom, s.nnode, s.nlight, s.nrender);
  int32_t staged = -1;
  for (;;) {
    int32_t item = 0;
    if (lane == 0) item = atomicAdd(s.work_counter + 1, 1);
    item = __shfl_sync(full, item, 0);
    if (item >= qm.total) break;
    const int32_t w = item / qm.items_per_world;
    const int32_t li = item - w * qm.items_per_world;
    int32_t cam = 0;
    while (cam + 1 < qm.ncam && li >= qm.item_base[cam + 1]) ++cam;
    if (w != staged) {
      __syncwarp();
      const float4* src = reinterpret_cast<const float4*>(s.world_blocks + (int64_t)w * s.world_block_floats);
      float4* dst = reinterpret_cast<float4*>(blk);
      for (int32_t i = lane; i < (s.world_block_floats >> 2); i += 32) dst[i] = __ldg(src + i);
      __syncwarp();
      staged = w;
    }
    const int32_t first = (li - qm.item_base[cam]) * qm.per_item;
#pragma unroll 1
    for (int32_t j = 0; j < qm.per_item; ++j) {
      const int32_t wt = first + j;
      if (wt >= qm.wtiles[cam]) break;
      Pixel p;
      p.cam = cam;
      p.width = s.cam_res[cam][0];
      p.height = s.cam_res[cam][1];
      p.px = (wt % qm.wtiles_x[cam]) * 8 + (lane & 7);
      p.py = (wt / qm.wtiles_x[cam]) * 4 + (lane >> 3);
      if (p.px < p.width && p.py < p.height) render_pixel<kMesh, kTex>(s, seed, blk, L, w, p, stack);
    }
  }
}

// Largest dynamic shared memory a CTA may use while MJPBR_RT_MIN_BLOCKS CTAs stay resident.
constexpr size_t kSmemPerSm = 228 * 1024;
constexpr size_t kQueueSmemLimit = kSmemPerSm / MJPBR_RT_MIN_BLOCKS - 2048;

size_t stack_bytes(const MjpbrScene& s) { return (size_t)kThreads * stack_entries(s.settings.stack_depth) * 8; }

template <bool kMesh, bool kTex, bool kStaged>
int launch_variant(const MjpbrScene& s, uint32_t seed, const TileMap& tm, cudaStream_t stream) {
  const size_t smem = (kStaged ? (size_t)s.world_block_floats * sizeof(float) : 0) + stack_bytes(s);
  auto kern = rt_kernel<kMesh, kTex, kStaged>;
  if (int rc = ensure_smem(reinterpret_cast<const void*>(kern), smem, "render")) return rc;
  TileMap part = tm;
  for (int32_t w0 = 0; w0 < s.nworld; w0 += kMaxGridWorlds) {
    part.w0 = w0;
    const dim3 grid(tm.tile_base[tm.ncam], std::min(kMaxGridWorlds, s.nworld - w0));
    kern<<<grid, kThreads, smem, stream>>>(s, seed, part);
    const int rc = check_launch("rt_kernel");
    if (rc) return rc;
  }
  return MJPBR_OK;
}

template <bool kMesh, bool kTex>
int launch_queue_variant(const MjpbrScene& s, uint32_t seed, const QueueMap& qm, cudaStream_t stream) {
  const size_t smem = (size_t)(kThreads / 32) * s.world_block_floats * sizeof(float) + stack_bytes(s);
  auto kern = rt_queue_kernel<kMesh, kTex>;
  if (int rc = ensure_smem(reinterpret_cast<const void*>(kern), smem, "render queue")) return rc;
  cudaError_t e = cudaMemsetAsync(s.work_counter + 1, 0, sizeof(int32_t), stream);
  if (e != cudaSuccess) return set_error(MJPBR_ERR_CUDA, "render queue: work counter: %s", cudaGetErrorString(e));
  const int grid = std::min(qm.total, device_sm_count() * MJPBR_RT_MIN_BLOCKS);
  kern<<<grid, kThreads, smem, stream>>>(s, seed, qm);
  return check_launch("rt_queue_kernel");
}

int render_rt_queue(const MjpbrScene& s, uint32_t seed, cudaStream_t stream) {
  QueueMap qm;
  qm.ncam = s.nrender;
  qm.per_item = std::max(1, s.settings.queue_item / 32);
  qm.item_base[0] = 0;
  for (int32_t c = 0; c < s.nrender; ++c) {
    const int32_t W = s.cam_res[c][0], H = s.cam_res[c][1];
    const bool any = s.render_rgb[c] || s.render_depth[c] || s.render_seg[c];
    qm.wtiles_x[c] = (W + 7) / 8;
    qm.wtiles[c] = any ? qm.wtiles_x[c] * ((H + 3) / 4) : 0;
    qm.item_base[c + 1] = qm.item_base[c] + (qm.wtiles[c] + qm.per_item - 1) / qm.per_item;
  }
  qm.items_per_world = qm.item_base[s.nrender];
  const int64_t total = (int64_t)qm.items_per_world * s.nworld;
  if (total == 0) return MJPBR_OK;
  if (total > INT32_MAX) return set_error(MJPBR_ERR_ARG, "render queue: %lld work items exceed the counter", (long long)total);
  qm.total = (int32_t)total;
  const bool mesh = s.nmesh + s.nhfield > 0 && s.blas_root != nullptr;
  const bool tex = s.settings.textures || s.settings.has_env || s.settings.env_background;
  if (mesh && tex) return launch_queue_variant<true, true>(s, seed, qm, stream);
  if (mesh) return launch_queue_variant<true, false>(s, seed, qm, stream);
  if (tex) return launch_queue_variant<false, true>(s, seed, qm, stream);
  return launch_queue_variant<false, false>(s, seed, qm, stream);
}

}  // namespace

// True when the queue schedule's per-warp world blocks fit the shared memory of the resident CTAs.
bool rt_queue_fits(const MjpbrScene& s) {
  return (size_t)(kThreads / 32) * s.world_block_floats * sizeof(float) + stack_bytes(s) <= kQueueSmemLimit;
}

int render_rt_launch(const MjpbrScene& s, uint32_t seed, cudaStream_t stream) {
  // scenes the wavefront does not stage (translucent layers, more than 65535 geoms) render with the
  // grid schedule (same images)
  if (s.settings.schedule == MJPBR_SCHEDULE_WAVEFRONT && wave_supported(s)) return render_wave_launch(s, seed, stream);
  if (s.settings.schedule == MJPBR_SCHEDULE_QUEUE) {
    if (!s.work_counter) return set_error(MJPBR_ERR_ARG, "the queue schedule needs the work_counter scratch");
    if (!rt_queue_fits(s)) {
      return set_error(MJPBR_ERR_ARG, "queue schedule: 8 world blocks of %d floats do not fit shared memory; use the grid schedule",
                       s.world_block_floats);
    }
    return render_rt_queue(s, seed, stream);
  }
  TileMap tm;
  tm.w0 = 0;
  tm.ncam = s.nrender;
  if (s.settings.render_order == MJPBR_ORDER_ROW) {
    tm.tile_w = 32;
    tm.tile_h = 8;
  } else {
    tm.tile_w = 16;
    tm.tile_h = 16;
  }
  tm.tile_base[0] = 0;
  for (int32_t c = 0; c < s.nrender; ++c) {
    int32_t W = s.cam_res[c][0], H = s.cam_res[c][1];
    bool any = s.render_rgb[c] || s.render_depth[c] || s.render_seg[c];
    tm.tiles_x[c] = (W + tm.tile_w - 1) / tm.tile_w;
    int32_t ty = (H + tm.tile_h - 1) / tm.tile_h;
    tm.tile_base[c + 1] = tm.tile_base[c] + (any ? tm.tiles_x[c] * ty : 0);
  }
  if (tm.tile_base[s.nrender] == 0 || s.nworld == 0) return MJPBR_OK;
  bool mesh = s.nmesh + s.nhfield > 0 && s.blas_root != nullptr;
  bool tex = s.settings.textures || s.settings.has_env || s.settings.env_background;
  if (world_block_staged(s.world_block_floats, stack_bytes(s))) {
    if (mesh && tex) return launch_variant<true, true, true>(s, seed, tm, stream);
    if (mesh) return launch_variant<true, false, true>(s, seed, tm, stream);
    if (tex) return launch_variant<false, true, true>(s, seed, tm, stream);
    return launch_variant<false, false, true>(s, seed, tm, stream);
  }
  // world blocks too large for shared memory are read in place
  if (mesh && tex) return launch_variant<true, true, false>(s, seed, tm, stream);
  if (mesh) return launch_variant<true, false, false>(s, seed, tm, stream);
  if (tex) return launch_variant<false, true, false>(s, seed, tm, stream);
  return launch_variant<false, false, false>(s, seed, tm, stream);
}

}  // namespace mjpbr

#ifdef MJPBR_COUNT_OPS
namespace mjpbr {
int pt_count_set(void* counts);
int wave_count_set(void* counts);
int pt_wave_count_set(void* counts);
}

// Counting build only: the device array (kOpCountN x kOpCopies uint64) the real-time and path
// kernels add to, or NULL.
extern "C" int mjpbr_count_set(void* counts) {
  if (cudaMemcpyToSymbol(mjpbr::g_op_counts, &counts, sizeof(counts)) != cudaSuccess) return 1;
  return mjpbr::pt_count_set(counts) | mjpbr::wave_count_set(counts) | mjpbr::pt_wave_count_set(counts);
}
#endif
