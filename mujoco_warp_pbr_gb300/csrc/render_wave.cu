// Real-time tier as a staged wavefront (the schedule MJPBR_SCHEDULE_WAVEFRONT): the per-sample
// work of mujoco_warp_pbr/_src/render.py:242-395 split into kernels that each run one stage over
// every sample of a chunk of worlds, with compacted ray queues between them:
//
//   1. primary    one thread per camera sample: camera ray, closest hit -> hit record;
//                 depth / segmentation of the pixel from its first sample
//   2. surface 0  eval_surface at the primary hit -> surface record; every light the shading will
//                 ask about appends one shadow entry, a reflective surface one mirror ray
//   3. mirror     closest hit of every queued mirror ray -> hit record (persistent; lanes take a
//                 new ray as soon as theirs is done: refill.cuh)
//   4. surface 1  eval_surface at the mirror hit -> surface record, shadow entries
//   5. shadow     every shadow entry's rays (any hit, persistent with lane refill) -> count of
//                 unoccluded rays
//   6. resolve    one thread per camera sample: the shading of both segments with the stored
//                 counts, tone map; the pixel's first thread averages its samples in sample
//                 order and encodes; guides
//
// Each stage has its own small register budget and instruction footprint, and its warps run one
// kind of work (the megakernel interleaves traversal, texturing and shading in every warp and is
// bound by instruction fetch and divergence). Queues are filled with one atomic per CTA
// (__ballot_sync / __popc offsets within a warp, a shared-memory scan over the warps), so each
// CTA's entries form one run in its pixel order and the tracing warps get neighbouring rays of one
// world. The shading of stage 6 is the megakernel's own code (rt_shade.cuh)
// with the shadow visibility read from the counts instead of traced where it is needed, and the
// rays of stages 3-5 are set up by the same functions, so the images are bit-identical to the
// megakernel's. Translucent layers are not staged: contexts with has_transparency render with the
// megakernel.
//
// Scratch (MjpbrScene.wave_scratch): per sample of a chunk two hit records (32 B), two surface
// records (64 B), a mirror queue entry (48 B) and per model light two visibility counts (8 B) and
// two shadow entries (64 B); the library renders as many worlds per chunk as the scratch holds.
#include <algorithm>
#include <climits>
#include <vector>

#include "abi_internal.h"
#include "refill.cuh"
#include "rt_shade.cuh"

namespace mjpbr {
namespace {

constexpr int kThreads = 256;
constexpr int kTile = 16;  // pixel tiles of 16 x 16, addressed in Z order within the tile
// Resident CTAs per SM the register allocation of the ray-tracing stages (primary, mirror,
// shadow: 64 KB of traversal stacks per CTA) and of the surface / shading stages targets.
#ifndef MJPBR_WAVE_TRACE_CTAS
#define MJPBR_WAVE_TRACE_CTAS 3
#endif
#ifndef MJPBR_WAVE_MIRROR_CTAS
#define MJPBR_WAVE_MIRROR_CTAS 3
#endif
#ifndef MJPBR_WAVE_SHADE_CTAS
#define MJPBR_WAVE_SHADE_CTAS 3
#endif

struct __align__(16) HitRec {
  float dist;
  int32_t ref;  // -1: miss; else slot | (mesh + 1) << 16
  int32_t face;
  float u, v;
  float nx, ny, nz;
};

struct __align__(16) SurfRec {
  float4 a;  // base colour, metallic
  float4 b;  // roughness, reflectance, occlusion, hit distance
  float4 c;  // emissive, slot (int bits; -1: the segment missed)
  float4 d;  // shading normal (world), alpha
};

struct __align__(16) MirrorEntry {
  float4 o;    // origin, cone footprint at the reflecting surface
  float4 d;    // direction, pixel spread
  int4 index;  // x: sample
};

struct __align__(16) ShadowEntry {
  float4 o;  // origin (offset along the shading normal), distance to the light
  float4 l;  // direction to the light (centre), target (int bits): (sample * 2 + segment) * nlight + light
};

constexpr int64_t kHitBytes = sizeof(HitRec), kSurfBytes = sizeof(SurfRec), kMirrorBytes = sizeof(MirrorEntry),
                  kShadowBytes = sizeof(ShadowEntry);
static_assert(sizeof(HitRec) == 32 && sizeof(SurfRec) == 64 && sizeof(MirrorEntry) == 48 && sizeof(ShadowEntry) == 32,
              "record sizes");

struct WaveMap {
  int32_t w0, nw;        // worlds of this chunk
  int32_t nn;            // samples per pixel (samples_per_axis^2)
  int32_t per_world;     // samples per world over the RGB cameras
  int32_t nl;            // model lights
  int32_t sample_base[MJPBR_MAX_RENDER];  // first sample of each RGB camera within a world
  TileMap geo;           // tiles of every camera with an output
  TileMap rgb;           // tiles of the RGB cameras
  HitRec* hit[2];
  SurfRec* surf[2];
  int32_t* vis;          // (sample, segment, light) unoccluded shadow rays
  MirrorEntry* mirror;
  ShadowEntry* shadow;
  int32_t* counters;     // [0] mirror entries, [1] shadow entries; 64-bit fetch counters of the shadow [2..3] and mirror [4..5] stages
  int64_t mirror_cap, shadow_cap;
};

MJ_DEV int32_t z_x(int32_t q) { return (q & 1) | ((q >> 1) & 2) | ((q >> 2) & 4) | ((q >> 3) & 8); }
MJ_DEV int32_t z_y(int32_t q) { return ((q >> 1) & 1) | ((q >> 2) & 2) | ((q >> 3) & 4) | ((q >> 4) & 8); }

MJ_DEV Stack wave_stack(const MjpbrScene& s, float* base) {
  return shared_stack(base, kThreads, stack_entries(s.settings.stack_depth));
}

// Camera and tile coordinates of CTA tile `tile` in a tile map.
MJ_DEV void tile_of(const TileMap& tm, int32_t tile, int32_t* cam, int32_t* tx, int32_t* ty) {
  int32_t c = 0;
  while (c + 1 < tm.ncam && tile >= tm.tile_base[c + 1]) ++c;
  const int32_t t = tile - tm.tile_base[c];
  *cam = c;
  *tx = t % tm.tiles_x[c];
  *ty = t / tm.tiles_x[c];
}

MJ_DEV HitRec pack_hit(const Hit& h) {
  HitRec r;
  r.dist = h.dist;
  r.ref = h.geom == -1 ? -1 : (h.slot | ((h.mesh + 1) << 16));
  r.face = h.face;
  r.u = h.u;
  r.v = h.v;
  r.nx = h.normal.x;
  r.ny = h.normal.y;
  r.nz = h.normal.z;
  return r;
}

MJ_DEV Hit unpack_hit(const HitRec& r, const float* blk, const BlockLayout& L) {
  Hit h;
  h.dist = r.dist;
  h.slot = r.ref & 0xffff;
  h.mesh = (r.ref >> 16) - 1;
  h.geom = __float_as_int(blk[L.geom_off + h.slot * kGeomFloats + 16]);
  h.face = r.face;
  h.u = r.u;
  h.v = r.v;
  h.normal = V3{r.nx, r.ny, r.nz};
  return h;
}

MJ_DEV SurfRec pack_surface(const Surface& sf, V3 normal, float dist, int32_t slot) {
  SurfRec r;
  r.a = make_float4(sf.base_color.x, sf.base_color.y, sf.base_color.z, sf.metallic);
  r.b = make_float4(sf.roughness, sf.reflectance, sf.occlusion, dist);
  r.c = make_float4(sf.emissive.x, sf.emissive.y, sf.emissive.z, __int_as_float(slot));
  r.d = make_float4(normal.x, normal.y, normal.z, sf.alpha);
  return r;
}

MJ_DEV SurfRec missed_surface() {
  SurfRec r;
  r.a = r.b = r.d = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  r.c = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1));
  return r;
}

MJ_DEV int32_t surface_slot(const SurfRec& r) { return __float_as_int(r.c.w); }

MJ_DEV Surface unpack_surface(const SurfRec& r, V3* normal, float* dist) {
  Surface sf;
  sf.base_color = V3{r.a.x, r.a.y, r.a.z};
  sf.metallic = r.a.w;
  sf.roughness = r.b.x;
  sf.reflectance = r.b.y;
  sf.occlusion = r.b.z;
  sf.emissive = V3{r.c.x, r.c.y, r.c.z};
  sf.alpha = r.d.w;
  *normal = V3{r.d.x, r.d.y, r.d.z};
  *dist = r.b.w;
  return sf;
}

// Appends one entry per thread with `want` to a queue as one contiguous run per CTA (warps in
// order, lanes in order within a warp): one atomic per CTA, and the entries of a run stay in the
// CTA's pixel order, so a warp of the consuming kernel gets neighbouring rays of one world. Every
// thread of the CTA must make the call; `scan` is kThreads / 32 + 1 ints of shared memory.
MJ_DEV int64_t cta_append(bool want, int32_t* counter, int64_t cap, int32_t* scan, int32_t* err) {
  const unsigned full = 0xffffffffu;
  const unsigned m = __ballot_sync(full, want);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  constexpr int kWarps = kThreads / 32;
  if (lane == 0) scan[warp] = __popc(m);
  __syncthreads();
  if (threadIdx.x == 0) {
    int32_t total = 0;
    for (int k = 0; k < kWarps; ++k) {
      const int32_t c = scan[k];
      scan[k] = total;
      total += c;
    }
    scan[kWarps] = total > 0 ? atomicAdd(counter, total) : 0;
  }
  __syncthreads();
  const int64_t base = (int64_t)scan[kWarps] + scan[warp];
  __syncthreads();  // scan is reused by the next call
  if (!want) return -1;
  const int64_t pos = base + __popc(m & ((1u << lane) - 1u));
  if (pos >= cap) {
    *err |= kErrWorkQueue;
    return -1;
  }
  return pos;
}

// Camera, pixel id and sample of a chunk-local sample index.
MJ_DEV void sample_pixel(const MjpbrScene& s, const WaveMap& wm, int32_t sample, int32_t* w, int32_t* cam, int32_t* pixelid,
                         int32_t* smp) {
  const int32_t wl = sample / wm.per_world;
  const int32_t local = sample - wl * wm.per_world;
  int32_t c = 0;
  for (int32_t k = 0; k < s.nrender; ++k) {
    if (s.render_rgb[k] && wm.sample_base[k] <= local) c = k;
  }
  const int32_t rel = local - wm.sample_base[c];
  *w = wm.w0 + wl;
  *cam = c;
  *pixelid = rel / wm.nn;
  *smp = rel - *pixelid * wm.nn;
}

MJ_DEV uint32_t pixel_seed_of(const MjpbrScene& s, uint32_t seed, int32_t w, int32_t cam, int32_t pixelid) {
  return seed + (uint32_t)w * (uint32_t)s.total_rays + (uint32_t)(s.ray_adr[cam] + pixelid);
}

// Shadow entries of a shaded surface: one per model light whose visibility the shading will ask
// for (shadow_setup), every thread of the CTA calling.
MJ_DEV void emit_shadows(const MjpbrScene& s, const WaveMap& wm, const float* blk, const BlockLayout& L, bool shaded, V3 point,
                         V3 normal, int32_t sample, int32_t seg, int32_t* scan, int32_t* err) {
  const V3 origin = point + normal * kRayOffset;
  for (int32_t li = 0; li < L.nlight; ++li) {
    V3 l = v3(0.0f);
    float dist = 0.0f;
    bool want = false;
    if (shaded) {
      const Light light = load_light(blk + L.light_off + li * kLightFloats);
      want = light.active && shadow_setup(s.settings, light, point, normal, &l, &dist);
    }
    const int64_t pos = cta_append(want, wm.counters + 1, wm.shadow_cap, scan, err);
    if (pos >= 0) {
      ShadowEntry e;
      e.o = make_float4(origin.x, origin.y, origin.z, dist);
      e.l = make_float4(l.x, l.y, l.z, __int_as_float((sample * 2 + seg) * wm.nl + li));
      wm.shadow[pos] = e;
      wm.vis[(sample * 2 + seg) * wm.nl + li] = 0;  // the shadow stage adds its unoccluded rays
    }
  }
}

// ---------------------------------------------------------------- 1. primary rays
template <bool kMesh, bool kStaged>
__global__ void __launch_bounds__(kThreads, MJPBR_WAVE_TRACE_CTAS) wave_primary_kernel(const __grid_constant__ MjpbrScene s,
                                                                const __grid_constant__ WaveMap wm) {
  extern __shared__ __align__(16) float smem[];
  const int32_t w = wm.w0 + blockIdx.y;
  const float* blk = world_block_of<kStaged>(s, w, smem, kThreads);
  __syncthreads();
  const BlockLayout L = block_layout(s.nbvh_geom, s.nnode, s.nlight, s.nrender);
  const Stack st = wave_stack(s, smem + (kStaged ? s.world_block_floats : 0));
  int32_t cam, tx, ty;
  tile_of(wm.geo, blockIdx.x, &cam, &tx, &ty);
  Pixel p;
  p.cam = cam;
  p.width = s.cam_res[cam][0];
  p.height = s.cam_res[cam][1];
  p.rec = blk + L.cam_off + cam * kCamFloats;
  const bool rgb = s.render_rgb[cam] != 0;
  const int32_t n = rgb ? s.settings.samples_per_axis : 1;
  const int32_t nn = n * n;
  const M3 R = cam_mat(p.rec);
  const V3 cpos{p.rec[0], p.rec[1], p.rec[2]};
  const bool cull = s.settings.cull_backfaces != 0;
  HitRec* out = wm.hit[0] + (int64_t)blockIdx.y * wm.per_world + (rgb ? wm.sample_base[cam] : 0);
  int32_t err = 0;
#pragma unroll 1
  for (int32_t idx = threadIdx.x; idx < kTile * kTile * nn; idx += kThreads) {
    const int32_t q = idx / nn, smp = idx - q * nn;
    p.px = tx * kTile + z_x(q);
    p.py = ty * kTile + z_y(q);
    if (p.px >= p.width || p.py >= p.height) continue;
    p.pixelid = p.py * p.width + p.px;
    V3 dcam, ocam;
    float max_dist, depth_z;
    primary_ray(s, p, n, smp % n, smp / n, &dcam, &ocam, &max_dist, &depth_z);
    const Ray ray{cpos + mul(R, ocam), mul(R, dcam)};
    const Hit hit = trace_ray<kMesh>(s, st, blk, L, ray, max_dist, cull, false, &err);
    if (smp == 0) write_geometry(s, w, p, hit, depth_z);
    if (rgb) out[(int64_t)p.pixelid * nn + smp] = pack_hit(hit);
  }
  if (err && s.error_word) atomicOr(s.error_word, err);
}

// ---------------------------------------------------------------- 2. surfaces at primary hits
template <bool kMesh, bool kTex, bool kStaged>
__global__ void __launch_bounds__(kThreads, MJPBR_WAVE_SHADE_CTAS) wave_surface_kernel(const __grid_constant__ MjpbrScene s,
                                                                const __grid_constant__ WaveMap wm) {
  extern __shared__ __align__(16) float smem[];
  __shared__ int32_t scan[kThreads / 32 + 1];
  const int32_t w = wm.w0 + blockIdx.y;
  const float* blk = world_block_of<kStaged>(s, w, smem, kThreads);
  __syncthreads();
  const BlockLayout L = block_layout(s.nbvh_geom, s.nnode, s.nlight, s.nrender);
  int32_t cam, tx, ty;
  tile_of(wm.rgb, blockIdx.x, &cam, &tx, &ty);
  Pixel p;
  p.cam = cam;
  p.width = s.cam_res[cam][0];
  p.height = s.cam_res[cam][1];
  p.rec = blk + L.cam_off + cam * kCamFloats;
  const int32_t n = s.settings.samples_per_axis, nn = wm.nn;
  const float inv_n = 1.0f / (float)n;
  const M3 R = cam_mat(p.rec);
  const V3 cpos{p.rec[0], p.rec[1], p.rec[2]};
  RtCtx c;
  init_ctx(c, s, blk, L, w, kTex);
  const int32_t first = blockIdx.y * wm.per_world + wm.sample_base[cam];
  int32_t err = 0;
#pragma unroll 1
  for (int32_t idx = threadIdx.x; idx < kTile * kTile * nn; idx += kThreads) {
    const int32_t q = idx / nn, smp = idx - q * nn;
    p.px = tx * kTile + z_x(q);
    p.py = ty * kTile + z_y(q);
    const bool valid = p.px < p.width && p.py < p.height;
    p.pixelid = p.py * p.width + p.px;
    const int32_t sample = first + p.pixelid * nn + smp;
    bool shaded = false, reflect = false;
    V3 point = v3(0.0f), normal = v3(0.0f), so = v3(0.0f), sd = v3(0.0f);
    float cone = 0.0f, spread = 0.0f;
    if (valid) {
      const HitRec hr = wm.hit[0][sample];
      if (hr.ref == -1) {
        wm.surf[0][sample] = missed_surface();
      } else {
        V3 dcam, ocam;
        float max_dist, depth_z, pixel_spread, pixel_width;
        primary_ray(s, p, n, smp % n, smp / n, &dcam, &ocam, &max_dist, &depth_z);
        const V3 origin = cpos + mul(R, ocam), dir = mul(R, dcam);
        pixel_cone(s, p, &pixel_spread, &pixel_width);
        spread = pixel_spread * inv_n;
        const float width = pixel_width * inv_n;
        const Hit hit = unpack_hit(hr, blk, L);
        point = origin + dir * hit.dist;
        cone = width + spread * (0.0f + hit.dist);
        const Surface sf = eval_surface<kMesh, kTex>(s, blk, L, w, hit, hit.slot, point, dir, cone, &normal);
        wm.surf[0][sample] = pack_surface(sf, normal, hit.dist, hit.slot);
        shaded = true;
        const float mirror = s.settings.has_reflection ? mirror_reflectance(c, hit.slot) : 0.0f;
        if (mirror > 0.0f) {
          mirror_ray(point, normal, dir, &so, &sd);
          reflect = true;
        }
      }
    }
    emit_shadows(s, wm, blk, L, shaded, point, normal, sample, 0, scan, &err);
    const int64_t pos = cta_append(reflect, wm.counters, wm.mirror_cap, scan, &err);
    if (pos >= 0) {
      MirrorEntry e;
      e.o = make_float4(so.x, so.y, so.z, cone);
      e.d = make_float4(sd.x, sd.y, sd.z, spread);
      e.index = make_int4(sample, 0, 0, 0);
      wm.mirror[pos] = e;
    }
  }
  if (err && s.error_word) atomicOr(s.error_word, err);
}

// ---------------------------------------------------------------- 3. mirror rays (persistent)
// Steps a lane runs between refills of the warp's idle lanes (mirror and shadow stages).
#ifndef MJPBR_WAVE_REFILL_STEPS
#define MJPBR_WAVE_REFILL_STEPS 32
#endif

// Closest hit of every queued mirror ray, lanes refilled from the queue (refill.cuh).
template <bool kMesh>
__global__ void __launch_bounds__(kThreads, MJPBR_WAVE_MIRROR_CTAS) wave_mirror_kernel(const __grid_constant__ MjpbrScene s,
                                                               const __grid_constant__ WaveMap wm) {
  extern __shared__ __align__(16) float smem[];
  const BlockLayout L = block_layout(s.nbvh_geom, s.nnode, s.nlight, s.nrender);
  const Stack st = wave_stack(s, smem);
  const bool cull = s.settings.cull_backfaces != 0;
  const int64_t items = min((int64_t)wm.counters[0], wm.mirror_cap);
  int32_t err = 0;
  ClosestQuery q;
  const float* blk = nullptr;
  int32_t sample = -1;
  refill_loop<MJPBR_WAVE_REFILL_STEPS>(
      items, reinterpret_cast<unsigned long long*>(wm.counters + 4), q,
      [&](int64_t item, ClosestQuery& qq) {
        const MirrorEntry e = wm.mirror[item];
        sample = e.index.x;
        blk = s.world_blocks + (int64_t)(wm.w0 + sample / wm.per_world) * s.world_block_floats;
        closest_begin(qq, st, Ray{V3{e.o.x, e.o.y, e.o.z}, V3{e.d.x, e.d.y, e.d.z}}, kMaxVal, &err);
        return true;
      },
      [&](ClosestQuery& qq) { return closest_step<kMesh>(qq, s, st, blk, L, cull, &err); },
      [&](ClosestQuery& qq, int32_t) { wm.hit[1][sample] = pack_hit(qq.h); }, &err);
  if (err && s.error_word) atomicOr(s.error_word, err);
}

// ---------------------------------------------------------------- 4. surfaces at mirror hits
template <bool kMesh, bool kTex>
__global__ void __launch_bounds__(kThreads, MJPBR_WAVE_SHADE_CTAS) wave_mirror_surface_kernel(const __grid_constant__ MjpbrScene s,
                                                                       const __grid_constant__ WaveMap wm) {
  __shared__ int32_t scan[kThreads / 32 + 1];
  const BlockLayout L = block_layout(s.nbvh_geom, s.nnode, s.nlight, s.nrender);
  const int32_t count = (int32_t)min((int64_t)*wm.counters, wm.mirror_cap);
  int32_t err = 0;
  // uniform trip count per CTA (the shadow entries are appended by whole CTAs)
  const int32_t stride = gridDim.x * kThreads;
  const int32_t rounds = (count + stride - 1) / stride;
  for (int32_t r = 0; r < rounds; ++r) {
    const int32_t i = r * stride + blockIdx.x * kThreads + threadIdx.x;
    bool shaded = false;
    V3 point = v3(0.0f), normal = v3(0.0f);
    int32_t sample = 0;
    const float* blk = s.world_blocks;
    if (i < count) {
      const MirrorEntry e = wm.mirror[i];
      sample = e.index.x;
      const int32_t w = wm.w0 + sample / wm.per_world;
      blk = s.world_blocks + (int64_t)w * s.world_block_floats;
      const HitRec hr = wm.hit[1][sample];
      if (hr.ref == -1) {
        wm.surf[1][sample] = missed_surface();
      } else {
        const Hit hit = unpack_hit(hr, blk, L);
        const V3 so{e.o.x, e.o.y, e.o.z}, sd{e.d.x, e.d.y, e.d.z};
        point = so + sd * hit.dist;
        const float cone = e.o.w + e.d.w * hit.dist;
        const Surface sf = eval_surface<kMesh, kTex>(s, blk, L, w, hit, hit.slot, point, sd, cone, &normal);
        wm.surf[1][sample] = pack_surface(sf, normal, hit.dist, hit.slot);
        shaded = true;
      }
    }
    emit_shadows(s, wm, blk, L, shaded, point, normal, sample, 1, scan, &err);
  }
  if (err && s.error_word) atomicOr(s.error_word, err);
}

// ---------------------------------------------------------------- 5. shadow rays (persistent)
// Work items: (entry, ray k < shadow_samples), traced as any-hit queries with lanes refilled from
// the queue (refill.cuh); each unoccluded ray adds one to its entry's count (an integer sum, so
// the counts do not depend on the order).
template <bool kMesh>
__global__ void __launch_bounds__(kThreads, MJPBR_WAVE_TRACE_CTAS) wave_shadow_kernel(const __grid_constant__ MjpbrScene s, uint32_t seed,
                                                               const __grid_constant__ WaveMap wm) {
  extern __shared__ __align__(16) float smem[];
  const BlockLayout L = block_layout(s.nbvh_geom, s.nnode, s.nlight, s.nrender);
  const Stack st = wave_stack(s, smem);
  const bool cull = s.settings.cull_backfaces != 0;
  const int32_t ns = max(s.settings.shadow_samples, 1);
  const int64_t items = min((int64_t)wm.counters[1], wm.shadow_cap) * ns;
  int32_t err = 0;
  AnyQuery q;
  const float* blk = nullptr;
  int32_t target = -1;
  refill_loop<MJPBR_WAVE_REFILL_STEPS>(
      items, reinterpret_cast<unsigned long long*>(wm.counters + 2), q,
      [&](int64_t item, AnyQuery& qq) {
        const int32_t ei = (int32_t)(item / ns), k = (int32_t)(item - (int64_t)ei * ns);
        const ShadowEntry e = wm.shadow[ei];
        const int32_t tgt = __float_as_int(e.l.w);
        const int32_t li = tgt % wm.nl;
        const int32_t sample = tgt / (2 * wm.nl);
        const int32_t seg = (tgt / wm.nl) & 1;
        int32_t w, cam, pixelid, smp;
        sample_pixel(s, wm, sample, &w, &cam, &pixelid, &smp);
        blk = s.world_blocks + (int64_t)w * s.world_block_floats;
        const Light light = load_light(blk + L.light_off + li * kLightFloats);
        if (k >= shadow_ray_count(light, ns)) return false;
        Ray r;
        float max_dist;
        r.o = V3{e.o.x, e.o.y, e.o.z};
        shadow_ray(light, ns, r.o, V3{e.l.x, e.l.y, e.l.z}, e.o.w, pixel_seed_of(s, seed, w, cam, pixelid), 2 * smp + seg, L.nlight, li, k,
                   &r.d, &max_dist);
        any_begin(qq, st, r, max_dist, &err);
        target = tgt;
        return true;
      },
      [&](AnyQuery& qq) { return any_step<kMesh>(qq, s, st, blk, L, cull, &err); },
      [&](AnyQuery&, int32_t res) {
        if (res == kAnyClear) atomicAdd(&wm.vis[target], 1);
      },
      &err);
  if (err && s.error_word) atomicOr(s.error_word, err);
}

// Shadow visibility of the resolve stage: the counts of stage 5.
struct StoredVis {
  const int32_t* counts;  // the segment's counts, indexed by model light
  MJ_DEV float visibility(RtCtx& c, const Light& light, V3, V3, V3, float, uint32_t, int32_t, int32_t, int32_t li) {
    const MjpbrSettings& st = c.s->settings;
    return visible_fraction(light, st.shadow_samples, counts[li], st.shadow_light_fraction);
  }
};

// ---------------------------------------------------------------- 6. shading and pixel outputs
template <bool kTex, bool kStaged>
__global__ void __launch_bounds__(kThreads, MJPBR_WAVE_SHADE_CTAS) wave_resolve_kernel(const __grid_constant__ MjpbrScene s, uint32_t seed,
                                                                const __grid_constant__ WaveMap wm) {
  using Shade = RtShade<kTex, StoredVis>;
  extern __shared__ __align__(16) float smem[];
  const int32_t w = wm.w0 + blockIdx.y;
  const float* blk = world_block_of<kStaged>(s, w, smem, kThreads);
  __syncthreads();
  const BlockLayout L = block_layout(s.nbvh_geom, s.nnode, s.nlight, s.nrender);
  // a CTA shades `ppc` pixels of a tile with one thread per camera sample (nn consecutive threads
  // per pixel); the pixel's first thread sums the samples in sample order through shared memory
  __shared__ float sums[kThreads * 6];
  const int32_t nn = wm.nn;
  const int32_t ppc = kThreads / nn, parts = (kTile * kTile + ppc - 1) / ppc;
  int32_t cam, tx, ty;
  tile_of(wm.rgb, blockIdx.x / parts, &cam, &tx, &ty);
  const int32_t lp = threadIdx.x / nn, smp = threadIdx.x - lp * nn;
  const int32_t q = (blockIdx.x % parts) * ppc + lp;
  Pixel p;
  p.cam = cam;
  p.width = s.cam_res[cam][0];
  p.height = s.cam_res[cam][1];
  p.rec = blk + L.cam_off + cam * kCamFloats;
  p.px = tx * kTile + z_x(q);
  p.py = ty * kTile + z_y(q);
  const bool active = lp < ppc && q < kTile * kTile && p.px < p.width && p.py < p.height;
  p.pixelid = p.py * p.width + p.px;
  const MjpbrSettings& st = s.settings;
  RtCtx c;
  init_ctx(c, s, blk, L, w, kTex);
  const M3 R = cam_mat(p.rec);
  const V3 cpos{p.rec[0], p.rec[1], p.rec[2]};
  const int32_t n = st.samples_per_axis;
  const float inv_n = 1.0f / (float)n;
  const V3 head_dir = -V3{R.m[2], R.m[5], R.m[8]};
  const uint32_t pseed = pixel_seed_of(s, seed, w, cam, p.pixelid);
  const int32_t first = blockIdx.y * wm.per_world + wm.sample_base[cam] + p.pixelid * nn;
  if (active) {
    float pixel_spread, pixel_width;
    pixel_cone(s, p, &pixel_spread, &pixel_width);  // reads the camera's rays: active pixels only
    const float spread = pixel_spread * inv_n;
    V3 dcam, ocam;
    float max_dist, depth_z;
    primary_ray(s, p, n, smp % n, smp / n, &dcam, &ocam, &max_dist, &depth_z);
    const V3 origin = cpos + mul(R, ocam), dir = mul(R, dcam);
    const int32_t sample = first + smp;
    const SurfRec r0 = wm.surf[0][sample];
    V3 radiance = v3(0.0f);
    V3 albedo = v3(0.0f), gnormal = v3(0.0f);
    const int32_t slot = surface_slot(r0);
    if (slot < 0) {
      radiance += Shade::background(c, dir, spread) * 1.0f;
    } else {
      V3 normal;
      float dist;
      const Surface sf = unpack_surface(r0, &normal, &dist);
      albedo = sf.base_color;
      gnormal = normal;
      const V3 point = origin + dir * dist;
      StoredVis vis{wm.vis + ((int64_t)sample * 2) * wm.nl};
      const V3 shaded = Shade::shade_surface(c, vis, sf, point, normal, -dir, head_dir, pseed, 2 * smp);
      const float mirror = st.has_reflection ? mirror_reflectance(c, slot) : 0.0f;
      const float wt = 1.0f * 1.0f;
      radiance += shaded * ((1.0f - mirror) * wt);
      if (mirror > 0.0f) {
        const float sweight = mirror * wt;
        V3 so, sd;
        mirror_ray(point, normal, dir, &so, &sd);
        const SurfRec r1 = wm.surf[1][sample];
        if (surface_slot(r1) < 0) {
          radiance += Shade::background(c, sd, spread) * sweight;
        } else {
          V3 n1;
          float d1;
          const Surface sf1 = unpack_surface(r1, &n1, &d1);
          const V3 p1 = so + sd * d1;
          StoredVis vis1{wm.vis + ((int64_t)sample * 2 + 1) * wm.nl};
          radiance += Shade::shade_surface(c, vis1, sf1, p1, n1, -sd, head_dir, pseed, 2 * smp + 1) * sweight;
        }
      }
    }
    if (smp == 0 && st.render_guides && s.guide_albedo) {
      const int64_t a = ((int64_t)w * s.rgb_stride + s.rgb_adr[cam] + p.pixelid) * 3;
      s.guide_albedo[a] = albedo.x;
      s.guide_albedo[a + 1] = albedo.y;
      s.guide_albedo[a + 2] = albedo.z;
      s.guide_normal[a] = gnormal.x;
      s.guide_normal[a + 1] = gnormal.y;
      s.guide_normal[a + 2] = gnormal.z;
    }
    const V3 display = display_transform(radiance * c.exposure, st.tone_mapper);
    float* slot_sum = sums + threadIdx.x * 6;
    slot_sum[0] = display.x, slot_sum[1] = display.y, slot_sum[2] = display.z;
    slot_sum[3] = radiance.x, slot_sum[4] = radiance.y, slot_sum[5] = radiance.z;
  }
  __syncthreads();
  if (!active || smp != 0) return;
  V3 display = v3(0.0f), hdr = v3(0.0f);
  for (int32_t k = 0; k < nn; ++k) {  // the samples in sample order, as one thread's loop would add them
    const float* v = sums + (threadIdx.x + k) * 6;
    display += V3{v[0], v[1], v[2]};
    hdr += V3{v[3], v[4], v[5]};
  }
  const int64_t adr = (int64_t)w * s.rgb_stride + s.rgb_adr[cam] + p.pixelid;
  const float inv_nn = inv_n * inv_n;
  if (st.render_hdr && s.hdr_data) {
    s.hdr_data[adr * 3] = hdr.x * inv_nn;
    s.hdr_data[adr * 3 + 1] = hdr.y * inv_nn;
    s.hdr_data[adr * 3 + 2] = hdr.z * inv_nn;
  }
  s.rgb_data[adr] = encode_display(display * inv_nn);
}

// ---------------------------------------------------------------- host side

// Stage profile of mjpbr_wave_profile_begin / _end (this host thread): per chunk, one event
// before the primary stage and one after each of the six stages (a stage that does not run still
// records), from a pool of events the library creates once and reuses.
constexpr int kStages = 6;

struct StageProfile {
  bool on = false;
  std::vector<cudaEvent_t> events;
  size_t used = 0;
  ~StageProfile() {
    for (cudaEvent_t e : events) cudaEventDestroy(e);
  }
};
thread_local StageProfile g_profile;

void stage_mark(cudaStream_t stream) {
  StageProfile& p = g_profile;
  if (!p.on) return;
  if (p.used == p.events.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) {
      p.on = false;
      return;
    }
    p.events.push_back(e);
  }
  cudaEventRecord(p.events[p.used++], stream);
}

int64_t align256(int64_t b) { return (b + 255) & ~int64_t(255); }

int32_t samples_per_world(const MjpbrScene& s) {
  const int64_t nn = (int64_t)s.settings.samples_per_axis * s.settings.samples_per_axis;
  int64_t total = 0;
  for (int32_t c = 0; c < s.nrender; ++c) {
    if (s.render_rgb[c]) total += (int64_t)s.cam_res[c][0] * s.cam_res[c][1] * nn;
  }
  return total > INT32_MAX ? -1 : (int32_t)total;
}

// Scratch layout for `worlds` worlds per chunk (pointers relative to base).
int64_t layout(WaveMap* wm, char* base, int32_t worlds, int32_t per_world, int32_t nlight) {
  const int64_t n = (int64_t)worlds * per_world;
  const int64_t nl = std::max(nlight, 0);
  int64_t off = 0;
  auto take = [&](int64_t bytes) {
    char* p = base + off;
    off += align256(bytes);
    return p;
  };
  if (wm) {
    wm->counters = reinterpret_cast<int32_t*>(take(256));
    for (int k = 0; k < 2; ++k) wm->hit[k] = reinterpret_cast<HitRec*>(take(n * kHitBytes));
    for (int k = 0; k < 2; ++k) wm->surf[k] = reinterpret_cast<SurfRec*>(take(n * kSurfBytes));
    wm->mirror = reinterpret_cast<MirrorEntry*>(take(n * kMirrorBytes));
    wm->vis = reinterpret_cast<int32_t*>(take(n * 2 * nl * 4));
    wm->shadow = reinterpret_cast<ShadowEntry*>(take(n * 2 * nl * kShadowBytes));
    wm->mirror_cap = n;
    wm->shadow_cap = n * 2 * nl;
    return off;
  }
  off = align256(256) + 2 * align256(n * kHitBytes) + 2 * align256(n * kSurfBytes) + align256(n * kMirrorBytes) +
        align256(n * 2 * nl * 4) + align256(n * 2 * nl * kShadowBytes);
  return off;
}

TileMap tile_map(const MjpbrScene& s, bool rgb_only) {
  TileMap tm;
  tm.w0 = 0;  // the stages take their chunk's first world from the WaveMap
  tm.ncam = s.nrender;
  tm.tile_w = kTile;
  tm.tile_h = kTile;
  tm.tile_base[0] = 0;
  for (int32_t c = 0; c < s.nrender; ++c) {
    const int32_t W = s.cam_res[c][0], H = s.cam_res[c][1];
    const bool any = rgb_only ? s.render_rgb[c] != 0 : (s.render_rgb[c] || s.render_depth[c] || s.render_seg[c]);
    tm.tiles_x[c] = (W + kTile - 1) / kTile;
    tm.tile_base[c + 1] = tm.tile_base[c] + (any ? tm.tiles_x[c] * ((H + kTile - 1) / kTile) : 0);
  }
  return tm;
}

// Resident CTAs per SM of a persistent kernel (the occupancy calculator's answer, at least 1).
template <class K>
int resident_ctas(K kern, size_t smem) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kern, kThreads, smem) != cudaSuccess || n < 1) n = 1;
  return n;
}

template <class K>
int set_smem(K kern, size_t smem, const char* what) {
  return ensure_smem(reinterpret_cast<const void*>(kern), smem, what);
}

template <bool kMesh, bool kTex, bool kStaged>
int launch_wave(const MjpbrScene& s, uint32_t seed, cudaStream_t stream, int32_t chunk, int32_t per_world) {
  const size_t stack = (size_t)kThreads * stack_entries(s.settings.stack_depth) * 8;
  // world blocks staged in shared memory, or read in place when they do not fit
  const size_t blk_bytes = kStaged ? (size_t)s.world_block_floats * sizeof(float) : 0;
  auto k_primary = wave_primary_kernel<kMesh, kStaged>;
  auto k_surface = wave_surface_kernel<kMesh, kTex, kStaged>;
  auto k_mirror = wave_mirror_kernel<kMesh>;
  auto k_msurface = wave_mirror_surface_kernel<kMesh, kTex>;
  auto k_shadow = wave_shadow_kernel<kMesh>;
  auto k_resolve = wave_resolve_kernel<kTex, kStaged>;
  int rc = set_smem(k_primary, blk_bytes + stack, "wavefront primary");
  if (!rc) rc = set_smem(k_surface, blk_bytes, "wavefront surface");
  if (!rc) rc = set_smem(k_mirror, stack, "wavefront mirror");
  if (!rc) rc = set_smem(k_shadow, stack, "wavefront shadow");
  if (!rc) rc = set_smem(k_resolve, blk_bytes, "wavefront resolve");
  if (rc) return rc;
  const int sms = device_sm_count();
  const int g_mirror = sms * resident_ctas(k_mirror, stack);
  const int g_msurface = sms * resident_ctas(k_msurface, 0);
  const int g_shadow = sms * resident_ctas(k_shadow, stack);
  WaveMap wm;
  wm.nn = s.settings.samples_per_axis * s.settings.samples_per_axis;
  wm.per_world = per_world;
  wm.nl = s.nlight;
  int32_t base = 0;
  for (int32_t c = 0; c < MJPBR_MAX_RENDER; ++c) {
    wm.sample_base[c] = base;
    if (c < s.nrender && s.render_rgb[c]) base += s.cam_res[c][0] * s.cam_res[c][1] * wm.nn;
  }
  wm.geo = tile_map(s, false);
  wm.rgb = tile_map(s, true);
  layout(&wm, static_cast<char*>(s.wave_scratch), chunk, per_world, s.nlight);
  const int32_t geo_tiles = wm.geo.tile_base[s.nrender], rgb_tiles = wm.rgb.tile_base[s.nrender];
  for (int32_t w0 = 0; w0 < s.nworld; w0 += chunk) {
    wm.w0 = w0;
    wm.nw = std::min(chunk, s.nworld - w0);
    stage_mark(stream);
    if (geo_tiles > 0) {
      k_primary<<<dim3(geo_tiles, wm.nw), kThreads, blk_bytes + stack, stream>>>(s, wm);
      if ((rc = check_launch("wave_primary_kernel"))) return rc;
    }
    stage_mark(stream);
    if (rgb_tiles > 0) {
      cudaError_t e = cudaMemsetAsync(wm.counters, 0, 6 * sizeof(int32_t), stream);  // queue lengths, fetch counters
      if (e != cudaSuccess) return set_error(MJPBR_ERR_CUDA, "wavefront queue counters: %s", cudaGetErrorString(e));
      k_surface<<<dim3(rgb_tiles, wm.nw), kThreads, blk_bytes, stream>>>(s, wm);
      if ((rc = check_launch("wave_surface_kernel"))) return rc;
    }
    stage_mark(stream);
    const bool mirrors = rgb_tiles > 0 && s.settings.has_reflection;
    if (mirrors) {
      k_mirror<<<g_mirror, kThreads, stack, stream>>>(s, wm);
      if ((rc = check_launch("wave_mirror_kernel"))) return rc;
    }
    stage_mark(stream);
    if (mirrors) {
      k_msurface<<<g_msurface, kThreads, 0, stream>>>(s, wm);
      if ((rc = check_launch("wave_mirror_surface_kernel"))) return rc;
    }
    stage_mark(stream);
    if (rgb_tiles > 0 && s.nlight > 0 && s.settings.use_shadows) {
      k_shadow<<<g_shadow, kThreads, stack, stream>>>(s, seed, wm);
      if ((rc = check_launch("wave_shadow_kernel"))) return rc;
    }
    stage_mark(stream);
    if (rgb_tiles > 0) {
      const int32_t ppc = kThreads / wm.nn, parts = (kTile * kTile + ppc - 1) / ppc;
      k_resolve<<<dim3(rgb_tiles * parts, wm.nw), kThreads, blk_bytes, stream>>>(s, seed, wm);
      if ((rc = check_launch("wave_resolve_kernel"))) return rc;
    }
    stage_mark(stream);
  }
  return MJPBR_OK;
}

}  // namespace

int64_t wave_scratch_bytes(const MjpbrScene& s, int32_t worlds) {
  if (s.settings.tier == MJPBR_TIER_PATH) return pt_wave_scratch_bytes(s, worlds);
  const int32_t per_world = samples_per_world(s);
  if (per_world < 0 || worlds < 0) return -1;
  return layout(nullptr, nullptr, worlds, per_world, s.nlight);
}

// The wavefront's records pack geom slots and triangle BVH ids in 16 bits, and its stages do not
// render translucent layers; other scenes render with the grid schedule (the same images).
bool wave_supported(const MjpbrScene& s) {
  return !s.settings.has_transparency && s.nbvh_geom <= 0xffff && s.nmesh + s.nhfield < 0x7fff;
}

int render_wave_launch(const MjpbrScene& s, uint32_t seed, cudaStream_t stream) {
  if (!wave_supported(s)) {
    return set_error(MJPBR_ERR_UNSUPPORTED, "the wavefront schedule renders neither translucent layers nor more than 65535 geoms "
                                            "or 32766 triangle BVHs; use the grid schedule");
  }
  const int32_t per_world = samples_per_world(s);
  if (per_world < 0) return set_error(MJPBR_ERR_ARG, "wavefront: too many samples per world");
  if (!s.wave_scratch || (reinterpret_cast<uintptr_t>(s.wave_scratch) & 255u)) {
    return set_error(MJPBR_ERR_ARG, "the wavefront schedule needs wave_scratch (256-byte aligned)");
  }
  // worlds per chunk: as many as the scratch holds, sample / target indices within int32, and at
  // most kMaxGridWorlds (the stages put a chunk's worlds in grid y)
  int32_t chunk = std::min(s.nworld, kMaxGridWorlds);
  if (per_world > 0) {
    const int64_t nl2 = 2 * (int64_t)std::max(s.nlight, 1);
    chunk = (int32_t)std::min<int64_t>(chunk, (INT32_MAX / nl2) / per_world);
    if (wave_scratch_bytes(s, chunk) > s.wave_scratch_bytes) {
      int32_t lo = 0, hi = chunk;  // the largest chunk whose layout fits the scratch
      while (lo < hi) {
        const int32_t mid = lo + (hi - lo + 1) / 2;
        if (wave_scratch_bytes(s, mid) <= s.wave_scratch_bytes) {
          lo = mid;
        } else {
          hi = mid - 1;
        }
      }
      chunk = lo;
    }
    if (chunk < 1) {
      return set_error(MJPBR_ERR_ARG, "wave_scratch of %lld bytes holds no world (one needs %lld)", (long long)s.wave_scratch_bytes,
                       (long long)wave_scratch_bytes(s, 1));
    }
  }
  const bool mesh = s.nmesh + s.nhfield > 0 && s.blas_root != nullptr;
  const bool tex = s.settings.textures || s.settings.has_env || s.settings.env_background;
  const size_t stack = (size_t)kThreads * stack_entries(s.settings.stack_depth) * 8;
  if (world_block_staged(s.world_block_floats, stack)) {
    if (mesh && tex) return launch_wave<true, true, true>(s, seed, stream, chunk, per_world);
    if (mesh) return launch_wave<true, false, true>(s, seed, stream, chunk, per_world);
    if (tex) return launch_wave<false, true, true>(s, seed, stream, chunk, per_world);
    return launch_wave<false, false, true>(s, seed, stream, chunk, per_world);
  }
  if (mesh && tex) return launch_wave<true, true, false>(s, seed, stream, chunk, per_world);
  if (mesh) return launch_wave<true, false, false>(s, seed, stream, chunk, per_world);
  if (tex) return launch_wave<false, true, false>(s, seed, stream, chunk, per_world);
  return launch_wave<false, false, false>(s, seed, stream, chunk, per_world);
}

}  // namespace mjpbr

extern "C" int mjpbr_wave_profile_begin(void) {
  mjpbr::g_profile.on = true;
  mjpbr::g_profile.used = 0;
  return MJPBR_OK;
}

extern "C" int mjpbr_wave_profile_end(double* stage_ms, int32_t* chunks) {
  using namespace mjpbr;
  StageProfile& p = g_profile;
  const bool was_on = p.on;
  p.on = false;
  const size_t per = kStages + 1;
  const size_t used = p.used;
  p.used = 0;
  if (!stage_ms || !chunks) return set_error(MJPBR_ERR_ARG, "stage_ms and chunks must not be NULL");
  for (int k = 0; k < kStages; ++k) stage_ms[k] = 0.0;
  *chunks = 0;
  if (!was_on) return set_error(MJPBR_ERR_ARG, "no stage profile was started on this thread");
  if (used == 0) return MJPBR_OK;
  if (used % per) return set_error(MJPBR_ERR_CUDA, "stage profile: %zu events for %zu per chunk (an event could not be created)", used, per);
  cudaError_t e = cudaEventSynchronize(p.events[used - 1]);
  if (e != cudaSuccess) return set_error(MJPBR_ERR_CUDA, "stage profile: %s", cudaGetErrorString(e));
  for (size_t c = 0; c < used / per; ++c) {
    for (int k = 0; k < kStages; ++k) {
      float ms = 0.0f;
      e = cudaEventElapsedTime(&ms, p.events[c * per + k], p.events[c * per + k + 1]);
      if (e != cudaSuccess) return set_error(MJPBR_ERR_CUDA, "stage profile: %s", cudaGetErrorString(e));
      stage_ms[k] += ms;
    }
  }
  *chunks = (int32_t)(used / per);
  return MJPBR_OK;
}

extern "C" int64_t mjpbr_wave_scratch_bytes(const MjpbrScene* scene, int32_t worlds) {
  if (!scene) return -1;
  return mjpbr::wave_scratch_bytes(*scene, worlds);
}

#ifdef MJPBR_COUNT_OPS
namespace mjpbr {
// Counting build: this unit's copy of the counter array pointer (see opcount.cuh).
int wave_count_set(void* counts) { return cudaMemcpyToSymbol(g_op_counts, &counts, sizeof(counts)) == cudaSuccess ? 0 : 1; }
}  // namespace mjpbr
#endif
