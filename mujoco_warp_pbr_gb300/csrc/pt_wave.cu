// Path-traced tier as a staged wavefront (the schedule MJPBR_SCHEDULE_WAVEFRONT of the path tier):
// the bounce loop of mujoco_warp_pbr/_src/pathtrace.py:200-421 over every path of a chunk of
// worlds at once, one kernel per stage and compacted path queues between the bounces:
//
//   geometry depth / segmentation of cameras without RGB (one ray per pixel)
//   per bounce, over the queue of live paths:
//     extend   closest hit of every path (persistent, lanes refilled from the queue: refill.cuh);
//              depth / segmentation from sample 0's first hit; the first bounce's extend starts
//              the paths itself, one per (pixel, sample) of the RGB cameras (pt_bounce.cuh
//              start_sample), and writes each path record once, after its hit
//     shade    the bounce after the hit (PtCore::surface): emission, mirror lobe, next-event
//              estimation recorded per path (each light's unshadowed contribution, the environment
//              sample's term) with each shadow ray appended to the shadow queue as it is recorded
//              (one atomic per group of converged lanes), the BSDF sample and Russian roulette;
//              the paths that continue are appended to the next queue (one atomic per CTA)
//     shadow   any hit of every queued shadow ray (persistent, lanes refilled)
//   (the recorded terms of the unoccluded rays are added to the path's radiance, in light order,
//   by the next bounce's extend stage, or by the resolve stage for a path that ended: the
//   persistent kernel's exact additions in its order)
//   resolve  one thread per pixel: its samples summed in sample order, tone map / denoiser inputs
//
// Each stage runs one kind of work on a full set of lanes and has its own register budget; the
// image is the persistent kernel's, bit for bit (the random numbers are counter-based per sample
// and bounce, so the order in which paths run does not matter).
//
// Scratch (MjpbrScene.wave_scratch), per path of a chunk: the path record (80 B every bounce moves,
// 48 B of first-surface features), its hit (32 B), its next-event record (16 B + 16 B per slot: each
// light, the headlight, the environment), one visibility byte per slot, two queue entries and up to
// one shadow entry (32 B) per slot.
#include <algorithm>
#include <climits>

#include "abi_internal.h"
#include <cooperative_groups.h>

#include "pt_bounce.cuh"
#include "refill.cuh"

namespace mjpbr {
namespace {

namespace cg = cooperative_groups;

constexpr int kThreads = 256;
// Resident CTAs per SM the shade stage's register allocation targets.
#ifndef MJPBR_PTW_SHADE_CTAS
#define MJPBR_PTW_SHADE_CTAS 3
#endif

// A path between stages: 80 bytes every bounce reads and writes, then the first surface's denoiser
// features (48 bytes), read and written only by the bounce that can set them (a camera ray's).
struct __align__(16) PathRec {
  float4 o;     // origin, max_dist
  float4 d;     // direction, pdf_prev
  float4 beta;  // throughput, dcam_z
  float4 rad;   // radiance, first-hit depth (sample 0)
  int4 meta;    // depth, passes, sample, flags (1 camera ray, 2 delta)
  float4 f0;    // first surface: albedo xyz, normal x
  float4 f1;    // normal yz, emission xy
  float4 f2;    // emission z, base colour xyz
};

struct __align__(16) HitRec {
  float dist;
  int32_t ref;  // -1: miss; else slot | (mesh + 1) << 16
  int32_t face;
  float u, v;
  float nx, ny, nz;
};

struct __align__(16) ShadowEntry {
  float4 o;  // origin, ray length
  float4 d;  // direction, target (int bits): path * nslot + slot
};

static_assert(sizeof(PathRec) == 128 && sizeof(HitRec) == 32 && sizeof(ShadowEntry) == 32, "record sizes");

// next-event record flags of a slot
constexpr int32_t kNeeSkip = 0;      // inactive light: nothing added
constexpr int32_t kNeeZero = 1;      // the light does not reach the point: zero added
constexpr int32_t kNeeAdd = 2;       // unshadowed contribution: added
constexpr int32_t kNeeIfVisible = 3; // added if its shadow ray is unoccluded

struct PtWaveMap {
  int32_t w0, nw;          // worlds of this chunk
  int32_t nsample;         // samples per pixel
  int32_t pixels;          // RGB pixels per world
  int32_t npath;           // paths of this chunk: nw * pixels * nsample
  int32_t nslot;           // next-event slots: nlight, the headlight, the environment
  int32_t pix_base[MJPBR_MAX_RENDER];  // first RGB pixel of each camera within a world (-1: no RGB)
  int32_t geo_base[MJPBR_MAX_RENDER + 1];  // pixels of the cameras without RGB (prefix sums)
  PathRec* path;
  HitRec* hit;
  float4* nee;             // (npath, 1 + nslot): the bounce's throughput, then each slot's term and flag
  uint8_t* vis;            // (npath, nslot)
  int32_t* queue[2];
  ShadowEntry* shadow;
  int32_t* counters;       // [0], [1] queue lengths, [2] shadow entries; 64-bit fetch counters of extend [4..5], shadow [6..7]
  int64_t path_cap, shadow_cap;
};

MJ_DEV Stack wave_stack(const MjpbrScene& s, float* base) {
  return shared_stack(base, kThreads, stack_entries(s.settings.stack_depth));
}

// World, camera, pixel id and sample of a chunk-local path index (paths: world-major, then RGB
// pixels in camera order, then samples).
MJ_DEV void path_pixel(const MjpbrScene& s, const PtWaveMap& wm, int32_t path, int32_t* w, Pixel* p, int32_t* sample) {
  const int32_t pix_all = path / wm.nsample;
  *sample = path - pix_all * wm.nsample;
  const int32_t wl = pix_all / wm.pixels;
  const int32_t pix = pix_all - wl * wm.pixels;
  int32_t cam = 0;
  for (int32_t k = 0; k < s.nrender; ++k) {
    if (wm.pix_base[k] >= 0 && wm.pix_base[k] <= pix) cam = k;
  }
  *w = wm.w0 + wl;
  p->cam = cam;
  p->width = s.cam_res[cam][0];
  p->height = s.cam_res[cam][1];
  p->pixelid = pix - wm.pix_base[cam];
  p->px = p->pixelid % p->width;
  p->py = p->pixelid / p->width;
}

MJ_DEV const float* world_block(const MjpbrScene& s, int32_t w) { return s.world_blocks + (int64_t)w * s.world_block_floats; }

MJ_DEV uint32_t pixel_seed_of(const MjpbrScene& s, uint32_t seed, int32_t w, const Pixel& p) {
  return seed + (uint32_t)w * (uint32_t)s.total_rays + (uint32_t)(s.ray_adr[p.cam] + p.pixelid);
}

MJ_DEV void store_path_hot(PathRec& r, const PathState& ps, float first_depth) {
  r.o = make_float4(ps.o.x, ps.o.y, ps.o.z, ps.max_dist);
  r.d = make_float4(ps.d.x, ps.d.y, ps.d.z, ps.pdf_prev);
  r.beta = make_float4(ps.beta.x, ps.beta.y, ps.beta.z, ps.dcam_z);
  r.rad = make_float4(ps.radiance.x, ps.radiance.y, ps.radiance.z, first_depth);
  r.meta = make_int4(ps.depth, ps.passes, ps.sample, (ps.camera_ray ? 1 : 0) | (ps.delta ? 2 : 0));
}

MJ_DEV void store_path_features(PathRec& r, const PathState& ps) {
  r.f0 = make_float4(ps.albedo.x, ps.albedo.y, ps.albedo.z, ps.normal.x);
  r.f1 = make_float4(ps.normal.y, ps.normal.z, ps.emission.x, ps.emission.y);
  r.f2 = make_float4(ps.emission.z, ps.base_color.x, ps.base_color.y, ps.base_color.z);
}

MJ_DEV void store_path(PathRec& r, const PathState& ps, float first_depth) {
  store_path_hot(r, ps, first_depth);
  store_path_features(r, ps);
}

MJ_DEV PathState load_path_hot(const PathRec& r, float* first_depth) {
  PathState ps;
  const float4 o = r.o, d = r.d, beta = r.beta, rad = r.rad;
  const int4 meta = r.meta;
  ps.o = V3{o.x, o.y, o.z};
  ps.max_dist = o.w;
  ps.d = V3{d.x, d.y, d.z};
  ps.pdf_prev = d.w;
  ps.beta = V3{beta.x, beta.y, beta.z};
  ps.dcam_z = beta.w;
  ps.radiance = V3{rad.x, rad.y, rad.z};
  *first_depth = rad.w;
  ps.depth = meta.x;
  ps.passes = meta.y;
  ps.sample = meta.z;
  ps.camera_ray = (meta.w & 1) != 0;
  ps.delta = (meta.w & 2) != 0;
  return ps;
}

MJ_DEV void load_path_features(const PathRec& r, PathState& ps) {
  const float4 f0 = r.f0, f1 = r.f1, f2 = r.f2;
  ps.albedo = V3{f0.x, f0.y, f0.z};
  ps.normal = V3{f0.w, f1.x, f1.y};
  ps.emission = V3{f1.z, f1.w, f2.x};
  ps.base_color = V3{f2.y, f2.z, f2.w};
}

MJ_DEV PathState load_path(const PathRec& r, float* first_depth) {
  PathState ps = load_path_hot(r, first_depth);
  load_path_features(r, ps);
  return ps;
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
  if (r.ref == -1) {
    h.geom = h.slot = h.mesh = h.face = -1;
    h.u = h.v = 0.0f;
    h.normal = v3(0.0f);
    return h;
  }
  h.slot = r.ref & 0xffff;
  h.mesh = (r.ref >> 16) - 1;
  h.geom = __float_as_int(blk[L.geom_off + h.slot * kGeomFloats + 16]);
  h.face = r.face;
  h.u = r.u;
  h.v = r.v;
  h.normal = V3{r.nx, r.ny, r.nz};
  return h;
}

// Appends one entry per thread with `want` as one contiguous run per CTA (one atomic per CTA;
// warps in order, lanes in order). Every thread of the CTA must make the call; `scan` holds
// kThreads / 32 + 1 ints of shared memory. Returns the thread's position or -1.
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
  __syncthreads();
  if (!want) return -1;
  const int64_t pos = base + __popc(m & ((1u << lane) - 1u));
  if (pos >= cap) {
    *err |= kErrWorkQueue;
    return -1;
  }
  return pos;
}

// Next-event estimation of the wavefront: each slot's term is recorded in the path's record and
// its shadow ray appended to the shadow queue at once (one atomic per group of converged lanes);
// the shadow stage traces the rays and the next extend (or resolve) adds the terms.
struct RecordedNee {
  float4* rec;  // [0] beta, active; [1 + k] slot k's contribution, flag
  int32_t nslot, path;
  V3 origin;
  const PtWaveMap* wm;
  int32_t* err;
  MJ_DEV void begin(const PathState& ps, V3 o) {
    rec[0] = make_float4(ps.beta.x, ps.beta.y, ps.beta.z, __int_as_float(0));
    origin = o;
    for (int32_t k = 0; k < nslot; ++k) rec[1 + k].w = __int_as_float(kNeeSkip);
  }
  MJ_DEV void shadow_ray(int32_t slot, V3 dir, float len) {
    cg::coalesced_group g = cg::coalesced_threads();
    int32_t base = 0;
    if (g.thread_rank() == 0) base = atomicAdd(wm->counters + 2, (int32_t)g.size());
    const int64_t pos = (int64_t)g.shfl(base, 0) + g.thread_rank();
    if (pos >= wm->shadow_cap) {
      *err |= kErrWorkQueue;
      return;
    }
    ShadowEntry e;
    e.o = make_float4(origin.x, origin.y, origin.z, len);
    e.d = make_float4(dir.x, dir.y, dir.z, __int_as_float(path * nslot + slot));
    wm->shadow[pos] = e;
  }
  MJ_DEV void none(int32_t slot) { rec[1 + slot].w = __int_as_float(kNeeZero); }
  template <class F>
  MJ_DEV void light(RtCtx&, int32_t slot, bool shadowed, V3, V3 dir, float max_t, F contribution) {
    const V3 c = contribution();
    rec[1 + slot] = make_float4(c.x, c.y, c.z, __int_as_float(shadowed ? kNeeIfVisible : kNeeAdd));
    if (shadowed) shadow_ray(slot, dir, max_t);
  }
  MJ_DEV void lights_done(PathState&) { rec[0].w = __int_as_float(1); }
  template <class F>
  MJ_DEV void env(RtCtx&, PathState&, V3, V3 dir, F term) {
    const int32_t slot = nslot - 1;
    const V3 t = term();
    rec[1 + slot] = make_float4(t.x, t.y, t.z, __int_as_float(kNeeIfVisible));
    shadow_ray(slot, dir, kUnboundedShadow);
  }
};

// ---------------------------------------------------------------- next-event terms
// Adds a path's recorded next-event terms of its last shaded bounce to its radiance (the light
// terms in light order, times the bounce's throughput, then the environment term), each one only
// if its shadow ray was unoccluded, and marks the record applied. Run by the next bounce's extend
// stage before the path's next hit, and by the resolve stage for the paths that ended: the same
// additions in the same order as the persistent kernel.
MJ_DEV void apply_nee(const PtWaveMap& wm, int32_t path, PathRec& r) {
  float4* rec = wm.nee + (int64_t)path * (1 + wm.nslot);
  const float4 head = rec[0];
  if (__float_as_int(head.w) == 0) return;
  const int32_t nlights = wm.nslot - 1;  // the model's lights and the headlight
  const uint8_t* vis = wm.vis + (int64_t)path * wm.nslot;
  V3 direct = v3(0.0f);
  for (int32_t k = 0; k < nlights; ++k) {
    const float4 c = rec[1 + k];
    const int32_t flag = __float_as_int(c.w);
    if (flag == kNeeSkip) continue;
    const bool add = flag == kNeeAdd || (flag == kNeeIfVisible && vis[k]);
    direct += add ? V3{c.x, c.y, c.z} : v3(0.0f);
  }
  V3 radiance{r.rad.x, r.rad.y, r.rad.z};
  radiance += cmul(V3{head.x, head.y, head.z}, direct);
  const float4 e = rec[1 + nlights];
  if (__float_as_int(e.w) == kNeeIfVisible && vis[nlights]) radiance += V3{e.x, e.y, e.z};
  r.rad = make_float4(radiance.x, radiance.y, radiance.z, r.rad.w);
  rec[0].w = __int_as_float(0);
}

// ---------------------------------------------------------------- cameras without RGB
template <bool kMesh>
__global__ void __launch_bounds__(kThreads) ptw_geometry_kernel(const __grid_constant__ MjpbrScene s,
                                                                const __grid_constant__ PtWaveMap wm) {
  extern __shared__ __align__(16) float smem[];
  const Stack st = wave_stack(s, smem);
  const int32_t per_world = wm.geo_base[s.nrender];
  const int32_t i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= per_world * wm.nw) return;
  const int32_t wl = i / per_world, pix = i - wl * per_world;
  int32_t cam = 0;
  while (cam + 1 < s.nrender && pix >= wm.geo_base[cam + 1]) ++cam;
  const int32_t w = wm.w0 + wl;
  const BlockLayout L = block_layout(s.nbvh_geom, s.nnode, s.nlight, s.nrender);
  const float* blk = world_block(s, w);
  Pixel p;
  p.cam = cam;
  p.width = s.cam_res[cam][0];
  p.height = s.cam_res[cam][1];
  p.pixelid = pix - wm.geo_base[cam];
  p.px = p.pixelid % p.width;
  p.py = p.pixelid / p.width;
  p.rec = blk + L.cam_off + cam * kCamFloats;
  const M3 R = cam_mat(p.rec);
  const V3 cpos{p.rec[0], p.rec[1], p.rec[2]};
  V3 dcam, ocam;
  float max_dist, depth_z;
  primary_ray(s, p, kSubpixel, kSubpixel / 2, kSubpixel / 2, &dcam, &ocam, &max_dist, &depth_z);
  int32_t err = 0;
  const Hit hit = trace_ray<kMesh>(s, st, blk, L, Ray{cpos + mul(R, ocam), mul(R, dcam)}, max_dist, s.settings.cull_backfaces != 0,
                                   false, &err);
  write_geometry(s, w, p, hit, depth_z);
  if (err && s.error_word) atomicOr(s.error_word, err);
}

// ---------------------------------------------------------------- extend
// Steps a lane of the traversal stages runs between refills of the warp's idle lanes.
#ifndef MJPBR_PTW_REFILL_STEPS
#define MJPBR_PTW_REFILL_STEPS 32
#endif

// Closest hit of every live path, lanes refilled from the queue (refill.cuh); the pending
// next-event terms of the path's last bounce are added first.
template <bool kMesh>
__global__ void __launch_bounds__(kThreads, 3) ptw_extend_kernel(const __grid_constant__ MjpbrScene s,
                                                                 const __grid_constant__ PtWaveMap wm, int32_t cur, bool pending_nee) {
  extern __shared__ __align__(16) float smem[];
  const Stack st = wave_stack(s, smem);
  const BlockLayout L = block_layout(s.nbvh_geom, s.nnode, s.nlight, s.nrender);
  const bool cull = s.settings.cull_backfaces != 0;
  const int64_t items = min((int64_t)wm.counters[cur], wm.path_cap);
  int32_t err = 0;
  ClosestQuery q;
  const float* blk = nullptr;
  int32_t path = -1;
  refill_loop<MJPBR_PTW_REFILL_STEPS>(
      items, reinterpret_cast<unsigned long long*>(wm.counters + 4), q,
      [&](int64_t item, ClosestQuery& qq) {
        path = wm.queue[cur][item];
        PathRec& r = wm.path[path];
        if (pending_nee) apply_nee(wm, path, r);
        const float4 o = r.o, d = r.d;
        blk = world_block(s, wm.w0 + (path / wm.nsample) / wm.pixels);
        closest_begin(qq, st, Ray{V3{o.x, o.y, o.z}, V3{d.x, d.y, d.z}}, o.w, &err);
        return true;
      },
      [&](ClosestQuery& qq) { return closest_step<kMesh>(qq, s, st, blk, L, cull, &err); },
      [&](ClosestQuery& qq, int32_t) {
        const Hit& hit = qq.h;
        wm.hit[path] = pack_hit(hit);
        PathRec& r = wm.path[path];
        const int4 meta = r.meta;
        const int32_t sample = meta.z;
        const int32_t passes = meta.y;
        const bool camera_ray = (meta.w & 1) != 0;
        if (camera_ray && passes == 0 && sample == 0) {
          int32_t ww, smp;
          Pixel p;
          path_pixel(s, wm, path, &ww, &p, &smp);
          const float dcam_z = r.beta.w;
          write_geometry(s, ww, p, hit, dcam_z);
          if (hit.geom != -1) r.rad.w = hit.dist * -dcam_z;
        }
      },
      &err);
  if (err && s.error_word) atomicOr(s.error_word, err);
}

// The first bounce's extend, with the start folded in: each path's camera ray is generated where
// it is traced (start_sample, pt_bounce.cuh) and the path record written once, after the hit; the
// path queue of the shade stage is the identity.
template <bool kMesh>
__global__ void __launch_bounds__(kThreads, 3) ptw_first_extend_kernel(const __grid_constant__ MjpbrScene s, uint32_t seed,
                                                                       const __grid_constant__ PtWaveMap wm) {
  extern __shared__ __align__(16) float smem[];
  const Stack st = wave_stack(s, smem);
  const BlockLayout L = block_layout(s.nbvh_geom, s.nnode, s.nlight, s.nrender);
  const bool cull = s.settings.cull_backfaces != 0;
  if (blockIdx.x == 0 && threadIdx.x == 0) wm.counters[0] = wm.npath;  // the shade stage's queue
  int32_t err = 0;
  ClosestQuery q;
  const float* blk = nullptr;
  int32_t path = -1;
  // the path's start state (the same for the ray and for the record stored after the hit)
  auto start = [&](int32_t i, PathState& ps, Pixel& p, int32_t& w, int32_t& sample) {
    path_pixel(s, wm, i, &w, &p, &sample);
    p.rec = world_block(s, w) + L.cam_off + p.cam * kCamFloats;
    const M3 R = cam_mat(p.rec);
    const V3 cpos{p.rec[0], p.rec[1], p.rec[2]};
    start_sample(ps, s, p, pixel_seed_of(s, seed, w, p), R, cpos, sample);
  };
  refill_loop<MJPBR_PTW_REFILL_STEPS>(
      wm.npath, reinterpret_cast<unsigned long long*>(wm.counters + 4), q,
      [&](int64_t item, ClosestQuery& qq) {
        path = (int32_t)item;
        wm.queue[0][path] = path;
        PathState ps;
        Pixel p;
        int32_t w, sample;
        start(path, ps, p, w, sample);
        blk = world_block(s, w);
        closest_begin(qq, st, Ray{ps.o, ps.d}, ps.max_dist, &err);
        return true;
      },
      [&](ClosestQuery& qq) { return closest_step<kMesh>(qq, s, st, blk, L, cull, &err); },
      [&](ClosestQuery& qq, int32_t) {
        const Hit& hit = qq.h;
        wm.hit[path] = pack_hit(hit);
        PathState ps;
        Pixel p;
        int32_t w, sample;
        start(path, ps, p, w, sample);
        float first_depth = 0.0f;
        if (sample == 0) {
          write_geometry(s, w, p, hit, ps.dcam_z);
          if (hit.geom != -1) first_depth = hit.dist * -ps.dcam_z;
        }
        store_path(wm.path[path], ps, first_depth);
      },
      &err);
  if (err && s.error_word) atomicOr(s.error_word, err);
}

// ---------------------------------------------------------------- shade
template <bool kMesh, bool kTex>
__global__ void __launch_bounds__(kThreads, MJPBR_PTW_SHADE_CTAS) ptw_shade_kernel(const __grid_constant__ MjpbrScene s, uint32_t seed,
                                                                const __grid_constant__ PtWaveMap wm, int32_t cur) {
  __shared__ int32_t scan[kThreads / 32 + 1];
  const BlockLayout L = block_layout(s.nbvh_geom, s.nnode, s.nlight, s.nrender);
  const int32_t next = cur ^ 1;
  const int32_t count = (int32_t)min((int64_t)wm.counters[cur], wm.path_cap);
  const int32_t stride = gridDim.x * kThreads;
  const int32_t rounds = (count + stride - 1) / stride;
  int32_t err = 0;
  for (int32_t round = 0; round < rounds; ++round) {
    const int32_t i = round * stride + blockIdx.x * kThreads + threadIdx.x;
    int32_t path = -1;
    bool live = false;
    if (i < count) {
      path = wm.queue[cur][i];
      int32_t w, sample;
      Pixel p;
      path_pixel(s, wm, path, &w, &p, &sample);
      const float* blk = world_block(s, w);
      RtCtx c;
      init_ctx(c, s, blk, L, w, kTex);
      p.rec = blk + L.cam_off + p.cam * kCamFloats;
      const M3 R = cam_mat(p.rec);
      const V3 head_dir = -V3{R.m[2], R.m[5], R.m[8]};
      PathRec& r = wm.path[path];
      float first_depth;
      PathState ps = load_path_hot(r, &first_depth);
      // only a camera ray's bounce can set the first surface's features
      const bool features = ps.camera_ray;
      if (features) load_path_features(r, ps);
      const Hit hit = unpack_hit(wm.hit[path], blk, L);
      float4* rec = wm.nee + (int64_t)path * (1 + wm.nslot);
      rec[0].w = __int_as_float(0);
      RecordedNee nee{rec, wm.nslot, path, v3(0.0f), &wm, &err};
      live = !PtCore<kMesh, kTex>::surface(c, nee, ps, hit, pixel_seed_of(s, seed, w, p), head_dir);
      store_path_hot(r, ps, first_depth);
      if (features) store_path_features(r, ps);
      err |= c.err;
    }
    // the paths that continue
    const int64_t pos = cta_append(live, wm.counters + next, wm.path_cap, scan, &err);
    if (pos >= 0) wm.queue[next][pos] = path;
  }
  if (err && s.error_word) atomicOr(s.error_word, err);
}

// ---------------------------------------------------------------- shadow rays
// Any hit of every recorded shadow ray, lanes refilled from the queue (refill.cuh).
template <bool kMesh>
__global__ void __launch_bounds__(kThreads, 3) ptw_shadow_kernel(const __grid_constant__ MjpbrScene s,
                                                                 const __grid_constant__ PtWaveMap wm) {
  extern __shared__ __align__(16) float smem[];
  const Stack st = wave_stack(s, smem);
  const BlockLayout L = block_layout(s.nbvh_geom, s.nnode, s.nlight, s.nrender);
  const bool cull = s.settings.cull_backfaces != 0;
  const int64_t items = min((int64_t)wm.counters[2], wm.shadow_cap);
  int32_t err = 0;
  AnyQuery q;
  const float* blk = nullptr;
  int32_t target = -1;
  refill_loop<MJPBR_PTW_REFILL_STEPS>(
      items, reinterpret_cast<unsigned long long*>(wm.counters + 6), q,
      [&](int64_t item, AnyQuery& qq) {
        const ShadowEntry e = wm.shadow[item];
        target = __float_as_int(e.d.w);
        const int32_t path = target / wm.nslot;
        blk = world_block(s, wm.w0 + (path / wm.nsample) / wm.pixels);
        any_begin(qq, st, Ray{V3{e.o.x, e.o.y, e.o.z}, V3{e.d.x, e.d.y, e.d.z}}, e.o.w, &err);
        return true;
      },
      [&](AnyQuery& qq) { return any_step<kMesh>(qq, s, st, blk, L, cull, &err); },
      [&](AnyQuery&, int32_t res) { wm.vis[target] = res == kAnyClear ? 1 : 0; }, &err);
  if (err && s.error_word) atomicOr(s.error_word, err);
}

// ---------------------------------------------------------------- pixels
template <bool kTex>
__global__ void __launch_bounds__(kThreads) ptw_resolve_kernel(const __grid_constant__ MjpbrScene s, const __grid_constant__ PtWaveMap wm) {
  const int32_t pix_all = blockIdx.x * kThreads + threadIdx.x;
  if (pix_all >= wm.nw * wm.pixels) return;
  int32_t w, sample;
  Pixel p;
  path_pixel(s, wm, pix_all * wm.nsample, &w, &p, &sample);
  const BlockLayout L = block_layout(s.nbvh_geom, s.nnode, s.nlight, s.nrender);
  RtCtx c;
  init_ctx(c, s, world_block(s, w), L, w, kTex);
  PixelAcc acc;
  clear_pixel(acc);
  for (int32_t k = 0; k < wm.nsample; ++k) {
    float first_depth;
    const int32_t path = pix_all * wm.nsample + k;
    apply_nee(wm, path, wm.path[path]);
    const PathState ps = load_path(wm.path[path], &first_depth);
    if (k == 0) acc.first_depth = first_depth;
    add_sample(acc, ps, s.settings.denoise != 0, c.exposure);
  }
  write_pixel(s, c, (int64_t)w * s.rgb_stride + s.rgb_adr[p.cam] + p.pixelid, acc, wm.nsample);
}

// ---------------------------------------------------------------- host side

int64_t align256(int64_t b) { return (b + 255) & ~int64_t(255); }

int32_t slots_of(const MjpbrScene& s) { return std::max(s.nlight, 0) + 2; }

void rgb_pixels(const MjpbrScene& s, int32_t* pix_base, int32_t* geo_base, int64_t* pixels) {
  int64_t rgb = 0, geo = 0;
  geo_base[0] = 0;
  for (int32_t c = 0; c < s.nrender; ++c) {
    const int64_t npix = (int64_t)s.cam_res[c][0] * s.cam_res[c][1];
    pix_base[c] = s.render_rgb[c] ? (int32_t)rgb : -1;
    if (s.render_rgb[c]) rgb += npix;
    if (!s.render_rgb[c] && (s.render_depth[c] || s.render_seg[c])) geo += npix;
    geo_base[c + 1] = (int32_t)geo;
  }
  for (int32_t c = s.nrender; c < MJPBR_MAX_RENDER; ++c) pix_base[c] = -1;
  *pixels = rgb;
}

int64_t layout(PtWaveMap* wm, char* base, int64_t npath, int32_t nslot) {
  int64_t off = 0;
  auto take = [&](int64_t bytes) {
    char* p = base + off;
    off += align256(bytes);
    return p;
  };
  char* counters = take(256);
  char* path = take(npath * (int64_t)sizeof(PathRec));
  char* hit = take(npath * (int64_t)sizeof(HitRec));
  char* nee = take(npath * (1 + (int64_t)nslot) * 16);
  char* vis = take(npath * nslot);
  char* q0 = take(npath * 4);
  char* q1 = take(npath * 4);
  char* shadow = take(npath * nslot * (int64_t)sizeof(ShadowEntry));
  if (wm) {
    wm->counters = reinterpret_cast<int32_t*>(counters);
    wm->path = reinterpret_cast<PathRec*>(path);
    wm->hit = reinterpret_cast<HitRec*>(hit);
    wm->nee = reinterpret_cast<float4*>(nee);
    wm->vis = reinterpret_cast<uint8_t*>(vis);
    wm->queue[0] = reinterpret_cast<int32_t*>(q0);
    wm->queue[1] = reinterpret_cast<int32_t*>(q1);
    wm->shadow = reinterpret_cast<ShadowEntry*>(shadow);
    wm->path_cap = npath;
    wm->shadow_cap = npath * nslot;
  }
  return off;
}

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

template <bool kMesh, bool kTex>
int launch_pt_wave(const MjpbrScene& s, uint32_t seed, cudaStream_t stream, int32_t chunk, int64_t pixels) {
  const size_t stack = (size_t)kThreads * stack_entries(s.settings.stack_depth) * 8;
  auto k_geometry = ptw_geometry_kernel<kMesh>;
  auto k_extend = ptw_extend_kernel<kMesh>;
  auto k_first = ptw_first_extend_kernel<kMesh>;
  auto k_shade = ptw_shade_kernel<kMesh, kTex>;
  auto k_shadow = ptw_shadow_kernel<kMesh>;
  auto k_resolve = ptw_resolve_kernel<kTex>;
  int rc = set_smem(k_geometry, stack, "path wavefront geometry");
  if (!rc) rc = set_smem(k_extend, stack, "path wavefront extend");
  if (!rc) rc = set_smem(k_first, stack, "path wavefront first extend");
  if (!rc) rc = set_smem(k_shadow, stack, "path wavefront shadow");
  if (rc) return rc;
  const int sms = device_sm_count();
  const int g_extend = sms * resident_ctas(k_extend, stack);
  const int g_first = sms * resident_ctas(k_first, stack);
  const int g_shade = sms * resident_ctas(k_shade, 0);
  const int g_shadow = sms * resident_ctas(k_shadow, stack);
  PtWaveMap wm;
  wm.nsample = s.settings.path_samples;
  wm.pixels = (int32_t)pixels;
  wm.nslot = slots_of(s);
  rgb_pixels(s, wm.pix_base, wm.geo_base, &pixels);
  layout(&wm, static_cast<char*>(s.wave_scratch), (int64_t)chunk * pixels * wm.nsample, wm.nslot);
  const int32_t geo_pixels = wm.geo_base[s.nrender];
  const int32_t iterations = s.settings.max_depth + 1 + (s.settings.has_transparency ? 4 * s.settings.max_layers : 0);
  const bool shadows = true;  // every bounce may ask for shadow rays (lights, environment)
  for (int32_t w0 = 0; w0 < s.nworld; w0 += chunk) {
    wm.w0 = w0;
    wm.nw = std::min(chunk, s.nworld - w0);
    wm.npath = (int32_t)((int64_t)wm.nw * pixels * wm.nsample);
    if (geo_pixels > 0) {
      const int64_t n = (int64_t)geo_pixels * wm.nw;
      k_geometry<<<(unsigned)((n + kThreads - 1) / kThreads), kThreads, stack, stream>>>(s, wm);
      if ((rc = check_launch("ptw_geometry_kernel"))) return rc;
    }
    if (wm.npath == 0) continue;
    // queue lengths and the fetch counters; the first extend sets the shade stage's queue length
    cudaError_t ez = cudaMemsetAsync(wm.counters, 0, 8 * sizeof(int32_t), stream);
    if (ez != cudaSuccess) return set_error(MJPBR_ERR_CUDA, "path wavefront counters: %s", cudaGetErrorString(ez));
    for (int32_t it = 0; it < iterations; ++it) {
      const int32_t cur = it & 1, next = cur ^ 1;
      if (it == 0) {
        k_first<<<g_first, kThreads, stack, stream>>>(s, seed, wm);
        if ((rc = check_launch("ptw_first_extend_kernel"))) return rc;
      } else {
        k_extend<<<g_extend, kThreads, stack, stream>>>(s, wm, cur, true);
        if ((rc = check_launch("ptw_extend_kernel"))) return rc;
      }
      cudaError_t e = cudaMemsetAsync(wm.counters + next, 0, sizeof(int32_t), stream);
      // shadow entries [2], the fetch counters of the next extend [4..5] and of the shadow stage [6..7]
      if (e == cudaSuccess) e = cudaMemsetAsync(wm.counters + 2, 0, 6 * sizeof(int32_t), stream);
      if (e != cudaSuccess) return set_error(MJPBR_ERR_CUDA, "path wavefront queue counters: %s", cudaGetErrorString(e));
      k_shade<<<g_shade, kThreads, 0, stream>>>(s, seed, wm, cur);
      if ((rc = check_launch("ptw_shade_kernel"))) return rc;
      if (shadows) {
        k_shadow<<<g_shadow, kThreads, stack, stream>>>(s, wm);
        if ((rc = check_launch("ptw_shadow_kernel"))) return rc;
      }
    }
    const int64_t npix = (int64_t)wm.nw * pixels;
    k_resolve<<<(unsigned)((npix + kThreads - 1) / kThreads), kThreads, 0, stream>>>(s, wm);
    if ((rc = check_launch("ptw_resolve_kernel"))) return rc;
  }
  return MJPBR_OK;
}

}  // namespace

int64_t pt_wave_scratch_bytes(const MjpbrScene& s, int32_t worlds) {
  int32_t pix_base[MJPBR_MAX_RENDER], geo_base[MJPBR_MAX_RENDER + 1];
  int64_t pixels = 0;
  rgb_pixels(s, pix_base, geo_base, &pixels);
  if (worlds < 0 || s.settings.path_samples < 1) return -1;
  return layout(nullptr, nullptr, (int64_t)worlds * pixels * s.settings.path_samples, slots_of(s));
}

// The path wavefront's records pack geom slots and triangle BVH ids in 16 bits; larger scenes render
// with the persistent path kernel (the same images).
bool pt_wave_supported(const MjpbrScene& s) { return s.nbvh_geom <= 0xffff && s.nmesh + s.nhfield < 0x7fff; }

int render_pt_wave_launch(const MjpbrScene& s, uint32_t seed, cudaStream_t stream) {
  if (!pt_wave_supported(s)) {
    return set_error(MJPBR_ERR_UNSUPPORTED, "the path wavefront packs slots and triangle BVHs in 16 bits; use the grid schedule");
  }
  if (!s.wave_scratch || (reinterpret_cast<uintptr_t>(s.wave_scratch) & 255u)) {
    return set_error(MJPBR_ERR_ARG, "the path wavefront needs wave_scratch (256-byte aligned)");
  }
  int32_t pix_base[MJPBR_MAX_RENDER], geo_base[MJPBR_MAX_RENDER + 1];
  int64_t pixels = 0;
  rgb_pixels(s, pix_base, geo_base, &pixels);
  // worlds per chunk: as many as the scratch holds, with path and shadow-target indices in int32
  int32_t chunk = s.nworld;
  if (pixels > 0) {
    const int64_t per_world = pixels * s.settings.path_samples * slots_of(s);
    chunk = (int32_t)std::min<int64_t>(chunk, INT32_MAX / std::max<int64_t>(per_world, 1));
    if (pt_wave_scratch_bytes(s, chunk) > s.wave_scratch_bytes) {
      int32_t lo = 0, hi = chunk;
      while (lo < hi) {
        const int32_t mid = lo + (hi - lo + 1) / 2;
        if (pt_wave_scratch_bytes(s, mid) <= s.wave_scratch_bytes) {
          lo = mid;
        } else {
          hi = mid - 1;
        }
      }
      chunk = lo;
    }
    if (chunk < 1) {
      return set_error(MJPBR_ERR_ARG, "wave_scratch of %lld bytes holds no world (one needs %lld)", (long long)s.wave_scratch_bytes,
                       (long long)pt_wave_scratch_bytes(s, 1));
    }
  }
  const bool mesh = s.nmesh + s.nhfield > 0 && s.blas_root != nullptr;
  const bool tex = s.settings.textures || s.settings.has_env || s.settings.env_background;
  if (mesh && tex) return launch_pt_wave<true, true>(s, seed, stream, chunk, pixels);
  if (mesh) return launch_pt_wave<true, false>(s, seed, stream, chunk, pixels);
  if (tex) return launch_pt_wave<false, true>(s, seed, stream, chunk, pixels);
  return launch_pt_wave<false, false>(s, seed, stream, chunk, pixels);
}

}  // namespace mjpbr

#ifdef MJPBR_COUNT_OPS
namespace mjpbr {
// Counting build: this unit's copy of the counter array pointer (see opcount.cuh).
int pt_wave_count_set(void* counts) { return cudaMemcpyToSymbol(g_op_counts, &counts, sizeof(counts)) == cudaSuccess ? 0 : 1; }
}  // namespace mjpbr
#endif
