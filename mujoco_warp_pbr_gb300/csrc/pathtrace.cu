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
#include "pt_bounce.cuh"

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

// Next-event estimation of the persistent kernel: every shadow ray is traced where it is asked.
template <bool kMesh>
struct TracedNee {
  V3 direct;
  MJ_DEV bool occluded(RtCtx& c, V3 o, V3 d, float max_t) {
    return trace_ray<kMesh>(*c.s, c.st, c.blk, c.L, Ray{o, d}, max_t, c.s->settings.cull_backfaces != 0, true, &c.err).geom != -1;
  }
  MJ_DEV void begin(const PathState&, V3) { direct = v3(0.0f); }
  MJ_DEV void none(int32_t) { direct += v3(0.0f); }
  template <class F>
  MJ_DEV void light(RtCtx& c, int32_t, bool shadowed, V3 origin, V3 dir, float max_t, F contribution) {
    if (shadowed && occluded(c, origin, dir, max_t)) {
      direct += v3(0.0f);
      return;
    }
    direct += contribution();
  }
  MJ_DEV void lights_done(PathState& ps) { ps.radiance += cmul(ps.beta, direct); }
  template <class F>
  MJ_DEV void env(RtCtx& c, PathState& ps, V3 origin, V3 dir, F term) {
    if (!occluded(c, origin, dir, kUnboundedShadow)) ps.radiance += term();
  }
};

template <bool kMesh, bool kTex>
struct Pt {
  static MJ_DEV Hit trace(RtCtx& c, V3 o, V3 d, float max_dist, bool any) {
    return trace_ray<kMesh>(*c.s, c.st, c.blk, c.L, Ray{o, d}, max_dist, c.s->settings.cull_backfaces != 0, any, &c.err);
  }

  // One iteration of the bounce loop (pathtrace.py:230-337); true when the path has ended.
  static MJ_DEV bool bounce(RtCtx& c, PathState& ps, PixelAcc& acc, const Pixel& p, uint32_t seed, V3 head_dir) {
    const MjpbrScene& s = *c.s;
    if (ps.depth > s.settings.max_depth) return true;
    Hit hit = trace(c, ps.o, ps.d, ps.max_dist, false);
    if (ps.camera_ray && ps.passes == 0 && ps.sample == 0) {
      write_geometry(s, c.w, p, hit, ps.dcam_z);
      if (hit.geom != -1) acc.first_depth = hit.dist * -ps.dcam_z;
    }
    TracedNee<kMesh> nee;
    return PtCore<kMesh, kTex>::surface(c, nee, ps, hit, seed, head_dir);
  }
};

template <bool kMesh, bool kTex, bool kStaged>
__global__ void __launch_bounds__(kThreads, 2) pt_kernel(const __grid_constant__ MjpbrScene s, uint32_t seed,
                                                         const __grid_constant__ PtTiles tm) {
  extern __shared__ __align__(16) float smem[];
  __shared__ int32_t s_tile, s_next;
  const BlockLayout L = block_layout(s.nbvh_geom, s.nnode, s.nlight, s.nrender);
  const MjpbrSettings& st = s.settings;
  const int lane = threadIdx.x & 31;
  const unsigned full = 0xffffffffu;
  RtCtx c;
  c.st = shared_stack(smem + (kStaged ? s.world_block_floats : 0), kThreads, stack_entries(st.stack_depth));
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
    const float* blk = world_block_of<kStaged>(s, w, smem, kThreads);
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
                clear_pixel(acc);
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
      add_sample(acc, ps, st.denoise != 0, c.exposure);
      if (ps.sample + 1 < nsample) {
        start_sample(ps, s, p, pixel_seed, R, cpos, ps.sample + 1);
        continue;
      }
      // the pixel's last sample: write it
      has_pixel = false;
      write_pixel(s, c, (int64_t)w * s.rgb_stride + s.rgb_adr[cam] + p.pixelid, acc, nsample);
    }
    err |= c.err;
    __syncthreads();  // every lane done with this tile's block before the next one is staged
  }
  if (err && s.error_word) atomicOr(s.error_word, err);
}

template <bool kMesh, bool kTex, bool kStaged>
int launch_variant(const MjpbrScene& s, uint32_t seed, const PtTiles& tm, cudaStream_t stream) {
  size_t smem = (kStaged ? (size_t)s.world_block_floats * sizeof(float) : 0) + (size_t)kThreads * stack_entries(s.settings.stack_depth) * 8;
  auto kern = pt_kernel<kMesh, kTex, kStaged>;
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
  if (s.settings.schedule == MJPBR_SCHEDULE_WAVEFRONT && pt_wave_supported(s)) return render_pt_wave_launch(s, seed, stream);
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
  const int64_t total = (int64_t)tm.tiles_per_world * s.nworld;
  if (total > INT32_MAX) return set_error(MJPBR_ERR_ARG, "path tracer: %lld tiles exceed the work counter", (long long)total);
  tm.total = (int32_t)total;
  if (tm.total == 0) return MJPBR_OK;
  bool mesh = s.nmesh + s.nhfield > 0 && s.blas_root != nullptr;
  bool tex = s.settings.textures || s.settings.has_env || s.settings.env_background;
  if (world_block_staged(s.world_block_floats, (size_t)kThreads * stack_entries(s.settings.stack_depth) * 8)) {
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
// Counting build only: this unit's copy of the counter array pointer (set by mjpbr_count_set).
int pt_count_set(void* counts) { return cudaMemcpyToSymbol(g_op_counts, &counts, sizeof(counts)) == cudaSuccess ? 0 : 1; }
}  // namespace mjpbr
#endif
