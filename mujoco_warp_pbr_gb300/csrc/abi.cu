// C entry points of libmjpbr (declared in include/mjpbr.h): argument checks, error reporting and
// dispatch to the kernel launchers. Nothing here synchronises or allocates.
#include <atomic>
#include <map>
#include <mutex>
#include <utility>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <string>

#include "abi_internal.h"
#include "common.cuh"
#include "world_block.cuh"

namespace mjpbr {

namespace {
thread_local std::string g_last_error;
}

int set_error(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(MJPBR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return MJPBR_OK;
}

namespace {

constexpr int kMaxSmDevices = 64;
std::atomic<int> g_device_sms[kMaxSmDevices];
std::atomic<int> g_device_smem[kMaxSmDevices];

}  // namespace

int device_sm_count() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  if (dev >= 0 && dev < kMaxSmDevices) {
    const int cached = g_device_sms[dev].load(std::memory_order_relaxed);
    if (cached > 0) return cached;
  }
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 1;
  if (dev >= 0 && dev < kMaxSmDevices) g_device_sms[dev].store(n, std::memory_order_relaxed);
  return n;
}

size_t device_max_smem() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 48 * 1024;
  if (dev >= 0 && dev < kMaxSmDevices) {
    const int cached = g_device_smem[dev].load(std::memory_order_relaxed);
    if (cached > 0) return (size_t)cached;
  }
  int n = 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess || n <= 0) n = 48 * 1024;
  if (dev >= 0 && dev < kMaxSmDevices) g_device_smem[dev].store(n, std::memory_order_relaxed);
  return (size_t)n;
}

int ensure_smem(const void* kern, size_t bytes, const char* what) {
  // also below 48 KB: a kernel's static shared memory counts against the default limit too
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return set_error(MJPBR_ERR_CUDA, "%s: no current device", what);
  static std::mutex lock;
  static std::map<std::pair<const void*, int>, size_t> raised;
  std::lock_guard<std::mutex> guard(lock);
  size_t& have = raised[{kern, dev}];
  if (bytes <= have) return MJPBR_OK;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return set_error(MJPBR_ERR_CUDA, "%s: %zu bytes of shared memory: %s", what, bytes, cudaGetErrorString(e));
  have = bytes;
  return MJPBR_OK;
}

bool world_block_staged(int32_t floats, size_t other) {
  // 8 KB of headroom for the kernels' static shared arrays
  return (size_t)floats * sizeof(float) + other + 8 * 1024 <= device_max_smem();
}

namespace {

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace

int validate_scene(const MjpbrScene* s, bool need_outputs) {
  if (!s) return set_error(MJPBR_ERR_ARG, "scene is NULL");
  if (s->abi_version != MJPBR_ABI_VERSION) {
    return set_error(MJPBR_ERR_ARG, "scene abi_version %d, library %d", s->abi_version, MJPBR_ABI_VERSION);
  }
  if (s->settings.schedule < MJPBR_SCHEDULE_GRID || s->settings.schedule > MJPBR_SCHEDULE_WAVEFRONT) {
    return set_error(MJPBR_ERR_ARG, "settings.schedule must be 0 (grid), 1 (queue) or 2 (wavefront), got %d", s->settings.schedule);
  }
  if (s->nworld < 1 || s->nworld > kMaxWorlds) return set_error(MJPBR_ERR_ARG, "nworld must be in [1, %d], got %d", kMaxWorlds, s->nworld);
  if (s->nrender < 1 || s->nrender > MJPBR_MAX_RENDER) {
    return set_error(MJPBR_ERR_ARG, "nrender must be in [1, %d], got %d", MJPBR_MAX_RENDER, s->nrender);
  }
  if (s->nbvh_geom < 1 || s->nnode != (s->nbvh_geom > 1 ? s->nbvh_geom - 1 : 1)) {
    return set_error(MJPBR_ERR_ARG, "scene BVH: %d geoms need %d nodes, got %d", s->nbvh_geom,
                     s->nbvh_geom > 1 ? s->nbvh_geom - 1 : 1, s->nnode);
  }
  if (!s->world_blocks || !aligned16(s->world_blocks)) return set_error(MJPBR_ERR_ARG, "world_blocks must be 16-byte aligned");
  BlockLayout L = block_layout(s->nbvh_geom, s->nnode, s->nlight, s->nrender);
  if (s->world_block_floats < L.total || (s->world_block_floats & 3)) {
    return set_error(MJPBR_ERR_ARG, "world_block_floats must be a multiple of 4 and >= %d, got %d", L.total,
                     s->world_block_floats);
  }
  if (!s->geom_type || !s->geom_xpos || !s->geom_xmat || !s->cam_xpos || !s->cam_xmat || !s->enabled_geom_ids ||
      !s->tlas_child.ptr || !s->geom_size.ptr || !s->geom_rgba.ptr || !s->geom_matid.ptr) {
    return set_error(MJPBR_ERR_ARG, "scene is missing a geometry or camera array");
  }
  if (s->nlight > 0 && (!s->light_xpos || !s->light_xdir || !s->light_type.ptr || !s->light_active.ptr ||
                        !s->light_castshadow.ptr || !s->light_intensity.ptr || !s->light_range.ptr ||
                        !s->light_bulbradius.ptr || !s->light_diffuse.ptr || !s->light_specular.ptr ||
                        !s->light_attenuation.ptr || !s->light_cutoff.ptr || !s->light_exponent.ptr)) {
    return set_error(MJPBR_ERR_ARG, "scene is missing a light array");
  }
  for (int32_t c = 0; c < s->nrender; ++c) {
    if (s->cam_res[c][0] < 1 || s->cam_res[c][1] < 1) return set_error(MJPBR_ERR_ARG, "camera %d has no pixels", c);
    if (s->cam_id_map[c] < 0 || s->cam_id_map[c] >= s->ncam) return set_error(MJPBR_ERR_ARG, "camera map %d invalid", c);
  }
  if (need_outputs) {
    if (!s->dfg_lut || s->dfg_size < 2) return set_error(MJPBR_ERR_ARG, "scene has no DFG table");
    if (!s->exposure.ptr || !s->ambient_radiance.ptr || !s->geom_metallic.ptr || !s->geom_roughness.ptr ||
        !s->geom_reflectance.ptr) {
      return set_error(MJPBR_ERR_ARG, "scene is missing a material or exposure table");
    }
    const MjpbrSettings& st = s->settings;
    if (st.samples_per_axis < 1 || st.shadow_samples < 1 || st.max_layers < 1) {
      return set_error(MJPBR_ERR_ARG, "samples_per_axis, shadow_samples and max_layers must be at least 1");
    }
    if ((st.has_env || st.env_background) && (s->nenv < 1 || !s->env_sh || !s->env_prefiltered || !s->env_radiance)) {
      return set_error(MJPBR_ERR_ARG, "environment lighting is on but the scene has no environment maps");
    }
    if (st.textures && (!s->textures || !s->tex_data || !s->mat_texid.ptr || !s->mat_texrepeat.ptr)) {
      return set_error(MJPBR_ERR_ARG, "textures are on but the scene has no textures");
    }
    for (int32_t c = 0; c < s->nrender; ++c) {
      if (s->render_rgb[c] && (s->rgb_adr[c] < 0 || !s->rgb_data)) return set_error(MJPBR_ERR_ARG, "rgb buffer missing");
      if (s->render_depth[c] && (s->depth_adr[c] < 0 || !s->depth_data)) {
        return set_error(MJPBR_ERR_ARG, "depth buffer missing");
      }
      if (s->render_seg[c] && (s->seg_adr[c] < 0 || !s->seg_data)) return set_error(MJPBR_ERR_ARG, "seg buffer missing");
    }
    // The pixel maps the kernels index with: every camera image must lie inside its output rows and
    // inside the per-world ray range, and the flattened (world, ray) indices must fit 32 bits.
    int64_t rays = 0;
    for (int32_t c = 0; c < s->nrender; ++c) {
      const int64_t npix = (int64_t)s->cam_res[c][0] * s->cam_res[c][1];
      rays += npix;
      if (s->ray_adr[c] < 0 || s->ray_adr[c] + npix > s->total_rays) {
        return set_error(MJPBR_ERR_ARG, "pixel map: camera %d rays [%d, %lld) outside total_rays %d", c, s->ray_adr[c],
                         (long long)(s->ray_adr[c] + npix), s->total_rays);
      }
      const struct {
        bool on;
        int32_t adr, stride;
        const char* name;
      } maps[3] = {{s->render_rgb[c] != 0, s->rgb_adr[c], s->rgb_stride, "rgb"},
                   {s->render_depth[c] != 0, s->depth_adr[c], s->depth_stride, "depth"},
                   {s->render_seg[c] != 0, s->seg_adr[c], s->seg_stride, "seg"}};
      for (const auto& m : maps) {
        if (m.on && (int64_t)m.adr + npix > m.stride) {
          return set_error(MJPBR_ERR_ARG, "pixel map: camera %d %s pixels [%d, %lld) outside the row of %d", c, m.name, m.adr,
                           (long long)(m.adr + npix), m.stride);
        }
      }
    }
    if (rays > s->total_rays || (int64_t)s->total_rays * s->nworld >= (int64_t(1) << 31)) {
      return set_error(MJPBR_ERR_ARG, "pixel map: %d worlds x %d rays overflow the 32-bit ray index", s->nworld, s->total_rays);
    }
    if (st.schedule == MJPBR_SCHEDULE_QUEUE && st.tier == MJPBR_TIER_REALTIME &&
        st.queue_item != 32 && st.queue_item != 64 && st.queue_item != 128) {
      return set_error(MJPBR_ERR_ARG, "work queue: items of %d pixels; 32, 64 or 128", st.queue_item);
    }
    if (s->wave_scratch_bytes < 0) return set_error(MJPBR_ERR_ARG, "wave_scratch_bytes is negative");
    if (st.stack_depth != 0 && (st.stack_depth < 8 || st.stack_depth > kStackDepth)) {
      return set_error(MJPBR_ERR_ARG, "settings.stack_depth %d: 0 or 8..%d entries", st.stack_depth, kStackDepth);
    }
  }
  return MJPBR_OK;
}

}  // namespace mjpbr

using namespace mjpbr;

extern "C" {

int mjpbr_abi_version(void) { return MJPBR_ABI_VERSION; }

const char* mjpbr_last_error(void) { return g_last_error.c_str(); }

void mjpbr_struct_layout(int64_t out[8]) {
  out[0] = (int64_t)sizeof(MjpbrScene);
  out[1] = (int64_t)sizeof(MjpbrSettings);
  out[2] = (int64_t)sizeof(MjpbrTexture);
  out[3] = (int64_t)offsetof(MjpbrScene, nrender);
  out[4] = (int64_t)offsetof(MjpbrScene, world_blocks);
  out[5] = (int64_t)offsetof(MjpbrScene, env_prefiltered);
  out[6] = (int64_t)offsetof(MjpbrScene, error_word);
  out[7] = (int64_t)offsetof(MjpbrScene, settings);
}

int32_t mjpbr_world_block_floats(int32_t nbvh_geom, int32_t nnode, int32_t nlight, int32_t nrender) {
  return block_layout(nbvh_geom, nnode, nlight, nrender).total;
}

int mjpbr_refit_bvh(const MjpbrScene* scene, void* stream) {
  int rc = validate_scene(scene, false);
  if (rc) return rc;
  return refit_launch(*scene, static_cast<cudaStream_t>(stream));
}

int mjpbr_render(const MjpbrScene* scene, uint32_t seed, void* stream) {
  int rc = validate_scene(scene, true);
  if (rc) return rc;
  if (scene->settings.tier == MJPBR_TIER_PATH) return render_pt_launch(*scene, seed, static_cast<cudaStream_t>(stream));
  return render_rt_launch(*scene, seed, static_cast<cudaStream_t>(stream));
}

int mjpbr_get_rgb(const MjpbrScene* scene, int32_t cam, float* out, int32_t nworld_out, void* stream) {
  if (!scene) return set_error(MJPBR_ERR_ARG, "scene is NULL");
  return outputs_launch(*scene, 0, cam, 1.0f, out, nworld_out, static_cast<cudaStream_t>(stream));
}

int mjpbr_get_depth(const MjpbrScene* scene, int32_t cam, float depth_scale, float* out, int32_t nworld_out,
                    void* stream) {
  if (!scene) return set_error(MJPBR_ERR_ARG, "scene is NULL");
  return outputs_launch(*scene, 1, cam, depth_scale, out, nworld_out, static_cast<cudaStream_t>(stream));
}

int mjpbr_get_segmentation(const MjpbrScene* scene, int32_t cam, int32_t* out, int32_t nworld_out, void* stream) {
  if (!scene) return set_error(MJPBR_ERR_ARG, "scene is NULL");
  return outputs_launch(*scene, 2, cam, 1.0f, out, nworld_out, static_cast<cudaStream_t>(stream));
}

int mjpbr_get_image(const MjpbrScene* scene, int32_t which, int32_t cam, float* out, int32_t nworld_out, void* stream) {
  if (!scene) return set_error(MJPBR_ERR_ARG, "scene is NULL");
  if (which < 0 || which > 2) return set_error(MJPBR_ERR_ARG, "which must be 0 (hdr), 1 (albedo) or 2 (normal)");
  return outputs_launch(*scene, 3 + which, cam, 1.0f, out, nworld_out, static_cast<cudaStream_t>(stream));
}

int mjpbr_newton_sync_poses(const float* body_q, int32_t nbody, const int32_t* shape_body, const float* shape_transform,
                            int32_t nshape, const int32_t* geom_shape, int32_t geom_shape_rows, const float* geom_offset,
                            const float* camera_transforms, int32_t nworld, int32_t ngeom, int32_t ncam, int32_t cam,
                            float* geom_xpos, float* geom_xmat, float* cam_xpos, float* cam_xmat, int32_t* error_word,
                            void* stream) {
  return newton_sync_poses_launch(body_q, nbody, shape_body, shape_transform, nshape, geom_shape, geom_shape_rows, geom_offset,
                                  camera_transforms, nworld, ngeom, ncam, cam, geom_xpos, geom_xmat, cam_xpos, cam_xmat,
                                  error_word, static_cast<cudaStream_t>(stream));
}

int mjpbr_newton_images(const MjpbrScene* scene, int32_t cam, const int32_t* geom_shape, int32_t geom_shape_rows,
                        const float* ray_scale, uint32_t* color, float* depth, float* forward_depth, uint32_t* shape_index,
                        float* hdr, void* stream) {
  if (!scene) return set_error(MJPBR_ERR_ARG, "scene is NULL");
  int rc = validate_scene(scene, true);
  if (rc) return rc;
  return newton_images_launch(*scene, cam, geom_shape, geom_shape_rows, ray_scale, color, depth, forward_depth, shape_index,
                              hdr, static_cast<cudaStream_t>(stream));
}

int64_t mjpbr_mesh_bvh_device_scratch_bytes(int32_t nsrc, int32_t nface) { return lbvh_scratch_bytes(nsrc, nface); }

int mjpbr_build_mesh_bvh_device(const float* vert, const int32_t* face, const int32_t* vert_base, const int32_t* vert_num,
                                const int32_t* face_base, const int32_t* node_base, int32_t nsrc, int32_t nface, int32_t leaf_size,
                                float* nodes, float* tris, float* bounds, int32_t* nnode, void* scratch, int64_t scratch_bytes,
                                int32_t* error_word, void* stream) {
  return build_mesh_bvh_device_launch(vert, face, vert_base, vert_num, face_base, node_base, nsrc, nface, leaf_size, nodes, tris,
                                      bounds, nnode, scratch, scratch_bytes, error_word, static_cast<cudaStream_t>(stream));
}

int mjpbr_dfg_lut(float* lut, int32_t size, int32_t nsample, void* stream) {
  return dfg_lut_launch(lut, size, nsample, static_cast<cudaStream_t>(stream));
}

int mjpbr_build_mips(const MjpbrTexture* tex, uint8_t* data, void* stream) {
  return build_mips_launch(tex, data, static_cast<cudaStream_t>(stream));
}

int mjpbr_prefilter_env(const MjpbrTexture* radiance, const uint8_t* data, int32_t levels, int32_t height,
                        int32_t width, int32_t nsample, uint16_t* stack, void* stream) {
  return prefilter_launch(radiance, data, levels, height, width, nsample, stack, static_cast<cudaStream_t>(stream));
}

int mjpbr_env_sh9(const float* image, int32_t height, int32_t width, double* rows, float* sh, void* stream) {
  return env_sh9_launch(image, height, width, rows, sh, static_cast<cudaStream_t>(stream));
}

int mjpbr_env_sampling_tables(const double* image, int32_t height, int32_t width, float* prob, float* marginal,
                              float* conditional, void* stream) {
  return env_tables_launch(image, height, width, prob, marginal, conditional, static_cast<cudaStream_t>(stream));
}

int mjpbr_wait_probe(uint32_t polls, int32_t* error_word, int32_t* roles_done, void* stream) {
  return wait_probe_launch(polls, error_word, roles_done, static_cast<cudaStream_t>(stream));
}

int mjpbr_conv3x3_bf16(const MjpbrConv* conv, void* stream) {
  if (!conv) return set_error(MJPBR_ERR_ARG, "conv is NULL");
  return conv3x3_launch(*conv, static_cast<cudaStream_t>(stream));
}

int64_t mjpbr_kpcn_workspace_bytes(int32_t nimg, int32_t height, int32_t width) { return kpcn_workspace_bytes(nimg, height, width); }

int mjpbr_denoise_learned(const MjpbrScene* scene, const MjpbrKpcnWeights* weights, void* workspace, int64_t workspace_bytes,
                          int32_t chunk, void* stream) {
  if (!scene || !weights) return set_error(MJPBR_ERR_ARG, "scene or weights is NULL");
  int rc = validate_scene(scene, true);
  if (rc) return rc;
  return denoise_learned_launch(*scene, *weights, workspace, workspace_bytes, chunk, static_cast<cudaStream_t>(stream));
}

int mjpbr_conv3x3_wgrad_bf16(const MjpbrConvGrad* grad, void* stream) {
  if (!grad) return set_error(MJPBR_ERR_ARG, "grad is NULL");
  return conv3x3_wgrad_launch(*grad, static_cast<cudaStream_t>(stream));
}

int mjpbr_kpcn_features(const MjpbrScene* scene, int32_t cam, int32_t w0, int32_t nw, uint16_t* x0, void* stream) {
  if (!scene) return set_error(MJPBR_ERR_ARG, "scene is NULL");
  return kpcn_features_launch(*scene, cam, w0, nw, x0, static_cast<cudaStream_t>(stream));
}

int mjpbr_kpcn_target(const MjpbrScene* scene, int32_t cam, const double* hdr_sum, double inv_n, float* target, void* stream) {
  if (!scene) return set_error(MJPBR_ERR_ARG, "scene is NULL");
  return kpcn_target_launch(*scene, cam, hdr_sum, inv_n, target, static_cast<cudaStream_t>(stream));
}

int mjpbr_accumulate_f64(const float* src, double* acc, int64_t n, void* stream) {
  return accumulate_f64_launch(src, acc, n, static_cast<cudaStream_t>(stream));
}

int mjpbr_avgpool2_bf16(const uint16_t* in, uint16_t* out, int32_t nimg, int32_t h, int32_t w, int32_t c, void* stream) {
  return avgpool2_launch(in, out, nimg, h, w, c, static_cast<cudaStream_t>(stream));
}

int mjpbr_upsample2_bf16(const uint16_t* in, uint16_t* out, int32_t nimg, int32_t h, int32_t w, int32_t c, void* stream) {
  return upsample2_launch(in, out, nimg, h, w, c, static_cast<cudaStream_t>(stream));
}

int mjpbr_kpcn_apply(const float* logits, const float* radiance, float* weights, float* out, int32_t nimg, int32_t h, int32_t w,
                     void* stream) {
  return kpcn_apply_launch(logits, radiance, weights, out, nimg, h, w, static_cast<cudaStream_t>(stream));
}

int mjpbr_kpcn_loss(const float* out, const float* target, const float* scale, const float* offset, float* grad, float* sums,
                    int64_t npix, float w_l1, float w_rel, void* stream) {
  return kpcn_loss_launch(out, target, scale, offset, grad, sums, npix, w_l1, w_rel, static_cast<cudaStream_t>(stream));
}

int mjpbr_kpcn_remod(const MjpbrScene* scene, int32_t cam, float* scale, float* offset, void* stream) {
  if (!scene) return set_error(MJPBR_ERR_ARG, "scene is NULL");
  return kpcn_remod_launch(*scene, cam, scale, offset, static_cast<cudaStream_t>(stream));
}

int mjpbr_kpcn_apply_grad(const float* grad, const float* weights, const float* radiance, uint16_t* grad_logits, int32_t nimg,
                          int32_t h, int32_t w, void* stream) {
  return kpcn_apply_grad_launch(grad, weights, radiance, grad_logits, nimg, h, w, static_cast<cudaStream_t>(stream));
}

int mjpbr_split_concat_grad(const float* dcat, const uint16_t* low, float* dskip, uint16_t* dlow, int32_t nimg, int32_t h, int32_t w,
                            int32_t c1, int32_t c2, void* stream) {
  return split_concat_grad_launch(dcat, low, dskip, dlow, nimg, h, w, c1, c2, static_cast<cudaStream_t>(stream));
}

int mjpbr_unpool_add_grad(const float* dskip, const float* dpool, const uint16_t* act, uint16_t* dact, int32_t nimg, int32_t h,
                          int32_t w, int32_t c, void* stream) {
  return unpool_add_grad_launch(dskip, dpool, act, dact, nimg, h, w, c, static_cast<cudaStream_t>(stream));
}

int mjpbr_adam(float* param, float* grad, float* m, float* v, uint16_t* copy, uint16_t* flip, int64_t n, int32_t cout, int32_t cin,
               float lr, float beta1, float beta2, float eps, int32_t step, void* stream) {
  return adam_launch(param, grad, m, v, copy, flip, n, cout, cin, lr, beta1, beta2, eps, step, static_cast<cudaStream_t>(stream));
}

int mjpbr_gemm_bf16(const uint16_t* a, const uint16_t* b, float* d, int32_t m, int32_t n, int32_t k, int32_t* error_word,
                    void* stream) {
  return gemm_bf16_launch(a, b, d, m, n, k, error_word, static_cast<cudaStream_t>(stream));
}

int mjpbr_denoise_atrous(const MjpbrScene* scene, void* stream) {
  if (!scene) return set_error(MJPBR_ERR_ARG, "scene is NULL");
  return denoise_launch(*scene, static_cast<cudaStream_t>(stream));
}

}  // extern "C"
