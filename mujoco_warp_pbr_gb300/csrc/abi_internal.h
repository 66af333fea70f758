// Internal glue between the C entry points (abi.cu) and the kernel launchers of libmjpbr.
#pragma once

#include <cuda_runtime.h>

#include "mjpbr.h"

namespace mjpbr {

// Records a printf-style message for mjpbr_last_error() and returns code.
int set_error(int code, const char* fmt, ...);
// MJPBR_OK, or MJPBR_ERR_CUDA with the launch error of the last kernel.
int check_launch(const char* what);

// Streaming multiprocessors of the current device (looked up once per device, thread-safe).
int device_sm_count();
// Largest dynamic shared memory one CTA may opt in to on the current device (bytes).
size_t device_max_smem();
// Raises kernel `kern`'s dynamic shared-memory limit to at least `bytes` on the current device
// (each kernel and device once per larger size, whatever the size: the kernel's static shared
// memory counts against the default limit too; thread-safe). MJPBR_OK or MJPBR_ERR_CUDA.
int ensure_smem(const void* kern, size_t bytes, const char* what);
// Whether a world block of `floats` floats fits in a CTA's shared memory beside `other` bytes
// (traversal stacks, static arrays); kernels read larger blocks in place from global memory.
bool world_block_staged(int32_t floats, size_t other);

// MJPBR_OK, or MJPBR_ERR_ARG with a message naming the first inconsistent field of the scene.
int validate_scene(const MjpbrScene* s, bool need_outputs);

int refit_launch(const MjpbrScene& s, cudaStream_t stream);
int render_rt_launch(const MjpbrScene& s, uint32_t seed, cudaStream_t stream);
int render_wave_launch(const MjpbrScene& s, uint32_t seed, cudaStream_t stream);
bool wave_supported(const MjpbrScene& s);
bool pt_wave_supported(const MjpbrScene& s);
int64_t wave_scratch_bytes(const MjpbrScene& s, int32_t worlds);
int render_pt_wave_launch(const MjpbrScene& s, uint32_t seed, cudaStream_t stream);
int64_t pt_wave_scratch_bytes(const MjpbrScene& s, int32_t worlds);
int render_pt_launch(const MjpbrScene& s, uint32_t seed, cudaStream_t stream);
int outputs_launch(const MjpbrScene& s, int which, int32_t cam, float depth_scale, void* out, int32_t nworld_out,
                   cudaStream_t stream);
int dfg_lut_launch(float* lut, int32_t size, int32_t nsample, cudaStream_t stream);
int build_mips_launch(const MjpbrTexture* tex, uint8_t* data, cudaStream_t stream);
int prefilter_launch(const MjpbrTexture* radiance, const uint8_t* data, int32_t levels, int32_t height, int32_t width,
                     int32_t nsample, uint16_t* stack, cudaStream_t stream);
int env_sh9_launch(const float* image, int32_t h, int32_t w, double* rows, float* sh, cudaStream_t stream);
int env_tables_launch(const double* image, int32_t h, int32_t w, float* prob, float* marginal, float* conditional,
                      cudaStream_t stream);
int denoise_launch(const MjpbrScene& s, cudaStream_t stream);
int conv3x3_launch(const MjpbrConv& c, cudaStream_t stream);
int64_t kpcn_workspace_bytes(int32_t nimg, int32_t height, int32_t width);
int denoise_learned_launch(const MjpbrScene& s, const MjpbrKpcnWeights& wts, void* workspace, int64_t workspace_bytes, int32_t chunk,
                           cudaStream_t st);
int conv3x3_wgrad_launch(const MjpbrConvGrad& c, cudaStream_t stream);
int wait_probe_launch(uint32_t polls, int32_t* error_word, int32_t* roles_done, cudaStream_t stream);
int kpcn_features_launch(const MjpbrScene& s, int32_t cam, int32_t w0, int32_t nw, uint16_t* x0, cudaStream_t st);
int kpcn_target_launch(const MjpbrScene& s, int32_t cam, const double* hdr_sum, double inv_n, float* target, cudaStream_t st);
int accumulate_f64_launch(const float* src, double* acc, int64_t n, cudaStream_t st);
int avgpool2_launch(const uint16_t* in, uint16_t* out, int32_t nimg, int32_t h, int32_t w, int32_t c, cudaStream_t st);
int upsample2_launch(const uint16_t* in, uint16_t* out, int32_t nimg, int32_t h, int32_t w, int32_t c, cudaStream_t st);
int kpcn_apply_launch(const float* logits, const float* radiance, float* weights, float* out, int32_t nimg, int32_t h, int32_t w,
                      cudaStream_t st);
int kpcn_loss_launch(const float* out, const float* target, const float* scale, const float* offset, float* grad, float* sums,
                     int64_t npix, float w_l1, float w_rel, cudaStream_t st);
int kpcn_remod_launch(const MjpbrScene& s, int32_t cam, float* scale, float* offset, cudaStream_t st);
int kpcn_apply_grad_launch(const float* grad, const float* weights, const float* radiance, uint16_t* grad_logits, int32_t nimg,
                           int32_t h, int32_t w, cudaStream_t st);
int split_concat_grad_launch(const float* dcat, const uint16_t* low, float* dskip, uint16_t* dlow, int32_t nimg, int32_t h, int32_t w,
                             int32_t c1, int32_t c2, cudaStream_t st);
int unpool_add_grad_launch(const float* dskip, const float* dpool, const uint16_t* act, uint16_t* dact, int32_t nimg, int32_t h,
                           int32_t w, int32_t c, cudaStream_t st);
int adam_launch(float* param, float* grad, float* m, float* v, uint16_t* copy, uint16_t* flip, int64_t n, int32_t cout, int32_t cin,
                float lr, float beta1, float beta2, float eps, int32_t step, cudaStream_t st);
int newton_sync_poses_launch(const float* body_q, int32_t nbody, const int32_t* shape_body, const float* shape_transform,
                             int32_t nshape, const int32_t* geom_shape, int32_t geom_shape_rows, const float* geom_offset,
                             const float* camera_transforms, int32_t nworld, int32_t ngeom, int32_t ncam, int32_t cam,
                             float* geom_xpos, float* geom_xmat, float* cam_xpos, float* cam_xmat, int32_t* error_word,
                             cudaStream_t stream);
int newton_images_launch(const MjpbrScene& s, int32_t cam, const int32_t* geom_shape, int32_t geom_shape_rows,
                         const float* ray_scale, uint32_t* color, float* depth, float* forward_depth, uint32_t* shape_index,
                         float* hdr, cudaStream_t stream);
int64_t lbvh_scratch_bytes(int32_t nsrc, int32_t nface);
int build_mesh_bvh_device_launch(const float* vert, const int32_t* face, const int32_t* vert_base, const int32_t* vert_num,
                                 const int32_t* face_base, const int32_t* node_base, int32_t nsrc, int32_t nface,
                                 int32_t leaf_size, float* nodes, float* tris, float* bounds, int32_t* nnode, void* scratch,
                                 int64_t scratch_bytes, int32_t* error_word, cudaStream_t st);
int gemm_bf16_launch(const uint16_t* a, const uint16_t* b, float* d, int32_t m, int32_t n, int32_t k, int32_t* error_word,
                     cudaStream_t stream);

}  // namespace mjpbr
