// Per-camera views of the output buffers: get_rgb / get_depth / get_segmentation (MuJoCo Warp's
// unpackers, third party; called at mujoco_warp_pbr/_src/output.py:34-52) and the per-RGB-pixel
// vec3 images get_hdr / get_albedo / get_normal (mujoco_warp_pbr/_src/output.py:55-152).
// One thread per output pixel; packed RGBA8 is unpacked as channel / 255.
#include "abi_internal.h"
#include "common.cuh"

namespace mjpbr {
namespace {

constexpr int kThreads = 256;

__global__ void rgb_kernel(const uint32_t* __restrict__ rgb, int32_t stride, int32_t adr, int32_t npix, int64_t total,
                           float* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (i >= total) return;
  int64_t w = i / npix, p = i - w * npix;
  uint32_t v = __ldg(rgb + w * stride + adr + p);
  out[i * 3] = (float)(v & 0xFFu) * (1.0f / 255.0f);
  out[i * 3 + 1] = (float)((v >> 8) & 0xFFu) * (1.0f / 255.0f);
  out[i * 3 + 2] = (float)((v >> 16) & 0xFFu) * (1.0f / 255.0f);
}

__global__ void depth_kernel(const float* __restrict__ depth, int32_t stride, int32_t adr, int32_t npix, int64_t total,
                             float inv_scale, float* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (i >= total) return;
  int64_t w = i / npix, p = i - w * npix;
  float d = __ldg(depth + w * stride + adr + p) * inv_scale;
  out[i] = fminf(fmaxf(d, 0.0f), 1.0f);
}

__global__ void seg_kernel(const int32_t* __restrict__ seg, int32_t stride, int32_t adr, int32_t npix, int64_t total,
                           int32_t* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (i >= total) return;
  int64_t w = i / npix, p = i - w * npix;
  int2 v = __ldg(reinterpret_cast<const int2*>(seg) + (w * stride + adr + p));
  reinterpret_cast<int2*>(out)[i] = v;
}

__global__ void vec3_kernel(const float* __restrict__ src, int32_t stride, int32_t adr, int32_t npix, int64_t total,
                            float* __restrict__ out) {
  int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
  if (i >= total) return;
  int64_t w = i / npix, p = i - w * npix;
  const float* q = src + (w * stride + adr + p) * 3;
  out[i * 3] = __ldg(q);
  out[i * 3 + 1] = __ldg(q + 1);
  out[i * 3 + 2] = __ldg(q + 2);
}

}  // namespace

// which: 0 rgb, 1 depth, 2 seg, 3 hdr, 4 albedo, 5 normal.
int outputs_launch(const MjpbrScene& s, int which, int32_t cam, float depth_scale, void* out, int32_t nworld_out,
                   cudaStream_t stream) {
  if (cam < 0 || cam >= s.nrender) return set_error(MJPBR_ERR_ARG, "camera_index must be in [0, %d), got %d", s.nrender, cam);
  if (nworld_out < 0 || nworld_out > s.nworld) {
    return set_error(MJPBR_ERR_ARG, "output has %d worlds, the context %d", nworld_out, s.nworld);
  }
  if (out == nullptr) return set_error(MJPBR_ERR_ARG, "output pointer is NULL");
  const int32_t npix = s.cam_res[cam][0] * s.cam_res[cam][1];
  const int64_t total = (int64_t)nworld_out * npix;
  if (total == 0) return MJPBR_OK;
  const int grid = (int)((total + kThreads - 1) / kThreads);
  switch (which) {
    case 0:
      if (s.rgb_adr[cam] < 0 || !s.rgb_data) return set_error(MJPBR_ERR_ARG, "camera %d renders no RGB", cam);
      rgb_kernel<<<grid, kThreads, 0, stream>>>(s.rgb_data, s.rgb_stride, s.rgb_adr[cam], npix, total,
                                                static_cast<float*>(out));
      break;
    case 1:
      if (s.depth_adr[cam] < 0 || !s.depth_data) return set_error(MJPBR_ERR_ARG, "camera %d renders no depth", cam);
      if (!(depth_scale > 0.0f)) return set_error(MJPBR_ERR_ARG, "depth_scale must be positive, got %g", depth_scale);
      depth_kernel<<<grid, kThreads, 0, stream>>>(s.depth_data, s.depth_stride, s.depth_adr[cam], npix, total,
                                                  1.0f / depth_scale, static_cast<float*>(out));
      break;
    case 2:
      if (s.seg_adr[cam] < 0 || !s.seg_data) return set_error(MJPBR_ERR_ARG, "camera %d renders no segmentation", cam);
      seg_kernel<<<grid, kThreads, 0, stream>>>(s.seg_data, s.seg_stride, s.seg_adr[cam], npix, total,
                                                static_cast<int32_t*>(out));
      break;
    default: {
      const float* src = which == 3 ? s.hdr_data : (which == 4 ? s.guide_albedo : s.guide_normal);
      if (s.rgb_adr[cam] < 0 || !src) return set_error(MJPBR_ERR_ARG, "camera %d has no such image", cam);
      vec3_kernel<<<grid, kThreads, 0, stream>>>(src, s.rgb_stride, s.rgb_adr[cam], npix, total,
                                                 static_cast<float*>(out));
      break;
    }
  }
  return check_launch("outputs");
}

}  // namespace mjpbr
