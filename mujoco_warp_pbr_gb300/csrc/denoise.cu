// Edge-avoiding a-trous denoiser of the path-traced tier (Dammertz et al. 2010;
// mujoco_warp_pbr/_src/denoise.py:101-248): `denoise_iterations` passes of a 5 x 5 B3-spline filter
// with holes (steps 1, 2, 4, ...) over the demodulated radiance, weighted by normal, depth, albedo
// and luminance differences, the luminance tolerance following the per-pixel noise estimate
// (sample variance, 3 x 3 Gaussian-smoothed, propagated through the passes as in SVGF).
//
// GB300 layout: the path tracer already wrote the demodulated radiance + variance (one float4 per
// pixel) into denoise_buffers[0] and the filter's guide as one 16-byte record per pixel (normal and
// albedo as half floats, depth), so a neighbour costs two 128-bit loads; 16 x 16-pixel blocks keep
// the 5 x 5 footprint's rows in L1. The last pass remodulates, tone maps and writes the display
// RGB (and the HDR) directly: no separate demodulate / finish passes over the image.
#include <algorithm>

#include "abi_internal.h"
#include "denoise_common.cuh"
#include "shading.cuh"

namespace mjpbr {
namespace {

constexpr int kTile = 16;

struct Images {
  int32_t ncam;
  int32_t width[MJPBR_MAX_RENDER], height[MJPBR_MAX_RENDER], adr[MJPBR_MAX_RENDER];
  int32_t tiles_x[MJPBR_MAX_RENDER];
  int32_t tile_base[MJPBR_MAX_RENDER + 1];
};

struct Filter {
  int32_t step;  // 0: no filtering (finish only)
  float sigma_color, sigma_normal, sigma_depth, sigma_albedo;
};

MJ_DEV float b3(int i) { return i == 2 ? 0.375f : ((i == 1 || i == 3) ? 0.25f : 0.0625f); }

template <bool kFinish>
__global__ void __launch_bounds__(kTile* kTile) atrous_kernel(const __grid_constant__ MjpbrScene s,
                                                              const __grid_constant__ Images im, Filter f,
                                                              const float4* __restrict__ src, float4* __restrict__ dst) {
  const int32_t t = blockIdx.x;
  int32_t cam = 0;
  while (cam + 1 < im.ncam && t >= im.tile_base[cam + 1]) ++cam;
  const int32_t lt = t - im.tile_base[cam];
  const int32_t W = im.width[cam], H = im.height[cam];
  const int32_t px = (lt % im.tiles_x[cam]) * kTile + (int32_t)(threadIdx.x % kTile);
  const int32_t py = (lt / im.tiles_x[cam]) * kTile + (int32_t)(threadIdx.x / kTile);
  if (px >= W || py >= H) return;
  for (int32_t w = blockIdx.y; w < s.nworld; w += gridDim.y) {
    const int64_t base = (int64_t)w * s.rgb_stride + im.adr[cam];
    const uint4* guide = reinterpret_cast<const uint4*>(s.aov_guide) + base;
    const float4* in = src + base;
    const int32_t idx = py * W + px;
    const Guide g0 = unpack_guide(__ldg(guide + idx));
    float4 out = __ldg(in + idx);
    if (f.step > 0 && length_sq(g0.normal) != 0.0f) {
      // 3 x 3 Gaussian of the variance: the per-pixel estimate from few samples is itself noisy
      float variance = 0.0f, variance_weight = 0.0f;
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const int32_t y = min(max(py + j - 1, 0), H - 1);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const int32_t x = min(max(px + i - 1, 0), W - 1);
          const float g = (i == 1 ? 0.5f : 0.25f) * (j == 1 ? 0.5f : 0.25f);
          variance += g * __ldg(in + y * W + x).w;
          variance_weight += g;
        }
      }
      const float inv_sigma_l = 1.0f / (f.sigma_color * sqrtf(fmaxf(variance / variance_weight, 0.0f)) + 1.0e-6f);
      const float l0 = luminance(V3{out.x, out.y, out.z});
      const float inv_sigma_a = 1.0f / f.sigma_albedo;
      // depth differences are relative and grow with the filter footprint
      const float inv_sigma_z = 1.0f / fmaxf(f.sigma_depth * g0.depth * (float)f.step, 1.0e-6f);
      V3 total = v3(0.0f);
      float total_variance = 0.0f, weight_sum = 0.0f;
#pragma unroll
      for (int j = 0; j < 5; ++j) {
        const int32_t y = py + (j - 2) * f.step;
        if (y < 0 || y >= H) continue;
#pragma unroll
        for (int i = 0; i < 5; ++i) {
          const int32_t x = px + (i - 2) * f.step;
          if (x < 0 || x >= W) continue;
          const int32_t q = y * W + x;
          const float4 sq = __ldg(in + q);
          const Guide gq = unpack_guide(__ldg(guide + q));
          const V3 c{sq.x, sq.y, sq.z};
          // background neighbours (zero normal) get zero weight
          const float wn = fast_pow(fmaxf(dot(g0.normal, gq.normal), 0.0f), f.sigma_normal);
          const float distance = fabsf(gq.depth - g0.depth) * inv_sigma_z + fabsf(luminance(c) - l0) * inv_sigma_l +
                                 length(gq.albedo - g0.albedo) * inv_sigma_a;
          const float weight = b3(i) * b3(j) * wn * __expf(-distance);
          total += c * weight;
          total_variance += weight * weight * sq.w;
          weight_sum += weight;
        }
      }
      // the centre pixel always contributes, so weight_sum > 0
      const V3 c = total / weight_sum;
      out = make_float4(c.x, c.y, c.z, total_variance / (weight_sum * weight_sum));
    }
    if (kFinish) {
      const int64_t adr = base + idx;
      const float* e = s.aov_emission + adr * 3;
      const V3 exposed = remodulate(out, V3{e[0], e[1], e[2]}, g0.albedo);
      if (s.settings.render_hdr) {
        const V3 hdr = exposed / bf(s.exposure, w, 1, 0);
        s.hdr_data[adr * 3] = hdr.x;
        s.hdr_data[adr * 3 + 1] = hdr.y;
        s.hdr_data[adr * 3 + 2] = hdr.z;
      }
      s.rgb_data[adr] = encode_display(display_transform(exposed, s.settings.tone_mapper));
    } else {
      dst[base + idx] = out;
    }
  }
}

}  // namespace

int denoise_launch(const MjpbrScene& s, cudaStream_t stream) {
  if (!s.aov_guide || !s.aov_emission || !s.denoise_buffers[0] || !s.denoise_buffers[1] || !s.rgb_data) {
    return set_error(MJPBR_ERR_ARG, "the denoiser needs aov_guide, aov_emission, denoise_buffers and rgb_data");
  }
  if (s.settings.render_hdr && !s.hdr_data) return set_error(MJPBR_ERR_ARG, "render_hdr needs hdr_data");
  if (s.denoise_iterations < 0 || s.denoise_iterations > 16) {
    return set_error(MJPBR_ERR_ARG, "denoise_iterations %d outside [0, 16]", s.denoise_iterations);
  }
  Images im{};
  im.ncam = 0;
  im.tile_base[0] = 0;
  for (int32_t c = 0; c < s.nrender; ++c) {
    if (!s.render_rgb[c] || s.rgb_adr[c] < 0) continue;
    const int32_t k = im.ncam++;
    im.width[k] = s.cam_res[c][0];
    im.height[k] = s.cam_res[c][1];
    im.adr[k] = s.rgb_adr[c];
    im.tiles_x[k] = (im.width[k] + kTile - 1) / kTile;
    im.tile_base[k + 1] = im.tile_base[k] + im.tiles_x[k] * ((im.height[k] + kTile - 1) / kTile);
  }
  const int32_t tiles = im.tile_base[im.ncam];
  if (tiles == 0 || s.nworld == 0) return MJPBR_OK;
  Filter f{0, s.settings.denoise_sigma_color, s.settings.denoise_sigma_normal, s.settings.denoise_sigma_depth,
           s.settings.denoise_sigma_albedo};
  const dim3 grid(tiles, std::min(s.nworld, 65535));
  float4* buf[2] = {reinterpret_cast<float4*>(s.denoise_buffers[0]), reinterpret_cast<float4*>(s.denoise_buffers[1])};
  const int32_t passes = s.denoise_iterations;
  for (int32_t i = 0; i < passes - 1; ++i) {
    f.step = 1 << i;
    atrous_kernel<false><<<grid, kTile * kTile, 0, stream>>>(s, im, f, buf[i & 1], buf[(i + 1) & 1]);
    if (int rc = check_launch("atrous_kernel")) return rc;
  }
  f.step = passes > 0 ? 1 << (passes - 1) : 0;
  atrous_kernel<true><<<grid, kTile * kTile, 0, stream>>>(s, im, f, buf[passes > 0 ? (passes - 1) & 1 : 0], nullptr);
  return check_launch("atrous_finish_kernel");
}

}  // namespace mjpbr
