// The learned denoiser's inference as one C entry point (mjpbr_denoise_learned): per RGB camera
// and chunk of worlds, the network input (mjpbr_kpcn_features), the U-Net forward pass (15 tensor-
// core convolutions, 3 poolings, 3 upsamplings), the 5 x 5 kernel application, and then the a-trous
// filter's finish pass without filtering (remodulation, tone map, outputs). The same launches, in
// the same order, as mujoco_warp_pbr_gb300.kpcn.KPCN.denoise, so that a caller without Python
// gets the same images. Host orchestration only: the kernels are conv.cu's and kpcn.cu's.
#include <algorithm>

#include "abi_internal.h"

namespace mjpbr {
namespace {

struct Layer {
  int32_t level, c_in, c_in2, c_out, relu;
};

constexpr int32_t kFeatures = 16, kLogits = 32;
// e0a e0b e1a e1b e2a e2b e3a e3b d2a d2b d1a d1b d0a d0b head (widths 32 / 48 / 64 / 96)
constexpr Layer kLayers[MJPBR_KPCN_LAYERS] = {
    {0, kFeatures, 0, 32, 1}, {0, 32, 0, 32, 1}, {1, 32, 0, 48, 1}, {1, 48, 0, 48, 1}, {2, 48, 0, 64, 1},
    {2, 64, 0, 64, 1},        {3, 64, 0, 96, 1}, {3, 96, 0, 96, 1}, {2, 64, 96, 64, 1}, {2, 64, 0, 64, 1},
    {1, 48, 64, 48, 1},       {1, 48, 0, 48, 1}, {0, 32, 48, 32, 1}, {0, 32, 0, 32, 1}, {0, 32, 0, kLogits, 0}};

// The workspace of one chunk: activations NHWC (BF16 unless noted), each 256-byte aligned.
struct Workspace {
  uint16_t *x0, *a0, *s0, *u0, *v0, *up0, *p1, *a1, *s1, *u1, *v1, *up1, *p2, *a2, *s2, *u2, *v2, *up2, *p3, *a3, *b3;
  float *radiance, *logits, *out;
};

int64_t layout(int32_t nimg, int32_t h, int32_t w, char* base, Workspace* ws) {
  int64_t off = 0;
  auto take = [&](int32_t level, int64_t channels, int64_t bytes_per_value) {
    char* p = base ? base + off : nullptr;
    off += ((int64_t)nimg * (h >> level) * (w >> level) * channels * bytes_per_value + 255) / 256 * 256;
    return p;
  };
  auto b16 = [&](int32_t level, int32_t c) { return reinterpret_cast<uint16_t*>(take(level, c, 2)); };
  auto f32 = [&](int32_t level, int32_t c) { return reinterpret_cast<float*>(take(level, c, 4)); };
  Workspace t;
  t.x0 = b16(0, kFeatures);
  t.radiance = f32(0, 4);
  t.a0 = b16(0, 32), t.s0 = b16(0, 32), t.u0 = b16(0, 32), t.v0 = b16(0, 32), t.up0 = b16(0, 48);
  t.p1 = b16(1, 32), t.a1 = b16(1, 48), t.s1 = b16(1, 48), t.u1 = b16(1, 48), t.v1 = b16(1, 48), t.up1 = b16(1, 64);
  t.p2 = b16(2, 48), t.a2 = b16(2, 64), t.s2 = b16(2, 64), t.u2 = b16(2, 64), t.v2 = b16(2, 64), t.up2 = b16(2, 96);
  t.p3 = b16(3, 64), t.a3 = b16(3, 96), t.b3 = b16(3, 96);
  t.logits = f32(0, kLogits);
  t.out = f32(0, 4);
  if (ws) *ws = t;
  return off;
}

// Image sizes whose four levels the 128-pixel convolution tiles cover (kpcn.supported).
bool supported(int32_t w, int32_t h) {
  if (w % 8 || h % 8) return false;
  for (int32_t lv = 0; lv < 4; ++lv) {
    const int32_t lw = w >> lv, lh = h >> lv;
    const bool ok = lw >= 128 ? (lw % 128 == 0) : (lw >= 16 && 128 % lw == 0);
    if (!ok || lh % (128 / std::min(lw, 128))) return false;
  }
  return true;
}

int conv(const MjpbrKpcnWeights& wts, int32_t k, const uint16_t* in, const uint16_t* in2, uint16_t* out, float* out_f32, int32_t nimg,
         int32_t h, int32_t w, int32_t* error_word, cudaStream_t st) {
  const Layer& l = kLayers[k];
  MjpbrConv c = {};
  c.in = in;
  c.in2 = in2;
  c.weight = wts.weight[k];
  c.bias = wts.bias[k];
  c.out = out;
  c.out_f32 = out_f32;
  c.error_word = error_word;
  c.nimg = nimg;
  c.height = h >> l.level;
  c.width = w >> l.level;
  c.c_in = l.c_in;
  c.c_in2 = l.c_in2;
  c.c_out = l.c_out;
  c.relu = l.relu;
  c.in2_full = 1;
  return conv3x3_launch(c, st);
}

// The U-Net forward pass of kpcn.KPCN.forward on ws.x0 / ws.radiance into ws.out.
int forward(const MjpbrKpcnWeights& wts, const Workspace& ws, int32_t n, int32_t h, int32_t w, int32_t* err, cudaStream_t st) {
  int rc = 0;
  auto c = [&](int32_t k, const uint16_t* in, uint16_t* out, const uint16_t* in2 = nullptr, float* out_f32 = nullptr) {
    if (!rc) rc = conv(wts, k, in, in2, out, out_f32, n, h, w, err, st);
  };
  auto pool = [&](const uint16_t* in, uint16_t* out, int32_t level, int32_t ch) {
    if (!rc) rc = avgpool2_launch(in, out, n, h >> level, w >> level, ch, st);
  };
  auto up = [&](const uint16_t* in, uint16_t* out, int32_t level, int32_t ch) {
    if (!rc) rc = upsample2_launch(in, out, n, h >> level, w >> level, ch, st);
  };
  c(0, ws.x0, ws.a0);
  c(1, ws.a0, ws.s0);
  pool(ws.s0, ws.p1, 0, 32);
  c(2, ws.p1, ws.a1);
  c(3, ws.a1, ws.s1);
  pool(ws.s1, ws.p2, 1, 48);
  c(4, ws.p2, ws.a2);
  c(5, ws.a2, ws.s2);
  pool(ws.s2, ws.p3, 2, 64);
  c(6, ws.p3, ws.a3);
  c(7, ws.a3, ws.b3);
  up(ws.b3, ws.up2, 3, 96);
  c(8, ws.s2, ws.u2, ws.up2);
  c(9, ws.u2, ws.v2);
  up(ws.v2, ws.up1, 2, 64);
  c(10, ws.s1, ws.u1, ws.up1);
  c(11, ws.u1, ws.v1);
  up(ws.v1, ws.up0, 1, 48);
  c(12, ws.s0, ws.u0, ws.up0);
  c(13, ws.u0, ws.v0);
  c(14, ws.v0, nullptr, nullptr, ws.logits);
  if (!rc) rc = kpcn_apply_launch(ws.logits, ws.radiance, nullptr, ws.out, n, h, w, st);
  return rc;
}

}  // namespace

int64_t kpcn_workspace_bytes(int32_t nimg, int32_t height, int32_t width) {
  if (nimg < 1 || !supported(width, height)) return -1;
  return layout(nimg, height, width, nullptr, nullptr);
}

int denoise_learned_launch(const MjpbrScene& s, const MjpbrKpcnWeights& wts, void* workspace, int64_t workspace_bytes, int32_t chunk,
                           cudaStream_t st) {
  if (s.settings.tier != MJPBR_TIER_PATH || !s.settings.denoise || !s.denoise_buffers[0] || !s.denoise_buffers[1] || !s.aov_guide) {
    return set_error(MJPBR_ERR_ARG, "denoise_learned: the scene is not a denoising path-traced render");
  }
  if (chunk < 1 || !workspace) return set_error(MJPBR_ERR_ARG, "denoise_learned: chunk must be >= 1 and workspace set");
  for (int32_t k = 0; k < MJPBR_KPCN_LAYERS; ++k) {
    if (!wts.weight[k] || !wts.bias[k]) return set_error(MJPBR_ERR_ARG, "denoise_learned: layer %d has no weights", k);
  }
  for (int32_t cam = 0; cam < s.nrender; ++cam) {
    if (!s.render_rgb[cam]) continue;
    const int32_t w = s.cam_res[cam][0], h = s.cam_res[cam][1];
    const int32_t nw_max = std::min(chunk, s.nworld);
    const int64_t need = kpcn_workspace_bytes(nw_max, h, w);
    if (need < 0) return set_error(MJPBR_ERR_ARG, "denoise_learned: camera %d of %dx%d is not tiled by the network (use the a-trous filter)", cam, w, h);
    if (need > workspace_bytes) return set_error(MJPBR_ERR_ARG, "denoise_learned: workspace of %lld bytes, %lld needed", (long long)workspace_bytes, (long long)need);
    const int64_t npix = (int64_t)w * h;
    for (int32_t w0 = 0; w0 < s.nworld; w0 += chunk) {
      const int32_t nw = std::min(chunk, s.nworld - w0);
      Workspace ws;
      layout(nw, h, w, static_cast<char*>(workspace), &ws);
      int rc = kpcn_features_launch(s, cam, w0, nw, ws.x0, st);
      if (rc) return rc;
      const size_t pitch = (size_t)s.rgb_stride * 16, bytes = (size_t)npix * 16;
      const float* src = s.denoise_buffers[0] + ((int64_t)w0 * s.rgb_stride + s.rgb_adr[cam]) * 4;
      cudaError_t e = cudaMemcpy2DAsync(ws.radiance, bytes, src, pitch, bytes, nw, cudaMemcpyDeviceToDevice, st);
      if (e != cudaSuccess) return set_error(MJPBR_ERR_CUDA, "denoise_learned: radiance copy: %s", cudaGetErrorString(e));
      rc = forward(wts, ws, nw, h, w, s.error_word, st);
      if (rc) return rc;
      float* dst = s.denoise_buffers[1] + ((int64_t)w0 * s.rgb_stride + s.rgb_adr[cam]) * 4;
      e = cudaMemcpy2DAsync(dst, pitch, ws.out, bytes, bytes, nw, cudaMemcpyDeviceToDevice, st);
      if (e != cudaSuccess) return set_error(MJPBR_ERR_CUDA, "denoise_learned: output copy: %s", cudaGetErrorString(e));
    }
  }
  // the a-trous filter's finish pass without filtering, on the network's radiance
  MjpbrScene fs = s;
  fs.denoise_buffers[0] = s.denoise_buffers[1];
  fs.denoise_iterations = 0;
  return denoise_launch(fs, st);
}

}  // namespace mjpbr
