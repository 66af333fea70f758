// Pixel-wise pieces of the learned kernel-predicting denoiser (KPCN): the network input built from
// the path tracer's denoiser buffers, 2 x 2 average pooling, the predicted per-pixel 5 x 5 kernels
// (softmax of 25 logits) applied to the noisy demodulated radiance, the training loss (L1 +
// relative MSE) and the backward passes of all of these, the routing of gradients through the
// U-Net's skip concatenations and poolings, FP64 accumulation of converged ground truth, and the
// Adam update that also refreshes the BF16 (and flipped, transposed for the input-gradient pass)
// weight copies. The 3 x 3 convolutions themselves run on the tensor cores (conv.cu).
//
// Layouts: NHWC with the image index n = world (one camera per network pass), BF16 activations,
// FP32 logits / kernels / radiance / gradients where noted.
#include <cuda_bf16.h>

#include <algorithm>

#include "abi_internal.h"
#include "denoise_common.cuh"

namespace mjpbr {
namespace {

constexpr int kKernel = 5;                    // predicted kernel edge
constexpr int kTaps = kKernel * kKernel;      // 25 weights per pixel
constexpr int kLogits = 32;                   // logit channels (25 used)
constexpr int kFeatures = 16;                 // network input channels (11 used)

__device__ __forceinline__ uint16_t bf16_bits(float v) { return __bfloat16_as_ushort(__float2bfloat16_rn(v)); }
__device__ __forceinline__ float bf16_value(uint16_t b) { return __uint_as_float((uint32_t)b << 16); }

struct CamImage {
  int32_t width, height, adr;
};

// Network input of camera image (world w): log(1 + demodulated radiance), first-hit albedo,
// normal, log(1 + depth), log(1 + standard deviation of the mean's luminance), zeros.
__global__ void features_kernel(const __grid_constant__ MjpbrScene s, CamImage c, int32_t w0, int32_t nw, uint16_t* __restrict__ x0) {
  const int64_t npix = (int64_t)c.width * c.height;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npix * nw) return;
  const int64_t w = w0 + i / npix, pid = i % npix;
  const int64_t adr = w * s.rgb_stride + c.adr + pid;
  const float4 r = reinterpret_cast<const float4*>(s.denoise_buffers[0])[adr];
  const Guide g = unpack_guide(reinterpret_cast<const uint4*>(s.aov_guide)[adr]);
  float f[kFeatures] = {log1pf(fmaxf(r.x, 0.0f)), log1pf(fmaxf(r.y, 0.0f)), log1pf(fmaxf(r.z, 0.0f)), g.albedo.x, g.albedo.y,
                        g.albedo.z, g.normal.x, g.normal.y, g.normal.z, log1pf(fmaxf(g.depth, 0.0f)), log1pf(sqrtf(fmaxf(r.w, 0.0f))),
                        0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
  uint32_t o[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) o[k] = (uint32_t)bf16_bits(f[2 * k]) | ((uint32_t)bf16_bits(f[2 * k + 1]) << 16);
  uint4* dst = reinterpret_cast<uint4*>(x0 + i * kFeatures);
  dst[0] = make_uint4(o[0], o[1], o[2], o[3]);
  dst[1] = make_uint4(o[4], o[5], o[6], o[7]);
}

// The demodulated target of camera image (world w) from the FP64 sum of n converged HDR frames,
// with the noisy frame's albedo and emission (the same remodulation the output goes through).
__global__ void target_kernel(const __grid_constant__ MjpbrScene s, CamImage c, const double* __restrict__ hdr_sum, double inv_n,
                              float4* __restrict__ target) {
  const int64_t npix = (int64_t)c.width * c.height;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npix * s.nworld) return;
  const int64_t w = i / npix, pid = i - w * npix;
  const int64_t adr = w * s.rgb_stride + c.adr + pid;
  const V3 hdr{(float)(hdr_sum[adr * 3] * inv_n), (float)(hdr_sum[adr * 3 + 1] * inv_n), (float)(hdr_sum[adr * 3 + 2] * inv_n)};
  const Guide g = unpack_guide(reinterpret_cast<const uint4*>(s.aov_guide)[adr]);
  const V3 em{s.aov_emission[adr * 3], s.aov_emission[adr * 3 + 1], s.aov_emission[adr * 3 + 2]};
  const float exposure = bf(s.exposure, (int32_t)w, 1, 0);
  target[i] = demodulate(hdr, exposure, em, g.albedo, 0.0f);
}

__global__ void accumulate_f64_kernel(const float* __restrict__ src, double* __restrict__ acc, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) acc[i] += (double)src[i];
}

__global__ void avgpool2_scalar_kernel(const uint16_t* __restrict__ in, uint16_t* __restrict__ out, int32_t nimg, int32_t h, int32_t w,
                                int32_t ch) {
  const int32_t h2 = h / 2, w2 = w / 2;
  const int64_t total = (int64_t)nimg * h2 * w2 * ch;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int32_t c = (int32_t)(i % ch);
  const int64_t pix = i / ch;
  const int32_t x = (int32_t)(pix % w2), y = (int32_t)((pix / w2) % h2);
  const int64_t n = pix / ((int64_t)w2 * h2);
  const int64_t base = ((n * h + 2 * y) * w + 2 * x) * ch + c;
  const float v = bf16_value(in[base]) + bf16_value(in[base + ch]) + bf16_value(in[base + (int64_t)w * ch]) +
                  bf16_value(in[base + (int64_t)w * ch + ch]);
  out[i] = bf16_bits(0.25f * v);
}

// One thread per 8 channels (16 bytes) of an output pixel: the same sums as the scalar kernel
// ((0,0) + (0,1) + (1,0) + (1,1) in FP32, times 1/4, rounded to BF16), 16-byte loads and stores.
__global__ void avgpool2_kernel(const uint4* __restrict__ in, uint4* __restrict__ out, int32_t nimg, int32_t h, int32_t w, int32_t c8) {
  const int32_t h2 = h / 2, w2 = w / 2;
  const int64_t total = (int64_t)nimg * h2 * w2 * c8;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int32_t g = (int32_t)(i % c8);
  const int64_t pix = i / c8;
  const int32_t x = (int32_t)(pix % w2), y = (int32_t)((pix / w2) % h2);
  const int64_t n = pix / ((int64_t)w2 * h2);
  const int64_t base = ((n * h + 2 * y) * w + 2 * x) * c8 + g;
  const uint4 a = __ldg(in + base), b = __ldg(in + base + c8), c = __ldg(in + base + (int64_t)w * c8), d = __ldg(in + base + (int64_t)w * c8 + c8);
  const uint32_t av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w}, cv[4] = {c.x, c.y, c.z, c.w}, dv[4] = {d.x, d.y, d.z, d.w};
  uint32_t o[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const float lo = __uint_as_float(av[k] << 16) + __uint_as_float(bv[k] << 16) + __uint_as_float(cv[k] << 16) + __uint_as_float(dv[k] << 16);
    const float hi = __uint_as_float(av[k] & 0xFFFF0000u) + __uint_as_float(bv[k] & 0xFFFF0000u) + __uint_as_float(cv[k] & 0xFFFF0000u) +
                     __uint_as_float(dv[k] & 0xFFFF0000u);
    o[k] = (uint32_t)bf16_bits(0.25f * lo) | ((uint32_t)bf16_bits(0.25f * hi) << 16);
  }
  out[i] = make_uint4(o[0], o[1], o[2], o[3]);
}

// One thread per 16-byte group of 8 channels of an output pixel.
__global__ void upsample2_kernel(const uint4* __restrict__ in, uint4* __restrict__ out, int32_t nimg, int32_t h, int32_t w, int32_t c8) {
  const int64_t total = (int64_t)nimg * 4 * h * w * c8;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int32_t g = (int32_t)(i % c8);
  const int64_t pix = i / c8;
  const int32_t x = (int32_t)(pix % (2 * w)), y = (int32_t)((pix / (2 * w)) % (2 * h));
  const int64_t n = pix / ((int64_t)4 * w * h);
  out[i] = __ldg(in + ((n * h + (y >> 1)) * w + (x >> 1)) * c8 + g);
}

__device__ __forceinline__ int32_t clampi(int32_t v, int32_t lo, int32_t hi) { return min(max(v, lo), hi); }

// Softmax of the 25 logits and the kernel applied to the radiance (float4 records, xyz used),
// borders clamped. Writes the weights (for the backward pass) and the filtered radiance (float4,
// w = 0, the demodulated format the a-trous finish pass remodulates).
__global__ void apply_kernel(const float* __restrict__ logits, const float4* __restrict__ radiance, float* __restrict__ weights,
                             float4* __restrict__ out, int32_t nimg, int32_t h, int32_t w) {
  const int64_t total = (int64_t)nimg * h * w;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int32_t x = (int32_t)(i % w), y = (int32_t)((i / w) % h);
  const int64_t base = i - ((int64_t)y * w + x);
  // the pixel's 32 logits as 16-byte loads (25 used)
  const float4* lg4 = reinterpret_cast<const float4*>(logits + i * kLogits);
  float e[28];
#pragma unroll
  for (int q = 0; q < 7; ++q) {
    const float4 v = __ldg(lg4 + q);
    e[4 * q] = v.x;
    e[4 * q + 1] = v.y;
    e[4 * q + 2] = v.z;
    e[4 * q + 3] = v.w;
  }
  float mx = e[0];
#pragma unroll
  for (int k = 1; k < kTaps; ++k) mx = fmaxf(mx, e[k]);
  float sum = 0.0f;
#pragma unroll
  for (int k = 0; k < kTaps; ++k) {
    e[k] = __expf(e[k] - mx);
    sum += e[k];
  }
  const float inv = 1.0f / sum;
  float3 acc = make_float3(0.0f, 0.0f, 0.0f);
#pragma unroll
  for (int dy = 0; dy < kKernel; ++dy) {
    const int64_t row = base + (int64_t)clampi(y + dy - 2, 0, h - 1) * w;
#pragma unroll
    for (int dx = 0; dx < kKernel; ++dx) {
      const int k = dy * kKernel + dx;
      const float wk = e[k] * inv;
      if (weights) weights[i * kTaps + k] = wk;
      const float4 r = __ldg(radiance + row + clampi(x + dx - 2, 0, w - 1));
      acc.x += wk * r.x;
      acc.y += wk * r.y;
      acc.z += wk * r.z;
    }
  }
  out[i] = make_float4(acc.x, acc.y, acc.z, 0.0f);
}

// Loss = w_l1 * mean(|o - t| / sqrt(t^2 + 0.01)) + w_rel * mean((o - t)^2 / (t^2 + 0.01)) over
// pixels and channels (t clamped at 0): relative L1 and relative MSE, both independent of the
// image's scale; its gradient with respect to the output; the two sums into sums[0..1]. With
// scale / offset (float4 records, may be NULL) both are first mapped to HDR, x -> offset + x *
// scale (the remodulation by albedo and emission over exposure), so that the loss is the relative
// error of the final image.
__global__ void loss_kernel(const float4* __restrict__ out, const float4* __restrict__ target, const float4* __restrict__ scale,
                            const float4* __restrict__ offset, float4* __restrict__ grad, float* __restrict__ sums, int64_t npix,
                            float w_l1, float w_rel) {
  __shared__ float part[2][256];
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  float l1 = 0.0f, rel = 0.0f;
  if (i < npix) {
    const float4 o = out[i], t = target[i];
    const float4 sc = scale ? scale[i] : make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    const float4 of = offset ? offset[i] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const float inv = 1.0f / (3.0f * (float)npix);
    const float ov[3] = {o.x, o.y, o.z}, tv[3] = {fmaxf(t.x, 0.0f), fmaxf(t.y, 0.0f), fmaxf(t.z, 0.0f)};
    const float sv[3] = {sc.x, sc.y, sc.z}, fv[3] = {of.x, of.y, of.z};
    float g[3];
    for (int c = 0; c < 3; ++c) {
      const float oh = fv[c] + ov[c] * sv[c], th = fv[c] + tv[c] * sv[c];
      const float d = oh - th;
      const float den = th * th + 0.01f;
      const float rden = rsqrtf(den);
      l1 += fabsf(d) * rden;
      rel += d * d / den;
      g[c] = (w_l1 * (d > 0.0f ? 1.0f : (d < 0.0f ? -1.0f : 0.0f)) * rden + w_rel * 2.0f * d / den) * inv * sv[c];
    }
    grad[i] = make_float4(g[0], g[1], g[2], 0.0f);
  }
  part[0][threadIdx.x] = l1;
  part[1][threadIdx.x] = rel;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) {
      part[0][threadIdx.x] += part[0][threadIdx.x + s];
      part[1][threadIdx.x] += part[1][threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    atomicAdd(sums, part[0][0]);
    atomicAdd(sums + 1, part[1][0]);
  }
}

// The HDR mapping of the demodulated radiance of camera image (world w): scale = max(albedo,
// 0.01) / exposure, offset = exposed emission / exposure (float4 records, w = 0).
__global__ void remod_kernel(const __grid_constant__ MjpbrScene s, CamImage c, float4* __restrict__ scale, float4* __restrict__ offset) {
  const int64_t npix = (int64_t)c.width * c.height;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npix * s.nworld) return;
  const int64_t w = i / npix, pid = i - w * npix;
  const int64_t adr = w * s.rgb_stride + c.adr + pid;
  const Guide g = unpack_guide(reinterpret_cast<const uint4*>(s.aov_guide)[adr]);
  const float inv_exposure = 1.0f / bf(s.exposure, (int32_t)w, 1, 0);
  scale[i] = make_float4(fmaxf(g.albedo.x, kMinAlbedo) * inv_exposure, fmaxf(g.albedo.y, kMinAlbedo) * inv_exposure,
                         fmaxf(g.albedo.z, kMinAlbedo) * inv_exposure, 0.0f);
  offset[i] = make_float4(s.aov_emission[adr * 3] * inv_exposure, s.aov_emission[adr * 3 + 1] * inv_exposure,
                          s.aov_emission[adr * 3 + 2] * inv_exposure, 0.0f);
}

// Backward of apply_kernel: d logit_k = w_k (g_k - sum_j w_j g_j), g_k = grad . radiance(tap k);
// BF16 logit gradients (channels 25-31 zero) for the head's weight and input gradients.
__global__ void apply_grad_kernel(const float4* __restrict__ grad, const float* __restrict__ weights,
                                  const float4* __restrict__ radiance, uint16_t* __restrict__ grad_logits, int32_t nimg, int32_t h,
                                  int32_t w) {
  const int64_t total = (int64_t)nimg * h * w;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int32_t x = (int32_t)(i % w), y = (int32_t)((i / w) % h);
  const int64_t base = i - ((int64_t)y * w + x);
  const float4 go = grad[i];
  float gk[kTaps], dot = 0.0f;
  for (int k = 0; k < kTaps; ++k) {
    const int32_t yy = clampi(y + k / kKernel - 2, 0, h - 1), xx = clampi(x + k % kKernel - 2, 0, w - 1);
    const float4 r = radiance[base + (int64_t)yy * w + xx];
    gk[k] = go.x * r.x + go.y * r.y + go.z * r.z;
    dot += weights[i * kTaps + k] * gk[k];
  }
  uint32_t o[kLogits / 2];
  for (int k = 0; k < kLogits / 2; ++k) {
    float a = 0.0f, b = 0.0f;
    if (2 * k < kTaps) a = weights[i * kTaps + 2 * k] * (gk[2 * k] - dot);
    if (2 * k + 1 < kTaps) b = weights[i * kTaps + 2 * k + 1] * (gk[2 * k + 1] - dot);
    o[k] = (uint32_t)bf16_bits(a) | ((uint32_t)bf16_bits(b) << 16);
  }
  uint4* dst = reinterpret_cast<uint4*>(grad_logits + i * kLogits);
  for (int k = 0; k < 4; ++k) dst[k] = make_uint4(o[4 * k], o[4 * k + 1], o[4 * k + 2], o[4 * k + 3]);
}

// Gradient of a skip concatenation [skip (c1), upsampled low (c2)]: the skip part is copied to
// dskip (FP32), the upsampled part summed over each 2 x 2 block and masked by the ReLU of the
// low-resolution activation into dlow (BF16).
__global__ void split_concat_grad_kernel(const float* __restrict__ dcat, const uint16_t* __restrict__ low, float* __restrict__ dskip,
                                         uint16_t* __restrict__ dlow, int32_t nimg, int32_t h, int32_t w, int32_t c1, int32_t c2) {
  const int32_t ct = c1 + c2;
  const int32_t h2 = h / 2, w2 = w / 2;
  const int64_t nskip = (int64_t)nimg * h * w * c1;
  const int64_t nlow = (int64_t)nimg * h2 * w2 * c2;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nskip) {
    const int64_t pix = i / c1;
    dskip[i] = dcat[pix * ct + (i - pix * c1)];
  }
  if (i < nlow) {
    const int32_t c = (int32_t)(i % c2);
    const int64_t pix = i / c2;
    const int32_t x = (int32_t)(pix % w2), y = (int32_t)((pix / w2) % h2);
    const int64_t n = pix / ((int64_t)w2 * h2);
    const int64_t b = ((n * h + 2 * y) * w + 2 * x) * ct + c1 + c;
    const float v = dcat[b] + dcat[b + ct] + dcat[b + (int64_t)w * ct] + dcat[b + (int64_t)w * ct + ct];
    dlow[i] = (low[i] & 0x8000u) || !(low[i] & 0x7FFFu) ? 0 : bf16_bits(v);
  }
}

__device__ __forceinline__ uint32_t relu_masked_bf16x2(float a, float b, uint32_t act2) {
  // a BF16 activation is > 0 when its sign bit is clear and it is not zero
  const uint32_t lo = (act2 & 0x8000u) || !(act2 & 0x7FFFu) ? 0u : (uint32_t)bf16_bits(a);
  const uint32_t hi = (act2 & 0x80000000u) || !(act2 & 0x7FFF0000u) ? 0u : (uint32_t)bf16_bits(b);
  return lo | (hi << 16);
}

// 4 channels per thread (the 16-byte form of split_concat_grad_kernel; same sums and masks).
__global__ void split_concat_grad4_kernel(const float4* __restrict__ dcat, const uint2* __restrict__ low, float4* __restrict__ dskip,
                                          uint2* __restrict__ dlow, int32_t nimg, int32_t h, int32_t w, int32_t c1q, int32_t c2q) {
  const int32_t ctq = c1q + c2q;
  const int32_t h2 = h / 2, w2 = w / 2;
  const int64_t nskip = (int64_t)nimg * h * w * c1q;
  const int64_t nlow = (int64_t)nimg * h2 * w2 * c2q;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < nskip) {
    const int64_t pix = i / c1q;
    dskip[i] = __ldg(dcat + pix * ctq + (i - pix * c1q));
  }
  if (i < nlow) {
    const int32_t q = (int32_t)(i % c2q);
    const int64_t pix = i / c2q;
    const int32_t x = (int32_t)(pix % w2), y = (int32_t)((pix / w2) % h2);
    const int64_t n = pix / ((int64_t)w2 * h2);
    const int64_t b = ((n * h + 2 * y) * w + 2 * x) * ctq + c1q + q;
    const float4 a = __ldg(dcat + b), bb = __ldg(dcat + b + ctq), c = __ldg(dcat + b + (int64_t)w * ctq), d = __ldg(dcat + b + (int64_t)w * ctq + ctq);
    const uint2 lw = __ldg(low + i);
    dlow[i] = make_uint2(relu_masked_bf16x2(a.x + bb.x + c.x + d.x, a.y + bb.y + c.y + d.y, lw.x),
                         relu_masked_bf16x2(a.z + bb.z + c.z + d.z, a.w + bb.w + c.w + d.w, lw.y));
  }
}

// 4 channels per thread (the 16-byte form of unpool_add_grad_kernel; same sums and masks).
__global__ void unpool_add_grad4_kernel(const float4* __restrict__ dskip, const float4* __restrict__ dpool, const uint2* __restrict__ act,
                                        uint2* __restrict__ dact, int32_t nimg, int32_t h, int32_t w, int32_t cq) {
  const int64_t total = (int64_t)nimg * h * w * cq;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int32_t q = (int32_t)(i % cq);
  const int64_t pix = i / cq;
  const int32_t x = (int32_t)(pix % w), y = (int32_t)((pix / w) % h);
  const int64_t n = pix / ((int64_t)w * h);
  const float4 dp = __ldg(dpool + ((n * (h / 2) + y / 2) * (w / 2) + x / 2) * cq + q);
  float4 v = make_float4(0.25f * dp.x, 0.25f * dp.y, 0.25f * dp.z, 0.25f * dp.w);
  if (dskip) {
    const float4 ds = __ldg(dskip + i);
    v = make_float4(v.x + ds.x, v.y + ds.y, v.z + ds.z, v.w + ds.w);
  }
  const uint2 ac = __ldg(act + i);
  dact[i] = make_uint2(relu_masked_bf16x2(v.x, v.y, ac.x), relu_masked_bf16x2(v.z, v.w, ac.y));
}

// Gradient of a skip activation s = (dskip + the 2 x 2 average-pool gradient of dpool) masked by
// the ReLU of s, as BF16 (dskip may be NULL at the bottom level).
__global__ void unpool_add_grad_kernel(const float* __restrict__ dskip, const float* __restrict__ dpool, const uint16_t* __restrict__ act,
                                       uint16_t* __restrict__ dact, int32_t nimg, int32_t h, int32_t w, int32_t c) {
  const int64_t total = (int64_t)nimg * h * w * c;
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= total) return;
  const int32_t ch = (int32_t)(i % c);
  const int64_t pix = i / c;
  const int32_t x = (int32_t)(pix % w), y = (int32_t)((pix / w) % h);
  const int64_t n = pix / ((int64_t)w * h);
  float v = 0.25f * dpool[((n * (h / 2) + y / 2) * (w / 2) + x / 2) * c + ch];
  if (dskip) v += dskip[i];
  dact[i] = (act[i] & 0x8000u) || !(act[i] & 0x7FFFu) ? 0 : bf16_bits(v);
}

// Adam on FP32 master parameters; refreshes the BF16 copy (c_out, 9, c_in) and, when flip is
// given, the input-gradient copy (c_in, 9, c_out) with the taps reversed; zeroes the gradient.
__global__ void adam_kernel(float* __restrict__ param, float* __restrict__ grad, float* __restrict__ m, float* __restrict__ v,
                            uint16_t* __restrict__ copy, uint16_t* __restrict__ flip, int64_t n, int32_t cout, int32_t cin, float lr,
                            float beta1, float beta2, float eps, float bc1, float bc2) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float g = grad[i];
  const float mi = beta1 * m[i] + (1.0f - beta1) * g;
  const float vi = beta2 * v[i] + (1.0f - beta2) * g * g;
  m[i] = mi;
  v[i] = vi;
  const float p = param[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  param[i] = p;
  grad[i] = 0.0f;
  if (copy) copy[i] = bf16_bits(p);
  if (flip) {
    const int32_t ci = (int32_t)(i % cin);
    const int32_t tap = (int32_t)((i / cin) % 9);
    const int32_t co = (int32_t)(i / ((int64_t)cin * 9));
    flip[((int64_t)ci * 9 + (8 - tap)) * cout + co] = bf16_bits(p);
  }
}

unsigned blocks(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

int cam_image(const MjpbrScene& s, int32_t cam, CamImage* c) {
  if (cam < 0 || cam >= s.nrender || !s.render_rgb[cam] || s.rgb_adr[cam] < 0) {
    return set_error(MJPBR_ERR_ARG, "kpcn: camera %d renders no RGB", cam);
  }
  c->width = s.cam_res[cam][0];
  c->height = s.cam_res[cam][1];
  c->adr = s.rgb_adr[cam];
  return MJPBR_OK;
}

}  // namespace

int kpcn_features_launch(const MjpbrScene& s, int32_t cam, int32_t w0, int32_t nw, uint16_t* x0, cudaStream_t st) {
  CamImage c;
  if (int rc = cam_image(s, cam, &c)) return rc;
  if (!x0 || !s.denoise_buffers[0] || !s.aov_guide) return set_error(MJPBR_ERR_ARG, "kpcn features: missing buffers");
  if (w0 < 0 || nw < 1 || w0 + nw > s.nworld) return set_error(MJPBR_ERR_ARG, "kpcn features: worlds [%d, %d) outside [0, %d)", w0, w0 + nw, s.nworld);
  const int64_t n = (int64_t)nw * c.width * c.height;
  features_kernel<<<blocks(n, 256), 256, 0, st>>>(s, c, w0, nw, x0);
  return check_launch("features_kernel");
}

int kpcn_target_launch(const MjpbrScene& s, int32_t cam, const double* hdr_sum, double inv_n, float* target, cudaStream_t st) {
  CamImage c;
  if (int rc = cam_image(s, cam, &c)) return rc;
  if (!hdr_sum || !target || !s.aov_guide || !s.aov_emission) return set_error(MJPBR_ERR_ARG, "kpcn target: missing buffers");
  const int64_t n = (int64_t)s.nworld * c.width * c.height;
  target_kernel<<<blocks(n, 256), 256, 0, st>>>(s, c, hdr_sum, inv_n, reinterpret_cast<float4*>(target));
  return check_launch("target_kernel");
}

int accumulate_f64_launch(const float* src, double* acc, int64_t n, cudaStream_t st) {
  if (!src || !acc || n < 0) return set_error(MJPBR_ERR_ARG, "accumulate: bad arguments");
  if (n == 0) return MJPBR_OK;
  accumulate_f64_kernel<<<blocks(n, 256), 256, 0, st>>>(src, acc, n);
  return check_launch("accumulate_f64_kernel");
}

int upsample2_launch(const uint16_t* in, uint16_t* out, int32_t nimg, int32_t h, int32_t w, int32_t c, cudaStream_t st) {
  if (!in || !out || nimg < 1 || h < 1 || w < 1 || c < 8 || c % 8) return set_error(MJPBR_ERR_ARG, "upsample2: bad arguments");
  if ((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15u) return set_error(MJPBR_ERR_ARG, "upsample2: tensors must be 16-byte aligned");
  const int64_t n = (int64_t)nimg * 4 * h * w * (c / 8);
  upsample2_kernel<<<blocks(n, 256), 256, 0, st>>>(reinterpret_cast<const uint4*>(in), reinterpret_cast<uint4*>(out), nimg, h, w, c / 8);
  return check_launch("upsample2_kernel");
}

int avgpool2_launch(const uint16_t* in, uint16_t* out, int32_t nimg, int32_t h, int32_t w, int32_t c, cudaStream_t st) {
  if (!in || !out || h % 2 || w % 2 || c < 1) return set_error(MJPBR_ERR_ARG, "avgpool2: bad arguments");
  if (c % 8 == 0 && !((reinterpret_cast<uintptr_t>(in) | reinterpret_cast<uintptr_t>(out)) & 15u)) {
    const int64_t n = (int64_t)nimg * (h / 2) * (w / 2) * (c / 8);
    avgpool2_kernel<<<blocks(n, 256), 256, 0, st>>>(reinterpret_cast<const uint4*>(in), reinterpret_cast<uint4*>(out), nimg, h, w, c / 8);
    return check_launch("avgpool2_kernel");
  }
  const int64_t n = (int64_t)nimg * (h / 2) * (w / 2) * c;
  avgpool2_scalar_kernel<<<blocks(n, 256), 256, 0, st>>>(in, out, nimg, h, w, c);
  return check_launch("avgpool2_scalar_kernel");
}

int kpcn_apply_launch(const float* logits, const float* radiance, float* weights, float* out, int32_t nimg, int32_t h, int32_t w,
                      cudaStream_t st) {
  if (!logits || !radiance || !out) return set_error(MJPBR_ERR_ARG, "kpcn apply: bad arguments");
  const int64_t n = (int64_t)nimg * h * w;
  apply_kernel<<<blocks(n, 128), 128, 0, st>>>(logits, reinterpret_cast<const float4*>(radiance), weights,
                                                reinterpret_cast<float4*>(out), nimg, h, w);
  return check_launch("apply_kernel");
}

int kpcn_loss_launch(const float* out, const float* target, const float* scale, const float* offset, float* grad, float* sums,
                     int64_t npix, float w_l1, float w_rel, cudaStream_t st) {
  if (!out || !target || !grad || !sums) return set_error(MJPBR_ERR_ARG, "kpcn loss: bad arguments");
  loss_kernel<<<blocks(npix, 256), 256, 0, st>>>(reinterpret_cast<const float4*>(out), reinterpret_cast<const float4*>(target),
                                                 reinterpret_cast<const float4*>(scale), reinterpret_cast<const float4*>(offset),
                                                 reinterpret_cast<float4*>(grad), sums, npix, w_l1, w_rel);
  return check_launch("loss_kernel");
}

int kpcn_remod_launch(const MjpbrScene& s, int32_t cam, float* scale, float* offset, cudaStream_t st) {
  CamImage c;
  if (int rc = cam_image(s, cam, &c)) return rc;
  if (!scale || !offset || !s.aov_guide || !s.aov_emission) return set_error(MJPBR_ERR_ARG, "kpcn remod: missing buffers");
  const int64_t n = (int64_t)s.nworld * c.width * c.height;
  remod_kernel<<<blocks(n, 256), 256, 0, st>>>(s, c, reinterpret_cast<float4*>(scale), reinterpret_cast<float4*>(offset));
  return check_launch("remod_kernel");
}

int kpcn_apply_grad_launch(const float* grad, const float* weights, const float* radiance, uint16_t* grad_logits, int32_t nimg,
                           int32_t h, int32_t w, cudaStream_t st) {
  if (!grad || !weights || !radiance || !grad_logits) return set_error(MJPBR_ERR_ARG, "kpcn apply grad: bad arguments");
  const int64_t n = (int64_t)nimg * h * w;
  apply_grad_kernel<<<blocks(n, 128), 128, 0, st>>>(reinterpret_cast<const float4*>(grad), weights,
                                                     reinterpret_cast<const float4*>(radiance), grad_logits, nimg, h, w);
  return check_launch("apply_grad_kernel");
}

int split_concat_grad_launch(const float* dcat, const uint16_t* low, float* dskip, uint16_t* dlow, int32_t nimg, int32_t h, int32_t w,
                             int32_t c1, int32_t c2, cudaStream_t st) {
  if (!dcat || !low || !dskip || !dlow || h % 2 || w % 2) return set_error(MJPBR_ERR_ARG, "split concat grad: bad arguments");
  if (c1 % 4 == 0 && c2 % 4 == 0 && !((reinterpret_cast<uintptr_t>(dcat) | reinterpret_cast<uintptr_t>(dskip)) & 15u) &&
      !((reinterpret_cast<uintptr_t>(low) | reinterpret_cast<uintptr_t>(dlow)) & 7u)) {
    const int64_t n = std::max<int64_t>((int64_t)nimg * h * w * (c1 / 4), (int64_t)nimg * (h / 2) * (w / 2) * (c2 / 4));
    split_concat_grad4_kernel<<<blocks(n, 256), 256, 0, st>>>(reinterpret_cast<const float4*>(dcat), reinterpret_cast<const uint2*>(low),
                                                             reinterpret_cast<float4*>(dskip), reinterpret_cast<uint2*>(dlow), nimg, h, w, c1 / 4,
                                                             c2 / 4);
    return check_launch("split_concat_grad4_kernel");
  }
  const int64_t n = std::max<int64_t>((int64_t)nimg * h * w * c1, (int64_t)nimg * (h / 2) * (w / 2) * c2);
  split_concat_grad_kernel<<<blocks(n, 256), 256, 0, st>>>(dcat, low, dskip, dlow, nimg, h, w, c1, c2);
  return check_launch("split_concat_grad_kernel");
}

int unpool_add_grad_launch(const float* dskip, const float* dpool, const uint16_t* act, uint16_t* dact, int32_t nimg, int32_t h,
                           int32_t w, int32_t c, cudaStream_t st) {
  if (!dpool || !act || !dact || h % 2 || w % 2) return set_error(MJPBR_ERR_ARG, "unpool add grad: bad arguments");
  if (c % 4 == 0 && !((reinterpret_cast<uintptr_t>(dskip) | reinterpret_cast<uintptr_t>(dpool)) & 15u) &&
      !((reinterpret_cast<uintptr_t>(act) | reinterpret_cast<uintptr_t>(dact)) & 7u)) {
    const int64_t n = (int64_t)nimg * h * w * (c / 4);
    unpool_add_grad4_kernel<<<blocks(n, 256), 256, 0, st>>>(reinterpret_cast<const float4*>(dskip), reinterpret_cast<const float4*>(dpool),
                                                           reinterpret_cast<const uint2*>(act), reinterpret_cast<uint2*>(dact), nimg, h, w, c / 4);
    return check_launch("unpool_add_grad4_kernel");
  }
  const int64_t n = (int64_t)nimg * h * w * c;
  unpool_add_grad_kernel<<<blocks(n, 256), 256, 0, st>>>(dskip, dpool, act, dact, nimg, h, w, c);
  return check_launch("unpool_add_grad_kernel");
}

int adam_launch(float* param, float* grad, float* m, float* v, uint16_t* copy, uint16_t* flip, int64_t n, int32_t cout, int32_t cin,
                float lr, float beta1, float beta2, float eps, int32_t step, cudaStream_t st) {
  if (!param || !grad || !m || !v || n <= 0 || step < 1) return set_error(MJPBR_ERR_ARG, "adam: bad arguments");
  if (flip && (cout < 1 || cin < 1 || (int64_t)cout * 9 * cin != n)) return set_error(MJPBR_ERR_ARG, "adam: flip needs n = c_out * 9 * c_in");
  const float bc1 = 1.0f - powf(beta1, (float)step), bc2 = 1.0f - powf(beta2, (float)step);
  adam_kernel<<<blocks(n, 256), 256, 0, st>>>(param, grad, m, v, copy, flip, n, cout, cin, lr, beta1, beta2, eps, bc1, bc2);
  return check_launch("adam_kernel");
}

}  // namespace mjpbr
