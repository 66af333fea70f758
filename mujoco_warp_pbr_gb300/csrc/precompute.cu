// Context-creation tables on the GPU: the split-sum DFG table (mujoco_warp_pbr/_src/ibl.py:62-101),
// box-filtered mip chains (texture.py:91-99, envmap.py:330-337: Warp builds them when it creates a
// mipmapped texture), the GGX-prefiltered environment stack with filtered importance sampling
// (envmap.py:171-221; Karis 2013, Krivanek & Colbert 2008), the environment's 9 spherical-harmonic
// coefficients of Lambertian radiance (envmap.py:224-249; Ramamoorthi & Hanrahan 2001) and its
// importance-sampling distribution (envmap.py:409-430).
#include "abi_internal.h"
#include "shading.cuh"

namespace mjpbr {
namespace {

MJ_DEV void hammersley(uint32_t i, float inv_n, float* x, float* y) {
  uint32_t bits = __brev(i);
  *x = (float)i * inv_n;
  *y = (float)bits * (1.0f / 4294967296.0f);
}

// Half vector around +z distributed as D(h) (h . n).
MJ_DEV V3 importance_sample_ggx(float ux, float uy, float alpha) {
  float a2 = alpha * alpha;
  float phi = 2.0f * kPi * ux;
  float cos2 = (1.0f - uy) / (1.0f + (a2 - 1.0f) * uy);
  float ct = sqrtf(cos2);
  float st = sqrtf(fmaxf(1.0f - cos2, 0.0f));
  return V3{st * cosf(phi), st * sinf(phi), ct};
}

__global__ void dfg_kernel(float* lut, int32_t n, int32_t nsample) {
  int32_t i = blockIdx.x * blockDim.x + threadIdx.x;  // NoV column
  int32_t j = blockIdx.y;                             // roughness row
  if (i >= n) return;
  float nov = ((float)i + 0.5f) / (float)n;
  float pr = ((float)j + 0.5f) / (float)n;
  float alpha = pr * pr;
  V3 v{sqrtf(1.0f - nov * nov), 0.0f, nov};
  float inv_n = 1.0f / (float)nsample;
  float x = 0.0f, y = 0.0f;
  for (int32_t s = 0; s < nsample; ++s) {
    float ux, uy;
    hammersley((uint32_t)s, inv_n, &ux, &uy);
    V3 h = importance_sample_ggx(ux, uy, alpha);
    float voh = dot(v, h);
    V3 l = h * (2.0f * voh) - v;
    float nol = l.z, noh = h.z;
    if (nol > 0.0f && voh > 0.0f) {
      float gv = v_smith_ggx_correlated(nov, nol, alpha) * 4.0f * voh * nol / noh;
      float fc = powf(1.0f - voh, 5.0f);
      x += gv * fc;
      y += gv;
    }
  }
  lut[(j * n + i) * 2] = x * inv_n;
  lut[(j * n + i) * 2 + 1] = y * inv_n;
}

__global__ void mip_kernel(const __grid_constant__ MjpbrTexture t, uint8_t* data, int32_t level) {
  int32_t sw = max(t.width >> (level - 1), 1), sh = max(t.height >> (level - 1), 1);
  int32_t dw = max(t.width >> level, 1), dh = max(t.height >> level, 1);
  int32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
  if (x >= dw || y >= dh) return;
  int32_t x0 = min(2 * x, sw - 1), x1 = min(2 * x + 1, sw - 1);
  int32_t y0 = min(2 * y, sh - 1), y1 = min(2 * y + 1, sh - 1);
  if (t.format == MJPBR_TEX_RGBA8) {
    const uchar4* src = reinterpret_cast<const uchar4*>(data + t.level_offset[level - 1]);
    uchar4 a = src[y0 * sw + x0], b = src[y0 * sw + x1], c = src[y1 * sw + x0], d = src[y1 * sw + x1];
    uchar4 o;
    o.x = (unsigned char)(((unsigned)a.x + b.x + c.x + d.x + 2u) >> 2);
    o.y = (unsigned char)(((unsigned)a.y + b.y + c.y + d.y + 2u) >> 2);
    o.z = (unsigned char)(((unsigned)a.z + b.z + c.z + d.z + 2u) >> 2);
    o.w = (unsigned char)(((unsigned)a.w + b.w + c.w + d.w + 2u) >> 2);
    reinterpret_cast<uchar4*>(data + t.level_offset[level])[y * dw + x] = o;
  } else {
    const uint16_t* src = reinterpret_cast<const uint16_t*>(data + t.level_offset[level - 1]);
    uint16_t* dst = reinterpret_cast<uint16_t*>(data + t.level_offset[level]);
    for (int k = 0; k < 4; ++k) {
      float s = half_to_float(src[(y0 * sw + x0) * 4 + k]) + half_to_float(src[(y0 * sw + x1) * 4 + k]) +
                half_to_float(src[(y1 * sw + x0) * 4 + k]) + half_to_float(src[(y1 * sw + x1) * 4 + k]);
      dst[(y * dw + x) * 4 + k] = float_to_half(s * 0.25f);
    }
  }
}

MJ_DEV V3 uv_to_direction(float u, float v) {
  float phi = (u - 0.5f) * (2.0f * kPi);
  float theta = v * kPi;
  float st = sinf(theta);
  return V3{st * cosf(phi), st * sinf(phi), cosf(theta)};
}

__global__ void prefilter_kernel(const __grid_constant__ MjpbrTexture t, const uint8_t* data, int32_t levels,
                                 int32_t height, int32_t width, int32_t nsample, uint16_t* stack) {
  int32_t x = blockIdx.x * blockDim.x + threadIdx.x;
  int32_t y = blockIdx.y;
  int32_t level = blockIdx.z;
  if (x >= width) return;
  V3 n = uv_to_direction(((float)x + 0.5f) / (float)width, ((float)y + 0.5f) / (float)height);
  float pr = (float)level / (float)(levels - 1);
  float alpha = fmaxf(pr * pr, 1.0e-4f);
  V3 up = fabsf(n.z) < 0.999f ? V3{0.0f, 0.0f, 1.0f} : V3{1.0f, 0.0f, 0.0f};
  V3 tt = normalize(cross(up, n));
  V3 bb = cross(n, tt);
  float texel_sa = 4.0f * kPi / (float)(t.width * t.height);
  float inv_n = 1.0f / (float)nsample;
  V3 color = v3(0.0f);
  float weight = 0.0f;
  for (int32_t s = 0; s < nsample; ++s) {
    float ux, uy;
    hammersley((uint32_t)s, inv_n, &ux, &uy);
    V3 hl = importance_sample_ggx(ux, uy, alpha);
    V3 h = tt * hl.x + bb * hl.y + n * hl.z;
    float noh = hl.z;
    V3 l = h * (2.0f * noh) - n;
    float nol = dot(n, l);
    if (nol > 0.0f) {
      float pdf = d_ggx(noh, alpha) * 0.25f;
      float sa = inv_n / fmaxf(pdf, 1.0e-8f);
      float lod = level == 0 ? 0.0f : 0.5f * log2f(sa / texel_sa) + 1.0f;
      float u, v;
      direction_to_uv(l, 0.0f, &u, &v);
      float4 c = sample_trilinear(t, data, u, v, fmaxf(lod, 0.0f), true, false);
      color += V3{c.x, c.y, c.z} * nol;
      weight += nol;
    }
  }
  color = color / fmaxf(weight, 1.0e-8f);
  uint16_t* o = stack + (((int64_t)level * height + y) * width + x) * 4;
  o[0] = float_to_half(color.x);
  o[1] = float_to_half(color.y);
  o[2] = float_to_half(color.z);
  o[3] = float_to_half(1.0f);
}

// ---------------------------------------------------------------- SH9 irradiance
// Projection of an equirect radiance image (row 0 = +z, column centre = +x) onto the real
// spherical harmonics of bands 0-2, weighted by each texel's solid angle (2 pi / w)(pi / h)
// sin(theta), accumulated in double precision: first one partial sum per row and coefficient
// (a CTA per row, a fixed-order tree over its threads), then the rows in order (deterministic).

constexpr int kShThreads = 256;

// Real SH basis of bands 0-2 at unit direction (x, y, z), with the usual normalisations
// 1 / (2 sqrt(pi)), sqrt(3 / (4 pi)), sqrt(15 / (4 pi)), sqrt(5 / (16 pi)), sqrt(15 / (16 pi))
// rounded to 6 digits.
__device__ __forceinline__ void sh_basis(double x, double y, double z, double* b) {
  b[0] = 0.282095;
  b[1] = 0.488603 * y;
  b[2] = 0.488603 * z;
  b[3] = 0.488603 * x;
  b[4] = 1.092548 * x * y;
  b[5] = 1.092548 * y * z;
  b[6] = 0.315392 * (3.0 * z * z - 1.0);
  b[7] = 1.092548 * x * z;
  b[8] = 0.546274 * (x * x - y * y);
}

__global__ void __launch_bounds__(kShThreads) sh9_rows_kernel(const float* image, int32_t h, int32_t w, double* rows) {
  __shared__ double red[kShThreads];
  const int32_t y = blockIdx.x;
  const double pi = 3.14159265358979323846;
  const double theta = ((double)y + 0.5) / (double)h * pi;
  const double st = sin(theta), ct = cos(theta);
  const double dw = (2.0 * pi / (double)w) * (pi / (double)h) * st;
  double acc[27];
  for (int k = 0; k < 27; ++k) acc[k] = 0.0;
  for (int32_t x = threadIdx.x; x < w; x += kShThreads) {
    const double phi = (((double)x + 0.5) / (double)w - 0.5) * 2.0 * pi;
    double b[9];
    sh_basis(st * cos(phi), st * sin(phi), ct, b);
    const float* px = image + ((int64_t)y * w + x) * 3;
    for (int k = 0; k < 9; ++k) {
      const double wb = b[k] * dw;
      for (int c = 0; c < 3; ++c) acc[k * 3 + c] += wb * (double)px[c];
    }
  }
  for (int k = 0; k < 27; ++k) {
    red[threadIdx.x] = acc[k];
    __syncthreads();
    for (int stride = kShThreads / 2; stride > 0; stride >>= 1) {
      if (threadIdx.x < stride) red[threadIdx.x] += red[threadIdx.x + stride];
      __syncthreads();
    }
    if (threadIdx.x == 0) rows[(int64_t)y * 27 + k] = red[0];
    __syncthreads();
  }
}

// Sums the rows (in row order) and applies the Lambertian band factors pi, 2 pi / 3, pi / 4,
// divided by pi: the coefficients of radiance, not irradiance.
__global__ void sh9_sum_kernel(const double* rows, int32_t h, float* sh) {
  const int k = threadIdx.x;
  if (k >= 27) return;
  double sum = 0.0;
  for (int32_t y = 0; y < h; ++y) sum += rows[(int64_t)y * 27 + k];
  const int band = k / 3 == 0 ? 0 : (k / 3 < 4 ? 1 : 2);
  const double factor = band == 0 ? 1.0 : (band == 1 ? 2.0 / 3.0 : 0.25);
  sh[k] = (float)(sum * factor);
}

// ---------------------------------------------------------------- importance-sampling tables
// A piecewise-constant distribution over the cells of an equirect image proportional to
// luminance (Rec. 709 weights) times sin(theta), with a floor of 1e-6 of the mean luminance so
// that no cell has zero probability: cell probabilities (h, w), the marginal CDF over rows
// (h + 1) and one conditional CDF over the columns of each row (h, w + 1); the last entry of
// every CDF is exactly 1. Double precision, one CTA per image, rows on threads (each row summed
// in column order, rows in row order: deterministic).
__global__ void env_tables_kernel(const double* image, int32_t h, int32_t w, float* prob, float* marginal, float* conditional) {
  extern __shared__ double row[];  // h entries
  __shared__ double total_s, eps_s;
  const double pi = 3.14159265358979323846;
  auto lum = [&](int32_t y, int32_t x) {
    const double* p = image + ((int64_t)y * w + x) * 3;
    return p[0] * 0.2126 + p[1] * 0.7152 + p[2] * 0.0722;
  };
  for (int32_t y = threadIdx.x; y < h; y += blockDim.x) {
    double s = 0.0;
    for (int32_t x = 0; x < w; ++x) s += lum(y, x);
    row[y] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int32_t y = 0; y < h; ++y) s += row[y];
    eps_s = 1.0e-6 * fmax(s / ((double)h * (double)w), 1.0e-12);
  }
  __syncthreads();
  const double eps = eps_s;
  for (int32_t y = threadIdx.x; y < h; y += blockDim.x) {
    const double st = sin(((double)y + 0.5) / (double)h * pi);
    double s = 0.0;
    for (int32_t x = 0; x < w; ++x) s += lum(y, x) * st + eps;
    row[y] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int32_t y = 0; y < h; ++y) s += row[y];
    total_s = s;
  }
  __syncthreads();
  const double inv_total = 1.0 / total_s;
  for (int32_t y = threadIdx.x; y < h; y += blockDim.x) {
    const double st = sin(((double)y + 0.5) / (double)h * pi);
    double r = 0.0;
    for (int32_t x = 0; x < w; ++x) {
      const double p = (lum(y, x) * st + eps) * inv_total;
      prob[(int64_t)y * w + x] = (float)p;
      r += p;
    }
    const double inv_r = 1.0 / fmax(r, 1.0e-30);
    float* cond = conditional + (int64_t)y * (w + 1);
    double c = 0.0;
    cond[0] = 0.0f;
    for (int32_t x = 0; x < w; ++x) {
      c += (lum(y, x) * st + eps) * inv_total;
      cond[x + 1] = (float)(c * inv_r);
    }
    cond[w] = 1.0f;
    row[y] = r;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double c = 0.0;
    marginal[0] = 0.0f;
    for (int32_t y = 0; y < h; ++y) {
      c += row[y];
      marginal[y + 1] = (float)c;
    }
    marginal[h] = 1.0f;
  }
}

}  // namespace

int env_sh9_launch(const float* image, int32_t h, int32_t w, double* rows, float* sh, cudaStream_t stream) {
  if (!image || !rows || !sh || h < 1 || w < 1) return set_error(MJPBR_ERR_ARG, "env_sh9: bad arguments");
  sh9_rows_kernel<<<h, kShThreads, 0, stream>>>(image, h, w, rows);
  int rc = check_launch("sh9_rows_kernel");
  if (rc) return rc;
  sh9_sum_kernel<<<1, 32, 0, stream>>>(rows, h, sh);
  return check_launch("sh9_sum_kernel");
}

int env_tables_launch(const double* image, int32_t h, int32_t w, float* prob, float* marginal, float* conditional,
                      cudaStream_t stream) {
  if (!image || !prob || !marginal || !conditional || h < 1 || w < 1 || h > 4096) {
    return set_error(MJPBR_ERR_ARG, "env_tables: bad arguments (height must be in [1, 4096])");
  }
  env_tables_kernel<<<1, 128, (size_t)h * sizeof(double), stream>>>(image, h, w, prob, marginal, conditional);
  return check_launch("env_tables_kernel");
}

int dfg_lut_launch(float* lut, int32_t size, int32_t nsample, cudaStream_t stream) {
  if (!lut || size < 2 || nsample < 1) return set_error(MJPBR_ERR_ARG, "dfg_lut: bad arguments");
  dim3 grid((size + 127) / 128, size);
  dfg_kernel<<<grid, 128, 0, stream>>>(lut, size, nsample);
  return check_launch("dfg_kernel");
}

// tex: host description of a texture whose level 0 is in data (device).
int build_mips_launch(const MjpbrTexture* tex, uint8_t* data, cudaStream_t stream) {
  if (!tex || !data) return set_error(MJPBR_ERR_ARG, "build_mips: NULL argument");
  const MjpbrTexture t = *tex;
  if (t.nlevel < 1 || t.nlevel > MJPBR_MAX_MIPS || t.width < 1 || t.height < 1) {
    return set_error(MJPBR_ERR_ARG, "build_mips: bad texture description");
  }
  for (int32_t level = 1; level < t.nlevel; ++level) {
    int32_t dw = max(t.width >> level, 1), dh = max(t.height >> level, 1);
    dim3 grid((dw + 127) / 128, dh);
    mip_kernel<<<grid, 128, 0, stream>>>(t, data, level);
    int rc = check_launch("mip_kernel");
    if (rc) return rc;
  }
  return MJPBR_OK;
}

int prefilter_launch(const MjpbrTexture* radiance, const uint8_t* data, int32_t levels, int32_t height, int32_t width,
                     int32_t nsample, uint16_t* stack, cudaStream_t stream) {
  if (levels < 2 || height < 1 || width < 1 || nsample < 1 || !stack) return set_error(MJPBR_ERR_ARG, "prefilter: bad arguments");
  dim3 grid((width + 127) / 128, height, levels);
  if (!radiance || !data) return set_error(MJPBR_ERR_ARG, "prefilter: NULL radiance");
  prefilter_kernel<<<grid, 128, 0, stream>>>(*radiance, data, levels, height, width, nsample, stack);
  return check_launch("prefilter_kernel");
}

}  // namespace mjpbr
