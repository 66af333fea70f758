// 3x3 convolutions of the learned denoiser as implicit GEMMs on the 5th-generation tensor cores.
//
// A CTA of 128 threads computes one tile of 128 output pixels (a run of one image row, or
// 128 / width whole rows) times all output channels: D (128 x c_out, FP32 in tensor memory) =
// sum over the 9 taps and the input channels of A_tap (128 x c_in) * W_tap^T. The input channels
// are processed 16 at a time. For each 16-channel chunk the threads stage into shared memory,
// in the K-major core-matrix layout, three copies of the tile's input rows plus a one-row halo
// above and below, shifted by -1, 0 and +1 pixel (the dx of the taps; zero outside the image), so
// that the A operand of tap (dy, dx) is one descriptor: copy dx, starting dy rows down, with a
// uniform 16-byte row stride across the whole tile (the rows are stored with pitch = tile row
// length, so consecutive output pixels, also across image rows, are consecutive operand rows).
// One elected thread then issues the chunk's 9 tcgen05.mma instructions (K = 16 each) and commits
// them to an mbarrier; the buffer is restaged after they completed. Two CTAs per SM overlap one
// CTA's staging with the other's MMAs. The epilogue reads the accumulator rows out of tensor
// memory (tcgen05.ld), adds the bias, applies ReLU and / or a ReLU-derivative mask and stores
// BF16 (and optionally FP32) NHWC.
//
// The U-Net's skip concatenation is read in place: channels past c_in come from the half-
// resolution tensor in2, upsampled x2 (nearest) while staging.
#include <cuda_bf16.h>

#include <algorithm>
#include <climits>

#include "abi_internal.h"
#include "common.cuh"
#include "umma.cuh"

namespace mjpbr {
namespace {

constexpr int kTilePx = 128;
constexpr int kConvThreads = 128;

struct ConvGeom {
  int32_t pitch;  // pixels per staged row (min(width, 128))
  int32_t rows;   // image rows per tile (128 / pitch)
  int32_t tiles_per_row, tiles_per_img;
  int32_t cin;    // c_in + c_in2
};

__device__ __forceinline__ uint4 load_px(const MjpbrConv& p, int32_t img, int32_t iy, int32_t ix, int32_t ch) {
  if (iy < 0 || iy >= p.height || ix < 0 || ix >= p.width) return make_uint4(0u, 0u, 0u, 0u);
  if (ch < p.c_in) {
    return __ldg(reinterpret_cast<const uint4*>(p.in + (((int64_t)img * p.height + iy) * p.width + ix) * p.c_in + ch));
  }
  const int32_t h2 = p.height >> 1, w2 = p.width >> 1;
  return __ldg(reinterpret_cast<const uint4*>(p.in2 + (((int64_t)img * h2 + (iy >> 1)) * w2 + (ix >> 1)) * p.c_in2 + (ch - p.c_in)));
}

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
  const uint32_t lo = __bfloat16_as_ushort(__float2bfloat16_rn(a));
  const uint32_t hi = __bfloat16_as_ushort(__float2bfloat16_rn(b));
  return lo | (hi << 16);
}

__global__ void __launch_bounds__(kConvThreads, 2) conv3x3_kernel(const __grid_constant__ MjpbrConv p, const ConvGeom g) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_slot;
  const int32_t P = g.pitch, R = g.rows;
  const int32_t plane = (R + 2) * P * 16;  // bytes of one (dx, channel group) plane
  uint8_t* sa = smem;                      // [dx 3][group 2][R + 2 rows][P] x 16 B
  uint8_t* sb = smem + 6 * plane;          // [tap 9][group 2][c_out] x 16 B
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int32_t cout = p.c_out;
  const int32_t img = blockIdx.x / g.tiles_per_img;
  const int32_t t = blockIdx.x - img * g.tiles_per_img;
  const int32_t y0 = (t / g.tiles_per_row) * R, x0 = (t % g.tiles_per_row) * P;
  uint32_t ncols = 32;
  while (ncols < (uint32_t)cout) ncols <<= 1;
  if (warp == 0) umma::tmem_alloc(&tmem_slot, ncols);
  if (tid == 0) {
    umma::mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = umma::make_idesc_bf16(kTilePx, cout);
  const int32_t nchunk = g.cin / 16;
  const int32_t halo_row = P + 2;
  bool ok = true;
  uint32_t phase = 0;
  for (int32_t c = 0; c < nchunk; ++c) {
    const int32_t cb = c * 16;
    // A: each input pixel of the halo'd tile rows is loaded once and stored into the copies
    // (dx = 0, 1, 2 for offsets -1, 0, +1) where it lands
    const int32_t nload = 2 * (R + 2) * halo_row;
    for (int32_t i = tid; i < nload; i += kConvThreads) {
      const int32_t grp = i / ((R + 2) * halo_row);
      const int32_t rem = i - grp * (R + 2) * halo_row;
      const int32_t j = rem / halo_row;
      const int32_t xi = rem - j * halo_row - 1;
      const uint4 v = load_px(p, img, y0 - 1 + j, x0 + xi, cb + grp * 8);
#pragma unroll
      for (int32_t dx = 0; dx < 3; ++dx) {
        const int32_t x = xi - dx + 1;
        if (x >= 0 && x < P) *reinterpret_cast<uint4*>(sa + (dx * 2 + grp) * plane + (j * P + x) * 16) = v;
      }
    }
    // B: the chunk's 16 input channels of every tap and output channel
    for (int32_t i = tid; i < 18 * cout; i += kConvThreads) {
      const int32_t tg = i / cout, co = i - tg * cout;
      const int32_t tap = tg >> 1, grp = tg & 1;
      const uint4 v = __ldg(reinterpret_cast<const uint4*>(p.weight + ((int64_t)co * 9 + tap) * g.cin + cb + grp * 8));
      *reinterpret_cast<uint4*>(sb + (tg * cout + co) * 16) = v;
    }
    umma::fence_async_shared();
    __syncthreads();
    umma::fence_after_sync();
    if (tid == 0) {
      const uint32_t a0 = umma::smem_addr(sa), b0 = umma::smem_addr(sb);
#pragma unroll 1
      for (int32_t tap = 0; tap < 9; ++tap) {
        const int32_t dy = tap / 3, dx = tap - dy * 3;
        const uint64_t ad = umma::make_desc(a0 + dx * 2 * plane + dy * P * 16, plane, 128);
        const uint64_t bd = umma::make_desc(b0 + tap * 2 * cout * 16, cout * 16, 128);
        umma::mma_bf16(tmem, ad, bd, idesc, c > 0 || tap > 0);
      }
      umma::commit(&bar);
    }
    ok = umma::mbar_wait(&bar, phase);
    phase ^= 1u;
    umma::fence_after_sync();
    __syncthreads();
    if (!ok) break;
  }
  if (ok) {
    const int32_t m = warp * 32 + lane;
    const int32_t y = y0 + m / P, x = x0 + m % P;
    const int64_t pix = ((int64_t)img * p.height + y) * p.width + x;
#pragma unroll 1
    for (int32_t c0 = 0; c0 < cout; c0 += 16) {
      float v[16];
      umma::tmem_load16(tmem + ((uint32_t)(warp * 32) << 16) + c0, v);
      if (p.bias) {
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] += __ldg(p.bias + c0 + i);
      }
      if (p.relu) {
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] = fmaxf(v[i], 0.0f);
      }
      if (p.mask) {
        const uint4* mk = reinterpret_cast<const uint4*>(p.mask + pix * cout + c0);
        const uint4 m0 = __ldg(mk), m1 = __ldg(mk + 1);
        const uint32_t w[8] = {m0.x, m0.y, m0.z, m0.w, m1.x, m1.y, m1.z, m1.w};
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          // a BF16 value is > 0 when its sign bit is clear and it is not zero
          if ((w[i] & 0x8000u) || !(w[i] & 0x7FFFu)) v[2 * i] = 0.0f;
          if ((w[i] & 0x80000000u) || !(w[i] & 0x7FFF0000u)) v[2 * i + 1] = 0.0f;
        }
      }
      if (p.out) {
        uint4* o = reinterpret_cast<uint4*>(p.out + pix * cout + c0);
        o[0] = make_uint4(pack_bf16x2(v[0], v[1]), pack_bf16x2(v[2], v[3]), pack_bf16x2(v[4], v[5]), pack_bf16x2(v[6], v[7]));
        o[1] = make_uint4(pack_bf16x2(v[8], v[9]), pack_bf16x2(v[10], v[11]), pack_bf16x2(v[12], v[13]), pack_bf16x2(v[14], v[15]));
      }
      if (p.out_f32) {
        float4* o = reinterpret_cast<float4*>(p.out_f32 + pix * cout + c0);
#pragma unroll
        for (int i = 0; i < 4; ++i) o[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
      }
    }
  } else {
    if (tid == 0 && p.error_word) atomicOr(p.error_word, kErrWaitTimeout);
    umma::mbar_wait(&bar, phase ^ 1u);
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) umma::tmem_free(tmem, ncols);
}

bool aligned16(const void* q) { return (reinterpret_cast<uintptr_t>(q) & 15u) == 0; }

}  // namespace

int conv3x3_launch(const MjpbrConv& c, cudaStream_t stream) {
  if (!c.in || !c.weight || (!c.out && !c.out_f32)) return set_error(MJPBR_ERR_ARG, "conv3x3: missing input, weight or output");
  if (c.nimg < 1 || c.height < 1 || c.width < 1) return set_error(MJPBR_ERR_ARG, "conv3x3: empty image batch");
  if (c.c_in < 16 || c.c_in % 16 || c.c_in2 < 0 || c.c_in2 % 16 || c.c_out < 16 || c.c_out % 16 || c.c_out > 256) {
    return set_error(MJPBR_ERR_ARG, "conv3x3: channels must be multiples of 16 (c_out <= 256), got %d + %d -> %d", c.c_in, c.c_in2,
                     c.c_out);
  }
  if (c.c_in2 > 0 && (!c.in2 || c.height % 2 || c.width % 2)) return set_error(MJPBR_ERR_ARG, "conv3x3: in2 needs even sizes");
  const int32_t w = c.width;
  const bool row_ok = (w >= 128) ? (w % 128 == 0) : (w >= 16 && 128 % w == 0);
  if (!row_ok) return set_error(MJPBR_ERR_ARG, "conv3x3: width %d is not a power of two in [16, 128] or a multiple of 128", w);
  ConvGeom g;
  g.pitch = std::min(w, 128);
  g.rows = 128 / g.pitch;
  if (c.height % g.rows) return set_error(MJPBR_ERR_ARG, "conv3x3: height %d is not a multiple of %d", c.height, g.rows);
  if (!aligned16(c.in) || !aligned16(c.in2) || !aligned16(c.weight) || !aligned16(c.out) || !aligned16(c.out_f32) ||
      !aligned16(c.mask)) {
    return set_error(MJPBR_ERR_ARG, "conv3x3: tensors must be 16-byte aligned");
  }
  g.tiles_per_row = w / g.pitch;
  g.tiles_per_img = (c.height / g.rows) * g.tiles_per_row;
  g.cin = c.c_in + c.c_in2;
  const int64_t tiles = (int64_t)c.nimg * g.tiles_per_img;
  if (tiles > INT32_MAX) return set_error(MJPBR_ERR_ARG, "conv3x3: too many tiles");
  const size_t smem = (size_t)6 * (g.rows + 2) * g.pitch * 16 + (size_t)18 * c.c_out * 16;
  static size_t smem_set = 0;
  if (smem > smem_set) {
    cudaError_t e = cudaFuncSetAttribute(conv3x3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return set_error(MJPBR_ERR_CUDA, "conv3x3: %zu bytes of shared memory: %s", smem, cudaGetErrorString(e));
    smem_set = smem;
  }
  conv3x3_kernel<<<(unsigned)tiles, kConvThreads, smem, stream>>>(c, g);
  return check_launch("conv3x3_kernel");
}

}  // namespace mjpbr

// ---------------------------------------------------------------- weight gradients
//
// grad_weight[co][tap][ci] = sum over pixels p of grad_out[p][co] * in[p + offset(tap)][ci]: a
// GEMM with M = the 9 x c_in (tap, channel) pairs, N = c_out and K = pixels. Both operands are
// K-major along pixels, so the staging transposes 8 x 8 blocks (8 pixels x 8 channels) in
// registers (byte permutes) before storing them as core-matrix rows. A CTA owns one 128-row block
// of (tap, channel) pairs and accumulates a run of 128-pixel tiles in tensor memory, then adds
// its accumulators to grad_weight with coalesced atomics.
namespace mjpbr {
namespace {

struct WgradGeom {
  int32_t pitch, rows, tiles_per_row, tiles_per_img;
  int32_t cin;        // c_in + c_in2
  int32_t total;      // tiles of the batch
  int32_t per_cta;    // tiles per CTA
};

// Transposes 8 rows (one 16-byte vector of 8 BF16 each) into 8 columns.
__device__ __forceinline__ void transpose8x8(const uint4 (&r)[8], uint4 (&c)[8]) {
  uint32_t w[8][4];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    w[i][0] = r[i].x;
    w[i][1] = r[i].y;
    w[i][2] = r[i].z;
    w[i][3] = r[i].w;
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    uint32_t o[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) o[j] = __byte_perm(w[2 * j][k >> 1], w[2 * j + 1][k >> 1], (k & 1) ? 0x7632 : 0x5410);
    c[k] = make_uint4(o[0], o[1], o[2], o[3]);
  }
}

__device__ __forceinline__ uint4 load_grad(const MjpbrConvGrad& p, int64_t pix, int32_t ch) {
  return __ldg(reinterpret_cast<const uint4*>(p.grad_out + pix * p.c_out + ch));
}

__device__ __forceinline__ uint4 load_in(const MjpbrConvGrad& p, int32_t img, int32_t iy, int32_t ix, int32_t ch) {
  if (iy < 0 || iy >= p.height || ix < 0 || ix >= p.width) return make_uint4(0u, 0u, 0u, 0u);
  if (ch < p.c_in) {
    return __ldg(reinterpret_cast<const uint4*>(p.in + (((int64_t)img * p.height + iy) * p.width + ix) * p.c_in + ch));
  }
  const int32_t h2 = p.height >> 1, w2 = p.width >> 1;
  return __ldg(reinterpret_cast<const uint4*>(p.in2 + (((int64_t)img * h2 + (iy >> 1)) * w2 + (ix >> 1)) * p.c_in2 + (ch - p.c_in)));
}

__global__ void __launch_bounds__(kConvThreads, 2) conv3x3_wgrad_kernel(const __grid_constant__ MjpbrConvGrad p, const WgradGeom g) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_slot;
  const int32_t cout = p.c_out;
  uint8_t* sa = smem;                  // [pixel group 16][row group 16][8 rows] x 16 B
  uint8_t* sb = smem + 16 * 16 * 128;  // [pixel group 16][c_out / 8][8 rows] x 16 B
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int32_t P = g.pitch;
  const int32_t mrows = 9 * g.cin;
  const int32_t m0 = blockIdx.x * 128;
  const int32_t t0 = blockIdx.y * g.per_cta, t1 = min(t0 + g.per_cta, g.total);
  uint32_t ncols = 32;
  while (ncols < (uint32_t)cout) ncols <<= 1;
  if (warp == 0) umma::tmem_alloc(&tmem_slot, ncols);
  if (tid == 0) {
    umma::mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = umma::make_idesc_bf16(128, cout);
  bool ok = true;
  uint32_t phase = 0;
  for (int32_t t = t0; t < t1; ++t) {
    const int32_t img = t / g.tiles_per_img;
    const int32_t tl = t - img * g.tiles_per_img;
    const int32_t y0 = (tl / g.tiles_per_row) * g.rows, x0 = (tl % g.tiles_per_row) * P;
    // A: (row group, pixel group) jobs; a row group is 8 channels of one tap
    for (int32_t job = tid; job < 16 * 16; job += kConvThreads) {
      const int32_t rg = job & 15, q = job >> 4;
      const int32_t m = m0 + rg * 8;
      uint4 r[8], c[8];
      if (m < mrows) {
        const int32_t tap = m / g.cin, ch = m - tap * g.cin;
        const int32_t dy = tap / 3 - 1, dx = tap % 3 - 1;
#pragma unroll
        for (int32_t i = 0; i < 8; ++i) {
          const int32_t ip = q * 8 + i;
          r[i] = load_in(p, img, y0 + ip / P + dy, x0 + ip % P + dx, ch);
        }
        transpose8x8(r, c);
      } else {
#pragma unroll
        for (int32_t i = 0; i < 8; ++i) c[i] = make_uint4(0u, 0u, 0u, 0u);
      }
#pragma unroll
      for (int32_t k = 0; k < 8; ++k) *reinterpret_cast<uint4*>(sa + (q * 16 + rg) * 128 + k * 16) = c[k];
    }
    // B: grad_out transposed, (channel group, pixel group) jobs
    const int32_t cgroups = cout / 8;
    for (int32_t job = tid; job < cgroups * 16; job += kConvThreads) {
      const int32_t cg = job % cgroups, q = job / cgroups;
      uint4 r[8], c[8];
#pragma unroll
      for (int32_t i = 0; i < 8; ++i) {
        const int32_t ip = q * 8 + i;
        const int64_t pix = ((int64_t)img * p.height + y0 + ip / P) * p.width + x0 + ip % P;
        r[i] = load_grad(p, pix, cg * 8);
      }
      transpose8x8(r, c);
#pragma unroll
      for (int32_t k = 0; k < 8; ++k) *reinterpret_cast<uint4*>(sb + (q * cgroups + cg) * 128 + k * 16) = c[k];
    }
    umma::fence_async_shared();
    __syncthreads();
    umma::fence_after_sync();
    if (tid == 0) {
      const uint32_t a0 = umma::smem_addr(sa), b0 = umma::smem_addr(sb);
#pragma unroll 1
      for (int32_t s = 0; s < 8; ++s) {
        const uint64_t ad = umma::make_desc(a0 + s * 2 * 16 * 128, 16 * 128, 128);
        const uint64_t bd = umma::make_desc(b0 + s * 2 * cgroups * 128, cgroups * 128, 128);
        umma::mma_bf16(tmem, ad, bd, idesc, t > t0 || s > 0);
      }
      umma::commit(&bar);
    }
    ok = umma::mbar_wait(&bar, phase);
    phase ^= 1u;
    umma::fence_after_sync();
    __syncthreads();
    if (!ok) break;
  }
  if (ok && t1 > t0) {
    const int32_t m = m0 + warp * 32 + lane;
    const int32_t tap = m / g.cin, ch = m - tap * g.cin;
#pragma unroll 1
    for (int32_t c0 = 0; c0 < cout; c0 += 16) {
      float v[16];
      umma::tmem_load16(tmem + ((uint32_t)(warp * 32) << 16) + c0, v);
      if (m < mrows) {
#pragma unroll
        for (int32_t k = 0; k < 16; ++k) atomicAdd(p.grad_weight + ((int64_t)(c0 + k) * 9 + tap) * g.cin + ch, v[k]);
      }
    }
  } else if (!ok) {
    if (tid == 0 && p.error_word) atomicOr(p.error_word, kErrWaitTimeout);
    umma::mbar_wait(&bar, phase ^ 1u);
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) umma::tmem_free(tmem, ncols);
}

// grad_bias[co] += sum over pixels of grad_out[p][co]: one CTA per 1024 pixels, shared partial
// sums, one atomic per channel and CTA.
__global__ void __launch_bounds__(256) bias_grad_kernel(const uint16_t* __restrict__ grad_out, int64_t npix, int32_t cout,
                                                        float* __restrict__ grad_bias) {
  __shared__ float part[256];
  for (int32_t i = threadIdx.x; i < cout; i += blockDim.x) part[i] = 0.0f;
  __syncthreads();
  const int64_t p0 = (int64_t)blockIdx.x * 1024;
  const int64_t p1 = min(p0 + 1024, npix);
  const int32_t groups = cout / 8;
  for (int64_t i = p0 * groups + threadIdx.x; i < p1 * groups; i += blockDim.x) {
    const int64_t pix = i / groups;
    const int32_t cg = (int32_t)(i - pix * groups);
    const uint4 v = __ldg(reinterpret_cast<const uint4*>(grad_out + pix * cout + cg * 8));
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      atomicAdd(&part[cg * 8 + 2 * k], __uint_as_float(w[k] << 16));
      atomicAdd(&part[cg * 8 + 2 * k + 1], __uint_as_float(w[k] & 0xFFFF0000u));
    }
  }
  __syncthreads();
  for (int32_t i = threadIdx.x; i < cout; i += blockDim.x) atomicAdd(grad_bias + i, part[i]);
}

}  // namespace

int conv3x3_wgrad_launch(const MjpbrConvGrad& c, cudaStream_t stream) {
  if (!c.in || !c.grad_out || !c.grad_weight) return set_error(MJPBR_ERR_ARG, "conv3x3 wgrad: missing input, gradient or output");
  if (c.nimg < 1 || c.height < 1 || c.width < 1) return set_error(MJPBR_ERR_ARG, "conv3x3 wgrad: empty image batch");
  if (c.c_in < 16 || c.c_in % 16 || c.c_in2 < 0 || c.c_in2 % 16 || c.c_out < 16 || c.c_out % 16 || c.c_out > 256) {
    return set_error(MJPBR_ERR_ARG, "conv3x3 wgrad: channels must be multiples of 16 (c_out <= 256), got %d + %d -> %d", c.c_in,
                     c.c_in2, c.c_out);
  }
  if (c.c_in2 > 0 && (!c.in2 || c.height % 2 || c.width % 2)) return set_error(MJPBR_ERR_ARG, "conv3x3 wgrad: in2 needs even sizes");
  const int32_t w = c.width;
  const bool row_ok = (w >= 128) ? (w % 128 == 0) : (w >= 16 && 128 % w == 0);
  if (!row_ok) return set_error(MJPBR_ERR_ARG, "conv3x3 wgrad: width %d is not a power of two in [16, 128] or a multiple of 128", w);
  WgradGeom g;
  g.pitch = std::min(w, 128);
  g.rows = 128 / g.pitch;
  if (c.height % g.rows) return set_error(MJPBR_ERR_ARG, "conv3x3 wgrad: height %d is not a multiple of %d", c.height, g.rows);
  if (!aligned16(c.in) || !aligned16(c.in2) || !aligned16(c.grad_out)) return set_error(MJPBR_ERR_ARG, "conv3x3 wgrad: tensors must be 16-byte aligned");
  g.tiles_per_row = w / g.pitch;
  g.tiles_per_img = (c.height / g.rows) * g.tiles_per_row;
  g.cin = c.c_in + c.c_in2;
  const int64_t total = (int64_t)c.nimg * g.tiles_per_img;
  if (total > INT32_MAX) return set_error(MJPBR_ERR_ARG, "conv3x3 wgrad: too many tiles");
  g.total = (int32_t)total;
  g.per_cta = c.tiles_per_cta > 0 ? c.tiles_per_cta : 64;
  const int32_t mblocks = (9 * g.cin + 127) / 128;
  const int32_t splits = (g.total + g.per_cta - 1) / g.per_cta;
  if (splits > 65535) return set_error(MJPBR_ERR_ARG, "conv3x3 wgrad: %d tile runs exceed the grid; raise tiles_per_cta", splits);
  const size_t smem = (size_t)16 * 16 * 128 + (size_t)16 * c.c_out * 16;
  static size_t smem_set = 0;
  if (smem > smem_set) {
    cudaError_t e = cudaFuncSetAttribute(conv3x3_wgrad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return set_error(MJPBR_ERR_CUDA, "conv3x3 wgrad: %zu bytes of shared memory: %s", smem, cudaGetErrorString(e));
    smem_set = smem;
  }
  conv3x3_wgrad_kernel<<<dim3(mblocks, splits), kConvThreads, smem, stream>>>(c, g);
  if (int rc = check_launch("conv3x3_wgrad_kernel")) return rc;
  if (c.grad_bias) {
    const int64_t npix = (int64_t)c.nimg * c.height * c.width;
    bias_grad_kernel<<<(unsigned)((npix + 1023) / 1024), 256, 0, stream>>>(c.grad_out, npix, c.c_out, c.grad_bias);
    return check_launch("bias_grad_kernel");
  }
  return MJPBR_OK;
}

}  // namespace mjpbr
