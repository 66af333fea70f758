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
