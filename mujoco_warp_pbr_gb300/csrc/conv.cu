// 3x3 convolutions of the learned denoiser as implicit GEMMs on the 5th-generation tensor cores.
//
// A tile is 128 output pixels (a run of one image row, or 128 / width whole rows) times all
// output channels: D (128 x c_out, FP32 in tensor memory) = sum over the 9 taps and the input
// channels of A_tap (128 x c_in) * W_tap^T, 16 input channels (one K = 16 MMA) at a time. The
// input rows of a tile plus a one-row halo above and below are staged in shared memory in the
// K-major core-matrix layout (8 pixels x 16 bytes), so that the A operand of tap (dy, dx) is one
// descriptor with a uniform 16-byte row stride.
//
// conv3x3_ws_kernel (the default, further below) is a persistent warp-specialised kernel whose
// operands arrive by TMA. conv3x3_kernel, directly below, is the first version: one CTA per tile
// staging three dx-shifted copies of its rows with plain loads (MJPBR_CONV_PIPELINE=0 selects it,
// as do batches of more than 2^31 pixels).
//
// The U-Net's skip concatenation is read in place: channels past c_in come from in2, either at
// the output resolution (in2_full) or at half of it, upsampled x2 (nearest) while staging.
//
// Weight gradients: conv3x3_wgrad_ws_kernel (persistent, warp-specialised, MN-major TMA operands,
// three MMA-issuing warps) for full-resolution skips, else conv3x3_wgrad_kernel (one CTA per 128
// rows of (tap, channel), register transposes into K-major operands); bias gradients by
// bias_grad_kernel.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <climits>
#include <cstdlib>
#include <cstring>

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
  if (p.in2_full) return __ldg(reinterpret_cast<const uint4*>(p.in2 + (((int64_t)img * p.height + iy) * p.width + ix) * p.c_in2 + (ch - p.c_in)));
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

// ---- warp-specialised variant: persistent CTAs of six warps. Warp 4 loads operands with the
// tensor memory accelerator (TMA) into up to kMaxStages stage buffers, warp 5 issues the MMAs,
// warps 0-3 run the epilogue; two accumulators in tensor memory let a tile's epilogue overlap
// the next tile's MMAs. The roles hand over through mbarriers:
//   full[s]   the TMA loads of the stage in buffer s landed (expect-tx arrival by the loader)
//   ready[s]  the loader is done with it: at once, or after upsampling a half-resolution in2
//             into its planes (one arrival; the MMA warp waits on full[s] and ready[s])
//   empty[s]  its MMAs completed (tcgen05.commit)
//   acc_full[b] / acc_empty[b]  accumulator b holds a finished tile / was read (128 arrivals)
//
// Operand layout of a stage (G 16-channel chunks): one 5-D TMA box per copy covering all 2G
// channel groups, so each group is a plane of (rows + 2) x spitch pixels x 16 bytes. A tile of
// one image row (width >= 128) is staged once with its halo columns (spitch = pitch + 2) and the
// dx shift of a tap is a one-pixel (16-byte) offset of the A descriptor; tiles of several short
// rows stage three dx-shifted copies (spitch = pitch), since a shifted start would wrap from one
// image row into the next. Outside the image the TMA reads zeros. A stage holds chunks of `in`
// or of the half-resolution in2, which is loaded as one box per stage covering the tile's
// footprint and upsampled x2 (nearest) into the planes by the loader warp; a full-resolution in2
// (in2_full) is staged like `in`.
//
// Weights are resident (one TMA box of all taps and channel groups) when they fit, else loaded
// per stage. Every wait is bounded; a wait that gives up raises the CTA's abort flag, which ends
// the other roles' loops, and the error word records kErrWaitTimeout.

constexpr int kWsThreads = 192;
constexpr int kMaxStages = 4;
constexpr int kMaxSlots = 8;  // row-ring slots

struct WsGeom {
  ConvGeom g;
  int32_t ntiles;
  int32_t single;    // tile = (part of) one image row: one staged copy with halo columns
  int32_t spitch;    // staged pixels per row
  int32_t plane;     // bytes of one channel-group plane: (rows + 2) x spitch x 16
  int32_t group;     // 16-channel chunks per stage (G)
  int32_t abuf;      // bytes of one stage's A region: copies x 2G planes (multiple of 128)
  int32_t s2w, s2h;  // in2 box: pixels, rows
  int32_t s2plane;   // bytes of one in2 group plane
  int32_t s2buf;     // bytes of one stage's in2 boxes (multiple of 128); 0 without in2
  int32_t bstage;    // bytes of one stage's weights; 0 when resident
  int32_t resident;  // weights resident: 9 x (cin / 8) x c_out x 16 bytes at b_off
  int32_t s2_off, b_off;
  int32_t nstage;
  int32_t acc_cols;  // tensor-memory columns of one accumulator
  // row ring (tiles of one image row, resident weights): each CTA takes a contiguous range of
  // tiles ordered down the image columns and loads every input row once into a ring of nslot
  // slots of 2 x (c_in + c_in2) / 16 planes of (pitch + 2) pixels
  int32_t ring;
  int32_t nslot;
  int32_t slot_bytes;
  int32_t rowplane;  // bytes of one row plane: (pitch + 2) x 16
  int32_t in2_off;   // offset of the in2 planes in a slot (a multiple of 128)
};

// The i-th tile of this CTA: strided over the grid, or (ring) the i-th of a contiguous range in
// column-major order (image, tile column, row). False past the CTA's last tile.
__device__ __forceinline__ bool cta_tile(const WsGeom& wg, int32_t i, int32_t& img, int32_t& y0, int32_t& x0) {
  const ConvGeom& g = wg.g;
  if (wg.ring) {
    const int32_t t = (int32_t)((int64_t)blockIdx.x * wg.ntiles / gridDim.x) + i;
    if (t >= (int32_t)((int64_t)(blockIdx.x + 1) * wg.ntiles / gridDim.x)) return false;
    const int32_t h = g.tiles_per_img / g.tiles_per_row;  // image rows
    const int32_t col = t / h;
    y0 = t - col * h;
    img = col / g.tiles_per_row;
    x0 = (col - img * g.tiles_per_row) * g.pitch;
    return true;
  }
  const int32_t tile = blockIdx.x + i * gridDim.x;
  if (tile >= wg.ntiles) return false;
  img = tile / g.tiles_per_img;
  const int32_t t = tile - img * g.tiles_per_img;
  y0 = (t / g.tiles_per_row) * g.rows;
  x0 = (t % g.tiles_per_row) * g.pitch;
  return true;
}

struct StageInfo {
  int32_t in2;  // chunks of in2 (else of in)
  int32_t cs;   // first chunk, in chunks of the concatenated input
  int32_t nc;   // chunks
};

__device__ __forceinline__ StageInfo stage_info(int32_t s, int32_t nci, int32_t nchunk, int32_t G) {
  const int32_t nsp_in = (nci + G - 1) / G;
  StageInfo st;
  st.in2 = s >= nsp_in;
  st.cs = st.in2 ? nci + (s - nsp_in) * G : s * G;
  st.nc = min(G, (st.in2 ? nchunk : nci) - st.cs);
  return st;
}

// Bounded wait that also gives up once another role raised the abort flag. Waiters off the MMA
// issue path sleep `backoff_ns` between polls, so that polling warps leave the SM's issue slots
// and memory pipeline to the MMA and copy instructions.
__device__ __forceinline__ bool ws_wait(uint64_t* bar, uint32_t parity, volatile int32_t* abort_flag, uint32_t backoff_ns = 0,
                                        uint32_t limit = umma::kWaitLimit) {
  for (uint32_t i = 0; i < limit; ++i) {
    if (umma::mbar_try_wait(bar, parity)) return true;
    if ((i & 255u) == 255u && *abort_flag) return false;
    if (backoff_ns) __nanosleep(backoff_ns);
  }
  *abort_flag = 1;
  return false;
}

constexpr uint32_t kLoaderBackoffNs = 256, kEpilogueBackoffNs = 128;

__device__ __forceinline__ void tile_origin(const ConvGeom& g, int32_t tile, int32_t& img, int32_t& y0, int32_t& x0) {
  img = tile / g.tiles_per_img;
  const int32_t t = tile - img * g.tiles_per_img;
  y0 = (t / g.tiles_per_row) * g.rows;
  x0 = (t % g.tiles_per_row) * g.pitch;
}

// Upsamples the in2 boxes of one stage (2 nc group planes; rows from (y0 - 1) >> 1, pixels from
// x0 / 2 - 1) into its operand planes: staged row j, pixel xs holds input (y0 - 1 + j,
// x0 + xs - 1) of the single copy, or (y0 - 1 + j, x + dx - 1) of copy dx at x.
__device__ __forceinline__ void ws_expand(const WsGeom& wg, uint8_t* smem, int32_t buf, int32_t nc, int32_t y0, int32_t lane) {
  const int32_t P = wg.g.pitch, R = wg.g.rows;
  const int32_t r0 = (y0 - 1) >> 1;
  const uint8_t* src0 = smem + wg.s2_off + buf * wg.s2buf;
  uint8_t* dst0 = smem + buf * wg.abuf;
  if (wg.single) {
    const int32_t hw = P + 2;
    const int32_t n = 2 * nc * 3 * hw;
    for (int32_t e = lane; e < n; e += 32) {
      const int32_t pl = e / (3 * hw);
      const int32_t r = e - pl * 3 * hw;
      const int32_t j = r / hw, xs = r - j * hw;
      const int32_t sr = ((y0 - 1 + j) >> 1) - r0, sc = (xs + 1) >> 1;
      *reinterpret_cast<uint4*>(dst0 + pl * wg.plane + (j * hw + xs) * 16) =
          *reinterpret_cast<const uint4*>(src0 + pl * wg.s2plane + (sr * wg.s2w + sc) * 16);
    }
  } else {
    const int32_t per_plane = (R + 2) * P;
    const int32_t n = 3 * 2 * nc * per_plane;
    const int32_t copy_stride = 2 * wg.group * wg.plane;
    for (int32_t e = lane; e < n; e += 32) {
      const int32_t dx = e / (2 * nc * per_plane);
      const int32_t r1 = e - dx * 2 * nc * per_plane;
      const int32_t pl = r1 / per_plane;
      const int32_t r = r1 - pl * per_plane;
      const int32_t j = r / P, x = r - j * P;
      const int32_t sr = ((y0 - 1 + j) >> 1) - r0, sc = (x + dx + 1) >> 1;
      *reinterpret_cast<uint4*>(dst0 + dx * copy_stride + pl * wg.plane + (j * P + x) * 16) =
          *reinterpret_cast<const uint4*>(src0 + pl * wg.s2plane + (sr * wg.s2w + sc) * 16);
    }
  }
}

__global__ void __launch_bounds__(kWsThreads, 1) conv3x3_ws_kernel(const __grid_constant__ MjpbrConv p, const __grid_constant__ WsGeom wg,
                                                                   const __grid_constant__ CUtensorMap tm_in, const __grid_constant__ CUtensorMap tm_in2,
                                                                   const __grid_constant__ CUtensorMap tm_w) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t full[kMaxSlots], ready[kMaxSlots], empty[kMaxSlots];
  __shared__ uint64_t acc_full[2], acc_empty[2], wbar, drain;
  __shared__ uint32_t tmem_slot;
  __shared__ int32_t abort_flag;
  const ConvGeom& g = wg.g;
  const int32_t cout = p.c_out;
  const int32_t nchunk = g.cin / 16;
  const int32_t nci = p.c_in / 16;
  const int32_t G = wg.group;
  const int32_t nsp = (nci + G - 1) / G + (nchunk - nci + G - 1) / G;  // stages per tile
  const int32_t nst = wg.nstage;
  const uint32_t s0 = umma::smem_addr(smem);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t ncols = 2u * (uint32_t)wg.acc_cols;
  if (warp == 0) umma::tmem_alloc(&tmem_slot, ncols);
  if (tid == 128) {
    for (int i = 0; i < (wg.ring ? wg.nslot : nst); ++i) {
      umma::mbar_init(&full[i], 1);
      umma::mbar_init(&ready[i], 1);
      umma::mbar_init(&empty[i], 1);
    }
    for (int i = 0; i < 2; ++i) {
      umma::mbar_init(&acc_full[i], 1);
      umma::mbar_init(&acc_empty[i], kTilePx);
    }
    umma::mbar_init(&wbar, 1);
    umma::mbar_init(&drain, 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tm_in)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tm_w)) : "memory");
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  volatile int32_t* abort_v = &abort_flag;
  bool ok = true;

  if (warp == 4) {
    // ---- loader: TMA loads of stage k, then the in2 upsampling of stage k - 1 ----
    const uint32_t in_box = (uint32_t)(16 * wg.spitch * (g.rows + 2) * 2 * G);
    const uint32_t in2_box = (uint32_t)(16 * wg.s2w * wg.s2h * 2 * G);
    const uint32_t copies = wg.single ? 1u : 3u;
    if (wg.resident && lane == 0) {
      umma::mbar_arrive_expect_tx(&wbar, (uint32_t)(9 * 2 * nchunk * cout * 16));
      umma::tma_load_4d(s0 + wg.b_off, &tm_w, &wbar, 0, 0, 0, 0);
    }
    int32_t k = 0, issued = 0, prev_in2 = 0, prev_nc = 0, prev_y0 = 0;
    if (wg.ring) {
      // one load per input row: the rows of a run of tiles down one tile column plus the
      // halo rows above and below (outside the image the TMA reads zeros)
      const uint32_t row_bytes = (uint32_t)(16 * wg.spitch * 2 * nchunk);
      int32_t i = 0, img, y0, x0;
      while (lane == 0 && ok && cta_tile(wg, i, img, y0, x0)) {
        int32_t n = 1, img2, y2, x2;
        while (cta_tile(wg, i + n, img2, y2, x2) && img2 == img && x2 == x0) ++n;
        for (int32_t r = y0 - 1; r <= y0 + n && ok; ++r, ++k) {
          const int32_t slot = k % wg.nslot;
          if (k >= wg.nslot) ok = ws_wait(&empty[slot], ((k / wg.nslot) + 1) & 1, abort_v, kLoaderBackoffNs);
          if (!ok) break;
          const uint32_t sa = s0 + slot * wg.slot_bytes;
          umma::mbar_arrive_expect_tx(&full[slot], row_bytes);
          umma::tma_load_5d(sa, &tm_in, &full[slot], 0, x0 - 1, r, 0, img);
          if (p.c_in2 > 0) umma::tma_load_5d(sa + wg.in2_off, &tm_in2, &full[slot], 0, x0 - 1, r, 0, img);
          issued = k + 1;
        }
        i += n;
      }
    }
    for (int32_t tile = wg.ring ? wg.ntiles : blockIdx.x; tile < wg.ntiles && ok; tile += gridDim.x) {
      int32_t img, y0, x0;
      tile_origin(g, tile, img, y0, x0);
      for (int32_t sidx = 0; sidx < nsp && ok; ++sidx, ++k) {
        const StageInfo st = stage_info(sidx, nci, nchunk, G);
        const int32_t buf = k % nst;
        if (k >= nst) ok = ws_wait(&empty[buf], ((k / nst) + 1) & 1, abort_v, kLoaderBackoffNs);
        if (!ok) break;
        if (lane == 0) {
          const uint32_t abase = s0 + buf * wg.abuf;
          const bool half = st.in2 && !p.in2_full;  // in2 box, upsampled below
          uint32_t bytes = half ? in2_box : copies * in_box;
          if (!wg.resident) bytes += (uint32_t)wg.bstage;
          umma::mbar_arrive_expect_tx(&full[buf], bytes);
          // a full-resolution in2 is staged like `in`, from its own tensor map
          const CUtensorMap* src = st.in2 ? &tm_in2 : &tm_in;
          const int32_t grp0 = 2 * (st.in2 ? st.cs - nci : st.cs);
          if (half) {
            umma::tma_load_5d(s0 + wg.s2_off + buf * wg.s2buf, &tm_in2, &full[buf], 0, x0 / 2 - 1, (y0 - 1) >> 1, grp0, img);
          } else if (wg.single) {
            umma::tma_load_5d(abase, src, &full[buf], 0, x0 - 1, y0 - 1, grp0, img);
          } else {
            for (int32_t dx = 0; dx < 3; ++dx) umma::tma_load_5d(abase + dx * 2 * G * wg.plane, src, &full[buf], 0, x0 - 1 + dx, y0 - 1, grp0, img);
          }
          if (!wg.resident) umma::tma_load_4d(s0 + wg.b_off + buf * wg.bstage, &tm_w, &full[buf], 0, 0, 2 * st.cs, 0);
        }
        issued = k + 1;
        const bool half = st.in2 && !p.in2_full;
        // stage k is ready once its loads land (the MMA warp waits on full[] too), unless its
        // half-resolution in2 must be upsampled first
        if (!half && lane == 0) umma::mbar_arrive(&ready[buf]);
        if (k >= 1 && prev_in2) {
          // stage k - 1: upsample its in2 once it landed
          const int32_t pb = (k - 1) % nst;
          ok = ws_wait(&full[pb], ((k - 1) / nst) & 1, abort_v);
          if (!ok) break;
          ws_expand(wg, smem, pb, prev_nc, prev_y0, lane);
          umma::fence_async_shared();
          __syncwarp();
          if (lane == 0) umma::mbar_arrive(&ready[pb]);
        }
        prev_in2 = half;
        prev_nc = st.nc;
        prev_y0 = y0;
      }
    }
    if (ok && k >= 1 && prev_in2) {
      const int32_t pb = (k - 1) % nst;
      ok = ws_wait(&full[pb], ((k - 1) / nst) & 1, abort_v);
      if (ok) {
        ws_expand(wg, smem, pb, prev_nc, prev_y0, lane);
        umma::fence_async_shared();
        __syncwarp();
        if (lane == 0) umma::mbar_arrive(&ready[pb]);
      }
    }
    if (!ok && lane == 0) {
      // the copies in flight land before the CTA's shared memory is released
      const int32_t nb = wg.ring ? wg.nslot : nst;
      for (int32_t kk = max(0, issued - nb); kk < issued; ++kk) umma::mbar_wait(&full[kk % nb], (kk / nb) & 1);
    }
  } else if (warp == 5) {
    // ---- MMA issuer ----
    if (lane == 0) {
      const uint32_t idesc = umma::make_idesc_bf16(kTilePx, cout);
      const uint32_t dy16 = (uint32_t)wg.spitch;
      const uint32_t dx16 = wg.single ? 1u : (uint32_t)(2 * G * wg.plane) >> 4;
      const uint32_t achunk16 = (uint32_t)(2 * wg.plane) >> 4;
      const uint32_t btap16 = (uint32_t)((wg.resident ? 2 * nchunk : 2 * G) * cout);
      const uint32_t bchunk16 = (uint32_t)(2 * cout);
      if (wg.resident) ok = ws_wait(&wbar, 0, abort_v);
      int32_t k = 0, i = 0, last = -1;
      if (wg.ring) {
        // tile row y of a run uses the ring rows y - 1, y, y + 1 (loads base + j, j = y - y_run
        // + dy); a row is released after its last tile: row y - 1 after tile y, and the run's last
        // two rows after its last tile
        const uint64_t b_all = umma::make_desc(s0 + wg.b_off, cout * 16, 128);
        const uint32_t plane16 = (uint32_t)wg.rowplane >> 4;
        int32_t base = 0, waited = 0, img, y0, x0;
        while (ok && cta_tile(wg, i, img, y0, x0)) {
          int32_t n = 1, img2, y2, x2;
          while (cta_tile(wg, i + n, img2, y2, x2) && img2 == img && x2 == x0) ++n;
          for (int32_t j = 0; j < n && ok; ++j, ++i) {
            const int32_t b = i & 1;
            if (i >= 2) ok = ws_wait(&acc_empty[b], ((i >> 1) + 1) & 1, abort_v);
            while (ok && waited <= base + j + 2) {
              ok = ws_wait(&full[waited % wg.nslot], (waited / wg.nslot) & 1, abort_v);
              ++waited;
            }
            if (!ok) break;
            umma::fence_after_sync();
            const uint32_t acc = tmem + (uint32_t)(b * wg.acc_cols);
            for (int32_t dy = 0; dy < 3; ++dy) {
              const uint32_t slot_addr = s0 + ((base + j + dy) % wg.nslot) * wg.slot_bytes;
              const uint64_t a_row = umma::make_desc(slot_addr, wg.rowplane, 128);
              const uint64_t a_in2 = umma::make_desc(slot_addr + wg.in2_off, wg.rowplane, 128);
              for (int32_t cc = 0; cc < nchunk; ++cc) {
                const uint64_t ad = cc < nci ? a_row + 2 * cc * plane16 : a_in2 + 2 * (cc - nci) * plane16;
                const uint64_t bd = b_all + cc * bchunk16;
#pragma unroll
                for (int32_t dx = 0; dx < 3; ++dx) {
                  umma::mma_bf16(acc, ad + dx, bd + (dy * 3 + dx) * btap16, idesc, dy > 0 || cc > 0 || dx > 0);
                }
              }
            }
            umma::commit(&empty[(base + j) % wg.nslot]);
            last = (base + j) % wg.nslot;
            if (j == n - 1) {
              umma::commit(&empty[(base + j + 1) % wg.nslot]);
              umma::commit(&empty[(base + j + 2) % wg.nslot]);
            }
            umma::commit(&acc_full[b]);
          }
          base += n + 2;
        }
        k = waited;
      }
      for (int32_t tile = wg.ring ? wg.ntiles : blockIdx.x; tile < wg.ntiles && ok; tile += gridDim.x, ++i) {
        const int32_t b = i & 1;
        if (i >= 2) ok = ws_wait(&acc_empty[b], ((i >> 1) + 1) & 1, abort_v);
        if (!ok) break;
        umma::fence_after_sync();
        const uint32_t acc = tmem + (uint32_t)(b * wg.acc_cols);
        for (int32_t sidx = 0; sidx < nsp; ++sidx, ++k) {
          const StageInfo st = stage_info(sidx, nci, nchunk, G);
          const int32_t buf = k % nst;
          ok = ws_wait(&full[buf], (k / nst) & 1, abort_v) && ws_wait(&ready[buf], (k / nst) & 1, abort_v);
          if (!ok) break;
          umma::fence_after_sync();
          const uint64_t a_stage = umma::make_desc(s0 + buf * wg.abuf, wg.plane, 128);
          const uint64_t b_stage = wg.resident ? umma::make_desc(s0 + wg.b_off, cout * 16, 128) + (uint64_t)(st.cs * bchunk16)
                                               : umma::make_desc(s0 + wg.b_off + buf * wg.bstage, cout * 16, 128);
          for (int32_t cc = 0; cc < st.nc; ++cc) {
            const uint64_t ad = a_stage + cc * achunk16;
            const uint64_t bd = b_stage + cc * bchunk16;
#pragma unroll
            for (int32_t tap = 0; tap < 9; ++tap) {
              const uint32_t dy = tap / 3, dx = tap % 3;
              umma::mma_bf16(acc, ad + dy * dy16 + dx * dx16, bd + tap * btap16, idesc, sidx > 0 || cc > 0 || tap > 0);
            }
          }
          umma::commit(&empty[buf]);
          last = buf;
        }
        if (!ok) break;
        umma::commit(&acc_full[b]);
      }
      if (!ok && last >= 0) {
        // the MMAs in flight complete before their operands and accumulators are released
        umma::commit(&drain);
        umma::mbar_wait(&drain, 0);
      }
    }
  } else {
    // ---- epilogue: warp w reads accumulator rows (pixels) 32 w .. 32 w + 31 ----
    const int32_t m = tid;
    int32_t img, y0, x0;
    for (int32_t i = 0; cta_tile(wg, i, img, y0, x0); ++i) {
      const int32_t b = i & 1;
      ok = ws_wait(&acc_full[b], (i >> 1) & 1, abort_v, kEpilogueBackoffNs);
      // tcgen05.ld is warp-collective
      if (!__all_sync(0xFFFFFFFFu, ok)) {
        ok = false;
        *abort_v = 1;
        break;
      }
      umma::fence_after_sync();
      const int64_t pix = ((int64_t)img * p.height + y0 + m / g.pitch) * p.width + x0 + m % g.pitch;
      const uint32_t acc = tmem + (uint32_t)(b * wg.acc_cols) + ((uint32_t)(warp * 32) << 16);
#pragma unroll 1
      for (int32_t c0 = 0; c0 < cout; c0 += 16) {
        float v[16];
        umma::tmem_load16(acc + c0, v);
        if (c0 + 16 >= cout) {
          // the accumulator is free for tile i + 2 once every thread has read its rows
          umma::fence_before_sync();
          umma::mbar_arrive(&acc_empty[b]);
        }
        if (p.bias) {
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] += __ldg(p.bias + c0 + j);
        }
        if (p.relu) {
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] = fmaxf(v[j], 0.0f);
        }
        if (p.mask) {
          const uint4* mk = reinterpret_cast<const uint4*>(p.mask + pix * cout + c0);
          const uint4 m0 = __ldg(mk), m1 = __ldg(mk + 1);
          const uint32_t wv[8] = {m0.x, m0.y, m0.z, m0.w, m1.x, m1.y, m1.z, m1.w};
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            if ((wv[j] & 0x8000u) || !(wv[j] & 0x7FFFu)) v[2 * j] = 0.0f;
            if ((wv[j] & 0x80000000u) || !(wv[j] & 0x7FFF0000u)) v[2 * j + 1] = 0.0f;
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
          for (int j = 0; j < 4; ++j) o[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
        }
      }
    }
  }
  if (!ok && tid % 32 == 0 && p.error_word) atomicOr(p.error_word, kErrWaitTimeout);
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) umma::tmem_free(tmem, ncols);
}

bool aligned16(const void* q) { return (reinterpret_cast<uintptr_t>(q) & 15u) == 0; }

}  // namespace

namespace {

// shared memory of one CTA of the pipelined kernel: two CTAs per SM
#ifndef MJPBR_CONV_SMEM_BUDGET
#define MJPBR_CONV_SMEM_BUDGET (110 * 1024)
#endif
constexpr size_t kPipeSmemBudget = MJPBR_CONV_SMEM_BUDGET;
// One CTA per SM with most of the shared memory: measured faster for the layers of 16-pixel rows and
// the 64-pixel-row layers of 96 or more input channels (their staged pipeline then holds bigger
// stages), slower for every other layer shape of the denoiser.
constexpr size_t kPipeSmemWide = 200 * 1024;

size_t pipe_budget(int32_t width, int32_t cin) {
  return (width <= 16 || (width == 64 && cin >= 96)) ? kPipeSmemWide : kPipeSmemBudget;
}
constexpr size_t kPipeSmemMax = 220 * 1024;
int conv_sm_count() { return device_sm_count(); }

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                   const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess && q == cudaDriverEntryPointSuccess) {
      fn = reinterpret_cast<EncodeTiledFn>(f);
    }
  }
  return fn;
}

int encode(CUtensorMap* m, const void* base, cuuint32_t rank, const cuuint64_t* dims, const cuuint64_t* strides, const cuuint32_t* box) {
  EncodeTiledFn fn = encode_tiled();
  if (!fn) return set_error(MJPBR_ERR_CUDA, "conv3x3: cuTensorMapEncodeTiled is unavailable");
  const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
  const CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, rank, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(MJPBR_ERR_CUDA, "conv3x3: cuTensorMapEncodeTiled failed (%d)", (int)r);
  return 0;
}

// Tensor map of a BF16 NHWC activation as 5-D (8 channels, pixel, row, channel group, image):
// the channel-group dimension (stride 16 bytes) is outside the pixel dimensions, so one box of
// groups x 8 channels x bw pixels x bh rows lands as `groups` planes of bh x bw x 16 bytes. Reads
// outside the tensor return zeros.
int make_act_map(CUtensorMap* m, const void* base, int32_t ch, int32_t w, int32_t h, int32_t n, int32_t bw, int32_t bh, int32_t groups) {
  const cuuint64_t dims[5] = {8, (cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)(ch / 8), (cuuint64_t)n};
  const cuuint64_t strides[4] = {(cuuint64_t)ch * 2, (cuuint64_t)w * ch * 2, 16, (cuuint64_t)h * w * ch * 2};
  const cuuint32_t box[5] = {8, (cuuint32_t)bw, (cuuint32_t)bh, (cuuint32_t)groups, 1};
  return encode(m, base, 5, dims, strides, box);
}

// Tensor map of the weights [c_out][9 taps][cin] as 4-D (8 channels, output channel, channel
// group, tap): a box of `groups` channel groups lands as [tap][group][c_out] x 16 bytes, the
// K-major B operand of every tap.
int make_weight_map(CUtensorMap* m, const void* base, int32_t cin, int32_t cout, int32_t groups) {
  const cuuint64_t dims[4] = {8, (cuuint64_t)cout, (cuuint64_t)(cin / 8), 9};
  const cuuint64_t strides[3] = {(cuuint64_t)9 * cin * 2, 16, (cuuint64_t)cin * 2};
  const cuuint32_t box[4] = {8, (cuuint32_t)cout, (cuuint32_t)groups, 9};
  return encode(m, base, 4, dims, strides, box);
}

// MJPBR_CONV_RING=0 keeps single-row tiles on the staged pipeline (kept for comparison).
bool conv_ring_enabled() {
  static int enabled = -1;
  if (enabled < 0) {
    const char* v = getenv("MJPBR_CONV_RING");
    enabled = (v && v[0] == '0') ? 0 : 1;
  }
  return enabled == 1;
}

// MJPBR_CONV_PIPELINE=0 selects the one-tile-per-CTA kernel (kept for comparison).
bool conv_pipeline_enabled() {
  static int enabled = -1;
  if (enabled < 0) {
    const char* v = getenv("MJPBR_CONV_PIPELINE");
    enabled = (v && v[0] == '0') ? 0 : 1;
  }
  return enabled == 1;
}

}  // namespace

int conv3x3_launch(const MjpbrConv& c, cudaStream_t stream) {
  if (!c.in || !c.weight || (!c.out && !c.out_f32)) return set_error(MJPBR_ERR_ARG, "conv3x3: missing input, weight or output");
  if (c.nimg < 1 || c.height < 1 || c.width < 1) return set_error(MJPBR_ERR_ARG, "conv3x3: empty image batch");
  if (c.c_in < 16 || c.c_in % 16 || c.c_in2 < 0 || c.c_in2 % 16 || c.c_out < 16 || c.c_out % 16 || c.c_out > 256) {
    return set_error(MJPBR_ERR_ARG, "conv3x3: channels must be multiples of 16 (c_out <= 256), got %d + %d -> %d", c.c_in, c.c_in2,
                     c.c_out);
  }
  if (c.c_in2 > 0 && !c.in2) return set_error(MJPBR_ERR_ARG, "conv3x3: c_in2 > 0 needs in2");
  if (c.c_in2 > 0 && !c.in2_full && (c.height % 2 || c.width % 2)) return set_error(MJPBR_ERR_ARG, "conv3x3: a half-resolution in2 needs even sizes");
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
  if (conv_pipeline_enabled() && (int64_t)c.nimg * c.height * c.width <= INT32_MAX) {
    // warp-specialised persistent variant (32-bit pixel indices)
    WsGeom wg;
    wg.g = g;
    wg.ntiles = (int32_t)tiles;
    wg.single = g.rows == 1;
    wg.spitch = wg.single ? g.pitch + 2 : g.pitch;
    wg.plane = (g.rows + 2) * wg.spitch * 16;
    wg.s2w = g.pitch / 2 + 2;
    wg.s2h = wg.single ? 2 : g.rows / 2 + 2;
    wg.s2plane = wg.s2w * wg.s2h * 16;
    int acc_cols = 32;
    while (acc_cols < c.c_out) acc_cols <<= 1;
    wg.acc_cols = acc_cols;
    const int32_t nchunk = g.cin / 16, nci = c.c_in / 16;
    const int32_t copies = wg.single ? 1 : 3;
    auto round128 = [](size_t v) { return (v + 127) / 128 * 128; };
    const bool half_in2 = c.c_in2 > 0 && !c.in2_full;
    const size_t wbytes = (size_t)9 * 2 * nchunk * c.c_out * 16;
    auto stage_bytes = [&](int32_t G, bool resident) {
      size_t b = round128((size_t)copies * 2 * G * wg.plane);
      if (half_in2) b += round128((size_t)2 * G * wg.s2plane);
      if (!resident) b += (size_t)9 * 2 * G * c.c_out * 16;
      return b;
    };
    // resident weights when they fit beside two one-chunk stages; then the largest stage (in
    // chunks) of which two fit, then as many stages as fit (at most kMaxStages)
    const size_t budget = pipe_budget(w, g.cin);
    const bool resident = wbytes + 2 * stage_bytes(1, true) <= budget;
    const size_t fixed = resident ? wbytes : 0;
    const int32_t gmax = std::max(nci, nchunk - nci);
    int32_t G = 1;
    while (G < gmax && fixed + 2 * stage_bytes(G + 1, resident) <= budget) ++G;
    int32_t nst = 2;
    while (nst < kMaxStages && fixed + (nst + 1) * stage_bytes(G, resident) <= budget) ++nst;
    wg.group = G;
    wg.nstage = nst;
    wg.resident = resident;
    // the row ring, when tiles are single rows, the skip input (if any) has full resolution and
    // the weights plus at least four row slots fit
    wg.rowplane = wg.spitch * 16;
    wg.in2_off = (int32_t)round128((size_t)2 * nci * wg.rowplane);
    wg.slot_bytes = (int32_t)round128((size_t)wg.in2_off + (size_t)2 * (nchunk - nci) * wg.rowplane);
    wg.nslot = (int32_t)std::min<size_t>(kMaxSlots, budget > wbytes ? (budget - wbytes) / wg.slot_bytes : 0);
    wg.ring = conv_ring_enabled() && wg.single && (c.c_in2 == 0 || c.in2_full) && wg.nslot >= 4;
    wg.abuf = (int32_t)round128((size_t)copies * 2 * G * wg.plane);
    wg.s2buf = half_in2 ? (int32_t)round128((size_t)2 * G * wg.s2plane) : 0;
    wg.bstage = resident ? 0 : 9 * 2 * G * c.c_out * 16;
    wg.s2_off = nst * wg.abuf;
    wg.b_off = wg.s2_off + nst * wg.s2buf;
    if (wg.ring) {
      wg.resident = 1;
      wg.b_off = wg.nslot * wg.slot_bytes;
    }
    const size_t smem = wg.ring ? (size_t)wg.b_off + wbytes : fixed + (size_t)nst * stage_bytes(G, resident);
    if (smem > kPipeSmemMax) return set_error(MJPBR_ERR_ARG, "conv3x3: %zu bytes of shared memory needed", smem);
    if (int rc = ensure_smem(reinterpret_cast<const void*>(conv3x3_ws_kernel), kPipeSmemMax, "conv3x3")) return rc;
    CUtensorMap tm_in, tm_in2, tm_w;
    memset(&tm_in2, 0, sizeof(tm_in2));
    if (wg.ring) {
      // boxes of one row of all channel groups of each input
      if (make_act_map(&tm_in, c.in, c.c_in, c.width, c.height, c.nimg, wg.spitch, 1, 2 * nci) != 0) return MJPBR_ERR_CUDA;
      if (c.c_in2 > 0 && make_act_map(&tm_in2, c.in2, c.c_in2, c.width, c.height, c.nimg, wg.spitch, 1, 2 * (nchunk - nci)) != 0) return MJPBR_ERR_CUDA;
    } else {
      if (make_act_map(&tm_in, c.in, c.c_in, c.width, c.height, c.nimg, wg.spitch, g.rows + 2, 2 * G) != 0) return MJPBR_ERR_CUDA;
      if (half_in2 && make_act_map(&tm_in2, c.in2, c.c_in2, c.width / 2, c.height / 2, c.nimg, wg.s2w, wg.s2h, 2 * G) != 0) return MJPBR_ERR_CUDA;
      if (c.c_in2 > 0 && c.in2_full && make_act_map(&tm_in2, c.in2, c.c_in2, c.width, c.height, c.nimg, wg.spitch, g.rows + 2, 2 * G) != 0) return MJPBR_ERR_CUDA;
    }
    if (make_weight_map(&tm_w, c.weight, g.cin, c.c_out, wg.resident ? 2 * nchunk : 2 * G) != 0) return MJPBR_ERR_CUDA;
    // resident CTAs per SM, limited by shared memory (1 KB of it reserved per CTA), registers
    // and the 512 tensor-memory columns (two accumulators per CTA)
    static cudaFuncAttributes attr = {};
    static int smem_per_sm = 0;
    if (smem_per_sm == 0) {
      int dev = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&smem_per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
      cudaFuncGetAttributes(&attr, conv3x3_ws_kernel);
    }
    const int regs = std::max(1, (attr.numRegs + 7) / 8 * 8) * kWsThreads;
    int per_sm = smem_per_sm / (int)(smem + attr.sharedSizeBytes + 1024);
    per_sm = std::min({per_sm, 65536 / regs, 512 / (2 * acc_cols)});
    per_sm = std::max(1, per_sm);
    const int64_t grid = std::min<int64_t>(tiles, (int64_t)conv_sm_count() * per_sm);
    conv3x3_ws_kernel<<<(unsigned)grid, kWsThreads, smem, stream>>>(c, wg, tm_in, tm_in2, tm_w);
    return check_launch("conv3x3_ws_kernel");
  }
  const size_t smem = (size_t)6 * (g.rows + 2) * g.pitch * 16 + (size_t)18 * c.c_out * 16;
  if (int rc = ensure_smem(reinterpret_cast<const void*>(conv3x3_kernel), smem, "conv3x3")) return rc;
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
  if (p.in2_full) return __ldg(reinterpret_cast<const uint4*>(p.in2 + (((int64_t)img * p.height + iy) * p.width + ix) * p.c_in2 + (ch - p.c_in)));
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

// grad_bias[co] += sum over pixels of grad_out[p][co]: one CTA per kBiasPix pixels. Thread t sums
// channel group t % (c_out / 8) of every (256 / groups)-th pixel in registers (consecutive threads
// read consecutive 16-byte groups), then one shared atomic per channel and thread and one global
// atomic per channel and CTA.
constexpr int32_t kBiasPix = 4096;

__global__ void __launch_bounds__(256) bias_grad_kernel(const uint16_t* __restrict__ grad_out, int64_t npix, int32_t cout,
                                                        float* __restrict__ grad_bias) {
  __shared__ float part[256];
  for (int32_t i = threadIdx.x; i < cout; i += blockDim.x) part[i] = 0.0f;
  __syncthreads();
  const int32_t groups = cout / 8;
  const int32_t step = blockDim.x / groups;
  const int32_t cg = threadIdx.x % groups, pofs = threadIdx.x / groups;
  if (pofs < step) {
    float acc[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    const int64_t p0 = (int64_t)blockIdx.x * kBiasPix;
    const int64_t p1 = min(p0 + kBiasPix, npix);
    for (int64_t pix = p0 + pofs; pix < p1; pix += step) {
      const uint4 v = __ldg(reinterpret_cast<const uint4*>(grad_out + pix * cout + cg * 8));
      const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        acc[2 * k] += __uint_as_float(w[k] << 16);
        acc[2 * k + 1] += __uint_as_float(w[k] & 0xFFFF0000u);
      }
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) atomicAdd(&part[cg * 8 + k], acc[k]);
  }
  __syncthreads();
  for (int32_t i = threadIdx.x; i < cout; i += blockDim.x) atomicAdd(grad_bias + i, part[i]);
}


// ---- weight gradients, warp-specialised: per tap, D_tap (c_out x cin, FP32 in tensor memory) +=
// grad_out (c_out x pixels) * input shifted by the tap (cin x pixels)^T, K = the tile's 128
// pixels, 16 per MMA. Both operands are MN-major (channels contiguous, as NHWC stores them), so
// they are the TMA boxes as they land: grad_out as channel-group planes of 128 pixels x 16 bytes,
// the input as the forward kernel stages it (halo rows, one copy with halo columns for one-row
// tiles, three dx-shifted copies otherwise). MN-major descriptors: leading byte offset = stride
// between 8-pixel groups (128 B), stride byte offset = stride between 8-channel groups (a plane).
// M = c_out padded to 64 or 128 (zero planes); an M = 64 accumulator holds row r in tensor-memory
// lane 32 (r / 16) + r % 16. Warp 4 loads, warps 5-7 issue the MMAs of taps j, j + 3, j + 6, and
// after the CTA's tiles warps 0-3 add the accumulators to grad_weight with atomics. A launch
// covers the taps whose accumulators fit the 512 tensor-memory columns (ntap x cin); the launcher
// loops over tap ranges.
constexpr int kWgThreads = 256;
constexpr int kWgIssuers = 3;
constexpr int kWgMaxStages = 6;

struct WgGeom {
  ConvGeom g;
  int32_t ntiles;
  int32_t single, spitch;
  int32_t mpad;        // MMA M: 64 or 128
  int32_t plane;       // bytes of one input channel-group plane: (rows + 2) x spitch x 16
  int32_t in_copy;     // bytes of one input copy: (c_in / 8) planes
  int32_t in2_copy;    // bytes of one in2 copy: (c_in2 / 8) planes
  int32_t a_bytes;     // grad_out planes per stage: mpad / 8 x 2 KB
  int32_t in_off, in2_off, stage_bytes;
  int32_t nstage;
  int32_t tap0, ntap;  // taps of this launch
  int32_t tmem_cols;
};

__global__ void __launch_bounds__(kWgThreads, 1) conv3x3_wgrad_ws_kernel(const __grid_constant__ MjpbrConvGrad p, const __grid_constant__ WgGeom wg,
                                                                         const __grid_constant__ CUtensorMap tm_go, const __grid_constant__ CUtensorMap tm_in,
                                                                         const __grid_constant__ CUtensorMap tm_in2) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t full[kWgMaxStages], empty[kWgMaxStages], done;
  __shared__ uint32_t tmem_slot;
  __shared__ int32_t abort_flag;
  const ConvGeom& g = wg.g;
  const int32_t cout = p.c_out, cin = g.cin;
  const int32_t nst = wg.nstage;
  const int32_t issuers = min(kWgIssuers, wg.ntap);
  const uint32_t s0 = umma::smem_addr(smem);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // zero planes of the padded M rows (never written by the TMA)
  for (int32_t st = 0; st < nst; ++st) {
    for (int32_t i = (cout / 8) * 128 + tid; i < wg.a_bytes / 16; i += kWgThreads) {
      *reinterpret_cast<uint4*>(smem + st * wg.stage_bytes + i * 16) = make_uint4(0u, 0u, 0u, 0u);
    }
  }
  umma::fence_async_shared();
  if (warp == 0) umma::tmem_alloc(&tmem_slot, (uint32_t)wg.tmem_cols);
  if (tid == 128) {
    for (int i = 0; i < nst; ++i) {
      umma::mbar_init(&full[i], 1);
      umma::mbar_init(&empty[i], issuers);
    }
    umma::mbar_init(&done, issuers);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  volatile int32_t* abort_v = &abort_flag;
  bool ok = true;
  const int32_t copies = wg.single ? 1 : 3;
  if (warp == 4) {
    if (lane == 0) {
      const uint32_t bytes = (uint32_t)(16 * kTilePx * (cout / 8) + copies * (wg.in_copy + wg.in2_copy));
      int32_t k = 0, issued = 0;
      for (int32_t tile = blockIdx.x; tile < wg.ntiles && ok; tile += gridDim.x, ++k) {
        int32_t img, y0, x0;
        tile_origin(g, tile, img, y0, x0);
        const int32_t buf = k % nst;
        if (k >= nst) ok = ws_wait(&empty[buf], ((k / nst) + 1) & 1, abort_v, kLoaderBackoffNs);
        if (!ok) break;
        const uint32_t base = s0 + buf * wg.stage_bytes;
        umma::mbar_arrive_expect_tx(&full[buf], bytes);
        umma::tma_load_5d(base, &tm_go, &full[buf], 0, x0, y0, 0, img);
        for (int32_t dx = 0; dx < copies; ++dx) {
          const int32_t xs = wg.single ? x0 - 1 : dx - 1;
          umma::tma_load_5d(base + wg.in_off + dx * wg.in_copy, &tm_in, &full[buf], 0, xs, y0 - 1, 0, img);
          if (p.c_in2 > 0) umma::tma_load_5d(base + wg.in2_off + dx * wg.in2_copy, &tm_in2, &full[buf], 0, xs, y0 - 1, 0, img);
        }
        issued = k + 1;
      }
      if (!ok) {
        // the copies in flight land before the CTA's shared memory is released
        for (int32_t kk = max(0, issued - nst); kk < issued; ++kk) umma::mbar_wait(&full[kk % nst], (kk / nst) & 1);
      }
    }
  } else if (warp >= 5 && warp < 5 + issuers) {
    if (lane == 0) {
      const int32_t j = warp - 5;
      const uint32_t id_in = umma::make_idesc_bf16((uint32_t)wg.mpad, (uint32_t)p.c_in) | (1u << 15) | (1u << 16);
      const uint32_t id_in2 = p.c_in2 > 0 ? umma::make_idesc_bf16((uint32_t)wg.mpad, (uint32_t)p.c_in2) | (1u << 15) | (1u << 16) : 0u;
      int32_t k = 0;
      bool issued = false;
      for (int32_t tile = blockIdx.x; tile < wg.ntiles && ok; tile += gridDim.x, ++k) {
        const int32_t buf = k % nst;
        ok = ws_wait(&full[buf], (k / nst) & 1, abort_v);
        if (!ok) break;
        umma::fence_after_sync();
        const uint32_t base = s0 + buf * wg.stage_bytes;
        const uint64_t a0 = umma::make_desc(base, 128, 2048);
        const uint64_t b_in = umma::make_desc(base + wg.in_off, 128, wg.plane);
        const uint64_t b_in2 = umma::make_desc(base + wg.in2_off, 128, wg.plane);
        for (int32_t t = j; t < wg.ntap; t += kWgIssuers) {
          const int32_t tap = wg.tap0 + t, dy = tap / 3, dx = tap % 3;
          // start of the tap's view of the staged input, in 16-byte units
          const uint32_t sh = wg.single ? (uint32_t)(dy * wg.spitch + dx) : (uint32_t)(dx * wg.in_copy + dy * g.pitch * 16) >> 4;
          const uint32_t sh2 = wg.single ? sh : (uint32_t)(dx * wg.in2_copy + dy * g.pitch * 16) >> 4;
          const uint32_t d = tmem + (uint32_t)(t * cin);
#pragma unroll 1
          for (int32_t ks = 0; ks < kTilePx / 16; ++ks) {
            const bool acc = k > 0 || ks > 0;
            umma::mma_bf16(d, a0 + ks * 16, b_in + sh + ks * 16, id_in, acc);
            if (p.c_in2 > 0) umma::mma_bf16(d + (uint32_t)p.c_in, a0 + ks * 16, b_in2 + sh2 + ks * 16, id_in2, acc);
          }
        }
        umma::commit(&empty[buf]);
        issued = true;
      }
      // done completes once every issuer's MMAs completed
      umma::commit(&done);
      if (!ok && issued) umma::mbar_wait(&done, 0);
    }
  } else if (warp < 4) {
    // ---- epilogue: accumulator rows -> grad_weight ----
    ok = ws_wait(&done, 0, abort_v, kEpilogueBackoffNs);
    if (__all_sync(0xFFFFFFFFu, ok)) {
      umma::fence_after_sync();
      const int32_t row = wg.mpad == 128 ? tid : (lane < 16 ? warp * 16 + lane : -1);
      for (int32_t t = 0; t < wg.ntap; ++t) {
        const int32_t tap = wg.tap0 + t;
        for (int32_t c0 = 0; c0 < cin; c0 += 16) {
          float v[16];
          umma::tmem_load16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(t * cin + c0), v);
          if (row >= 0 && row < cout) {
            float* gw = p.grad_weight + ((int64_t)row * 9 + tap) * cin + c0;
#pragma unroll
            for (int i = 0; i < 16; ++i) atomicAdd(gw + i, v[i]);
          }
        }
      }
    } else {
      ok = false;
    }
  }
  if (!ok && tid % 32 == 0 && p.error_word) atomicOr(p.error_word, kErrWaitTimeout);
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) umma::tmem_free(tmem, (uint32_t)wg.tmem_cols);
}


constexpr int kWgradWsUnsuitable = -1000;

// Plans and launches conv3x3_wgrad_ws_kernel over the tap ranges that fit tensor memory;
// kWgradWsUnsuitable when two stages do not fit shared memory (the caller falls back).
int wgrad_ws_launch(const MjpbrConvGrad& c, const WgradGeom& gg, cudaStream_t stream) {
  WgGeom wg;
  wg.g.pitch = gg.pitch;
  wg.g.rows = gg.rows;
  wg.g.tiles_per_row = gg.tiles_per_row;
  wg.g.tiles_per_img = gg.tiles_per_img;
  wg.g.cin = gg.cin;
  wg.ntiles = gg.total;
  wg.single = gg.rows == 1;
  wg.spitch = wg.single ? gg.pitch + 2 : gg.pitch;
  wg.mpad = c.c_out <= 64 ? 64 : 128;
  if (c.c_out > 128) return kWgradWsUnsuitable;
  const int32_t copies = wg.single ? 1 : 3;
  auto round128 = [](int64_t v) { return (int32_t)((v + 127) / 128 * 128); };
  wg.plane = (gg.rows + 2) * wg.spitch * 16;
  wg.in_copy = (c.c_in / 8) * wg.plane;
  wg.in2_copy = (c.c_in2 / 8) * wg.plane;
  wg.a_bytes = wg.mpad / 8 * 2048;
  wg.in_off = wg.a_bytes;
  wg.in2_off = round128((int64_t)wg.in_off + (int64_t)copies * wg.in_copy);
  wg.stage_bytes = round128((int64_t)wg.in2_off + (int64_t)copies * wg.in2_copy);
  // TMA destinations are 128-byte aligned: the dx copies must be too
  if (!wg.single && ((wg.in_copy % 128) || (wg.in2_copy % 128))) return kWgradWsUnsuitable;
  wg.nstage = std::min<int64_t>(kWgMaxStages, (int64_t)kPipeSmemMax / wg.stage_bytes);
  if (wg.nstage < 2) return kWgradWsUnsuitable;
  const size_t smem = (size_t)wg.nstage * wg.stage_bytes;
  if (int rc = ensure_smem(reinterpret_cast<const void*>(conv3x3_wgrad_ws_kernel), kPipeSmemMax, "conv3x3 wgrad")) return rc;
  CUtensorMap tm_go, tm_in, tm_in2;
  memset(&tm_in2, 0, sizeof(tm_in2));
  if (make_act_map(&tm_go, c.grad_out, c.c_out, c.width, c.height, c.nimg, gg.pitch, gg.rows, c.c_out / 8) != 0) return MJPBR_ERR_CUDA;
  if (make_act_map(&tm_in, c.in, c.c_in, c.width, c.height, c.nimg, wg.spitch, gg.rows + 2, c.c_in / 8) != 0) return MJPBR_ERR_CUDA;
  if (c.c_in2 > 0 && make_act_map(&tm_in2, c.in2, c.c_in2, c.width, c.height, c.nimg, wg.spitch, gg.rows + 2, c.c_in2 / 8) != 0) return MJPBR_ERR_CUDA;
  const int32_t per_pass = std::min(9, 512 / gg.cin);
  if (per_pass < 1) return kWgradWsUnsuitable;
  const int64_t grid = std::min<int64_t>(gg.total, conv_sm_count());
  for (int32_t t0 = 0; t0 < 9; t0 += per_pass) {
    wg.tap0 = t0;
    wg.ntap = std::min(per_pass, 9 - t0);
    int32_t cols = 32;
    while (cols < wg.ntap * gg.cin) cols <<= 1;
    wg.tmem_cols = cols;
    conv3x3_wgrad_ws_kernel<<<(unsigned)grid, kWgThreads, smem, stream>>>(c, wg, tm_go, tm_in, tm_in2);
    if (int rc = check_launch("conv3x3_wgrad_ws_kernel")) return rc;
  }
  return MJPBR_OK;
}

}  // namespace

int conv3x3_wgrad_launch(const MjpbrConvGrad& c, cudaStream_t stream) {
  if (!c.in || !c.grad_out || !c.grad_weight) return set_error(MJPBR_ERR_ARG, "conv3x3 wgrad: missing input, gradient or output");
  if (c.nimg < 1 || c.height < 1 || c.width < 1) return set_error(MJPBR_ERR_ARG, "conv3x3 wgrad: empty image batch");
  if (c.c_in < 16 || c.c_in % 16 || c.c_in2 < 0 || c.c_in2 % 16 || c.c_out < 16 || c.c_out % 16 || c.c_out > 256) {
    return set_error(MJPBR_ERR_ARG, "conv3x3 wgrad: channels must be multiples of 16 (c_out <= 256), got %d + %d -> %d", c.c_in,
                     c.c_in2, c.c_out);
  }
  if (c.c_in2 > 0 && !c.in2) return set_error(MJPBR_ERR_ARG, "conv3x3 wgrad: c_in2 > 0 needs in2");
  if (c.c_in2 > 0 && !c.in2_full && (c.height % 2 || c.width % 2)) return set_error(MJPBR_ERR_ARG, "conv3x3 wgrad: a half-resolution in2 needs even sizes");
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
  if (conv_pipeline_enabled() && (c.c_in2 == 0 || c.in2_full) && (int64_t)c.nimg * c.height * c.width <= INT32_MAX) {
    const int rc = wgrad_ws_launch(c, g, stream);
    if (rc != kWgradWsUnsuitable) {
      if (rc != MJPBR_OK) return rc;
      if (c.grad_bias) {
        const int64_t npix = (int64_t)c.nimg * c.height * c.width;
        bias_grad_kernel<<<(unsigned)((npix + kBiasPix - 1) / kBiasPix), 256, 0, stream>>>(c.grad_out, npix, c.c_out, c.grad_bias);
        return check_launch("bias_grad_kernel");
      }
      return MJPBR_OK;
    }
  }
  const int32_t mblocks = (9 * g.cin + 127) / 128;
  const int32_t splits = (g.total + g.per_cta - 1) / g.per_cta;
  if (splits > 65535) return set_error(MJPBR_ERR_ARG, "conv3x3 wgrad: %d tile runs exceed the grid; raise tiles_per_cta", splits);
  const size_t smem = (size_t)16 * 16 * 128 + (size_t)16 * c.c_out * 16;
  if (int rc = ensure_smem(reinterpret_cast<const void*>(conv3x3_wgrad_kernel), smem, "conv3x3 wgrad")) return rc;
  conv3x3_wgrad_kernel<<<dim3(mblocks, splits), kConvThreads, smem, stream>>>(c, g);
  if (int rc = check_launch("conv3x3_wgrad_kernel")) return rc;
  if (c.grad_bias) {
    const int64_t npix = (int64_t)c.nimg * c.height * c.width;
    bias_grad_kernel<<<(unsigned)((npix + kBiasPix - 1) / kBiasPix), 256, 0, stream>>>(c.grad_out, npix, c.c_out, c.grad_bias);
    return check_launch("bias_grad_kernel");
  }
  return MJPBR_OK;
}

namespace {

// Failure-detection check of the bounded waits above: one CTA in the roles of the warp-specialised
// kernels — warp 0 a consumer waiting (ws_wait) on a "full" mbarrier that no producer completes,
// warp 1 a waiter on a second barrier that only the abort flag releases, warp 2 a plain
// mbar_wait. Every wait is bounded by `polls`; the first to give up raises the CTA's abort flag,
// which ends the other role's wait, and the CTA ORs kErrWaitTimeout into the error word and
// returns. Nothing in it spins without a bound and nothing faults.
__global__ void __launch_bounds__(96) wait_probe_kernel(uint32_t polls, int32_t* error_word, int32_t* roles_done) {
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ int32_t abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    umma::mbar_init(&bars[0], 1);
    umma::mbar_init(&bars[1], 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  volatile int32_t* abort_v = &abort_flag;
  bool ok = true;
  if (lane == 0) {
    if (warp == 0) {
      ok = ws_wait(&bars[0], 0, abort_v, 0, polls);
    } else if (warp == 1) {
      // released by the abort flag (checked every 256 polls), or gives up after 256 x polls itself
      ok = ws_wait(&bars[1], 0, abort_v, 0, polls * 256u);
    } else {
      ok = umma::mbar_wait(&bars[0], 0, polls);
    }
    atomicAdd(roles_done, 1);
    if (!ok && error_word) atomicOr(error_word, kErrWaitTimeout);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(umma::smem_addr(&bars[0])) : "memory");
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(umma::smem_addr(&bars[1])) : "memory");
  }
}

}  // namespace

int wait_probe_launch(uint32_t polls, int32_t* error_word, int32_t* roles_done, cudaStream_t stream) {
  if (polls < 1 || polls > (1u << 20) || !error_word || !roles_done) {
    return set_error(MJPBR_ERR_ARG, "wait probe: polls must be in [1, 2^20] and both words given");
  }
  wait_probe_kernel<<<1, 96, 0, stream>>>(polls, error_word, roles_done);
  return check_launch("wait_probe_kernel");
}

}  // namespace mjpbr
