// BF16 GEMM on the 5th-generation tensor cores: D (M x N, FP32) = A (M x K, BF16, row-major) *
// B^T (B: N x K, BF16, row-major), FP32 accumulation in tensor memory. One CTA of 128 threads per
// 128-row block of A: the threads stage 64-wide K chunks of A and B into shared memory in the
// K-major core-matrix layout, one elected thread issues the tcgen05.mma instructions of the chunk
// and commits them to an mbarrier, and after the last chunk each warp reads its 32 accumulator
// rows out of tensor memory (tcgen05.ld) and writes them to D.
//
// Used by the learned denoiser (1 x 1 layers and the kernel-prediction head) and as the
// known-answer check of the tcgen05 descriptor encodings (tests compare it with a CPU product).
#include <algorithm>

#include "abi_internal.h"
#include "common.cuh"
#include "umma.cuh"

namespace mjpbr {
namespace {

constexpr int kRows = 128;
constexpr int kChunk = 64;  // K elements staged per round
constexpr int kGemmThreads = 128;

__global__ void __launch_bounds__(kGemmThreads) gemm_bf16_kernel(const uint16_t* __restrict__ a, const uint16_t* __restrict__ b,
                                                                 float* __restrict__ d, int32_t n, int32_t k, int32_t* error_word) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_slot;
  uint8_t* sa = smem;                               // [kChunk / 8][kRows][16 B]
  uint8_t* sb = smem + (kChunk / 8) * kRows * 16;   // [kChunk / 8][n][16 B]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t row0 = (int64_t)blockIdx.x * kRows;
  uint32_t ncols = 32;
  while (ncols < (uint32_t)n) ncols <<= 1;
  if (warp == 0) umma::tmem_alloc(&tmem_slot, ncols);
  if (tid == 0) {
    umma::mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = umma::make_idesc_bf16(kRows, n);
  bool ok = true;
  uint32_t phase = 0;
  for (int32_t k0 = 0; k0 < k; k0 += kChunk) {
    const int32_t kc = min(kChunk, k - k0);
    const int32_t groups = kc / 8;
    // stage A and B: one 16-byte core-matrix row per thread per step
    for (int32_t i = tid; i < groups * kRows; i += kGemmThreads) {
      const int32_t g = i / kRows, r = i - g * kRows;
      const uint4 v = *reinterpret_cast<const uint4*>(a + (row0 + r) * k + k0 + g * 8);
      *reinterpret_cast<uint4*>(sa + (g * kRows + r) * 16) = v;
    }
    for (int32_t i = tid; i < groups * n; i += kGemmThreads) {
      const int32_t g = i / n, r = i - g * n;
      const uint4 v = *reinterpret_cast<const uint4*>(b + (int64_t)r * k + k0 + g * 8);
      *reinterpret_cast<uint4*>(sb + (g * n + r) * 16) = v;
    }
    umma::fence_async_shared();
    __syncthreads();
    umma::fence_after_sync();
    if (tid == 0) {
      const uint32_t a0 = umma::smem_addr(sa), b0 = umma::smem_addr(sb);
      for (int32_t s = 0; s < kc / 16; ++s) {
        const uint64_t ad = umma::make_desc(a0 + s * 2 * kRows * 16, kRows * 16, 128);
        const uint64_t bd = umma::make_desc(b0 + s * 2 * n * 16, n * 16, 128);
        umma::mma_bf16(tmem, ad, bd, idesc, k0 > 0 || s > 0);
      }
      umma::commit(&bar);
    }
    // the staged chunk is reused only after its MMAs completed
    ok = ok && umma::mbar_wait(&bar, phase);
    phase ^= 1u;
    umma::fence_after_sync();
    __syncthreads();
    if (!ok) break;
  }
  if (ok) {
    const int64_t row = row0 + warp * 32 + lane;
    for (int32_t c = 0; c < n; c += 16) {
      float v[16];
      umma::tmem_load16(tmem + ((uint32_t)(warp * 32) << 16) + c, v);
      float4* out = reinterpret_cast<float4*>(d + row * n + c);
      out[0] = make_float4(v[0], v[1], v[2], v[3]);
      out[1] = make_float4(v[4], v[5], v[6], v[7]);
      out[2] = make_float4(v[8], v[9], v[10], v[11]);
      out[3] = make_float4(v[12], v[13], v[14], v[15]);
    }
  } else {
    if (tid == 0 && error_word) atomicOr(error_word, kErrWaitTimeout);
    // give the MMAs in flight a second bounded wait before their accumulators are freed
    umma::mbar_wait(&bar, phase ^ 1u);
  }
  umma::fence_before_sync();
  __syncthreads();
  if (warp == 0) umma::tmem_free(tmem, ncols);
}

}  // namespace

int gemm_bf16_launch(const uint16_t* a, const uint16_t* b, float* d, int32_t m, int32_t n, int32_t k, int32_t* error_word,
                     cudaStream_t stream) {
  if (!a || !b || !d) return set_error(MJPBR_ERR_ARG, "gemm: NULL operand");
  if (m <= 0 || m % kRows) return set_error(MJPBR_ERR_ARG, "gemm: M must be a positive multiple of %d, got %d", kRows, m);
  if (n < 16 || n > 256 || n % 16) return set_error(MJPBR_ERR_ARG, "gemm: N must be a multiple of 16 in [16, 256], got %d", n);
  if (k < 16 || k % 16) return set_error(MJPBR_ERR_ARG, "gemm: K must be a positive multiple of 16, got %d", k);
  if ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b) | reinterpret_cast<uintptr_t>(d)) & 15u) {
    return set_error(MJPBR_ERR_ARG, "gemm: operands must be 16-byte aligned");
  }
  // at least 64 KB: every operand read the descriptors can express for these shapes stays inside
  // the allocation
  const size_t smem = std::max<size_t>((size_t)(kChunk / 8) * (kRows + n) * 16, 64 * 1024);
  if (int rc = ensure_smem(reinterpret_cast<const void*>(gemm_bf16_kernel), smem, "gemm")) return rc;
  gemm_bf16_kernel<<<m / kRows, kGemmThreads, smem, stream>>>(a, b, d, n, k, error_word);
  return check_launch("gemm_bf16_kernel");
}

}  // namespace mjpbr
