// Internal glue between the C entry points (abi.cu) and the kernel launchers of libmjpbr.
#pragma once

#include <cuda_runtime.h>

#include "mjpbr.h"

namespace mjpbr {

// Records a printf-style message for mjpbr_last_error() and returns code.
int set_error(int code, const char* fmt, ...);
// MJPBR_OK, or MJPBR_ERR_CUDA with the launch error of the last kernel.
int check_launch(const char* what);

// MJPBR_OK, or MJPBR_ERR_ARG with a message naming the first inconsistent field of the scene.
int validate_scene(const MjpbrScene* s, bool need_outputs);

int refit_launch(const MjpbrScene& s, cudaStream_t stream);
int render_rt_launch(const MjpbrScene& s, uint32_t seed, cudaStream_t stream);
int render_pt_launch(const MjpbrScene& s, uint32_t seed, cudaStream_t stream);
int outputs_launch(const MjpbrScene& s, int which, int32_t cam, float depth_scale, void* out, int32_t nworld_out,
                   cudaStream_t stream);
int dfg_lut_launch(float* lut, int32_t size, int32_t nsample, cudaStream_t stream);
int build_mips_launch(const MjpbrTexture* tex, uint8_t* data, cudaStream_t stream);
int prefilter_launch(const MjpbrTexture* radiance, const uint8_t* data, int32_t levels, int32_t height, int32_t width,
                     int32_t nsample, uint16_t* stack, cudaStream_t stream);
int denoise_launch(const MjpbrScene& s, cudaStream_t stream);
int conv3x3_launch(const MjpbrConv& c, cudaStream_t stream);
int conv3x3_wgrad_launch(const MjpbrConvGrad& c, cudaStream_t stream);
int gemm_bf16_launch(const uint16_t* a, const uint16_t* b, float* d, int32_t m, int32_t n, int32_t k, int32_t* error_word,
                     cudaStream_t stream);

}  // namespace mjpbr
