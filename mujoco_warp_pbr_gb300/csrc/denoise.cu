// Edge-avoiding a-trous denoiser (placeholder until the fused tiled stencil lands).
#include "abi_internal.h"

namespace mjpbr {

int denoise_launch(const MjpbrScene& s, cudaStream_t stream) {
  (void)s;
  (void)stream;
  return set_error(MJPBR_ERR_UNSUPPORTED, "the a-trous denoiser is not built into this library yet");
}

}  // namespace mjpbr
