// Path-traced tier (placeholder until the wavefront path tracer lands).
#include "abi_internal.h"

namespace mjpbr {

int render_pt_launch(const MjpbrScene& s, uint32_t seed, cudaStream_t stream) {
  (void)s;
  (void)seed;
  (void)stream;
  return set_error(MJPBR_ERR_UNSUPPORTED, "the path-traced tier is not built into this library yet");
}

}  // namespace mjpbr
