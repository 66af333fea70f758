// mjpbr_refit_render_static: refit + render with the per-world blocks and the path tracer's work
// counter in library-owned static device memory, so the call allocates nothing and needs no
// scratch from its caller.
//
// Who needs it: hosts that cannot hand the library device memory after start-up, e.g. a process
// that runs inside a fixed device-memory arena (a simulator or game loop that pre-reserves its
// whole budget), or a plugin whose host owns every allocation and offers none for scratch. They
// only provide the inputs and the output images; scene->world_blocks and scene->work_counter are
// ignored.
//
// Limits: the blocks of all worlds must fit kStaticBlockFloats floats (16 MiB), i.e.
// nworld * world_block_floats <= 4,194,304, else the call fails with MJPBR_ERR_ARG before any
// work. The static buffers are shared by every call in the process on a device: calls that
// overlap in time (two streams, or two host threads without ordering) race on them. The first
// call on each device looks the buffers up (cudaGetSymbolAddress), so make that first call before
// any stream capture.
#include <mutex>

#include "abi_internal.h"

namespace mjpbr {
namespace {

constexpr int64_t kStaticBlockFloats = int64_t(4) << 20;
constexpr int kMaxDevices = 64;

__device__ __align__(256) float g_static_blocks[kStaticBlockFloats];
__device__ __align__(256) int32_t g_static_counter[4];

std::mutex g_lookup_mutex;
float* g_blocks[kMaxDevices];
int32_t* g_counter[kMaxDevices];

// Device addresses of the static buffers on the current device (looked up once per device).
int static_scratch(float** blocks, int32_t** counter) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error(MJPBR_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return set_error(MJPBR_ERR_ARG, "device %d beyond the %d supported", dev, kMaxDevices);
  std::lock_guard<std::mutex> lock(g_lookup_mutex);
  if (!g_blocks[dev]) {
    void* b = nullptr;
    void* c = nullptr;
    e = cudaGetSymbolAddress(&b, g_static_blocks);
    if (e != cudaSuccess) return set_error(MJPBR_ERR_CUDA, "static world blocks: %s", cudaGetErrorString(e));
    e = cudaGetSymbolAddress(&c, g_static_counter);
    if (e != cudaSuccess) return set_error(MJPBR_ERR_CUDA, "static work counter: %s", cudaGetErrorString(e));
    g_counter[dev] = static_cast<int32_t*>(c);
    g_blocks[dev] = static_cast<float*>(b);
  }
  *blocks = g_blocks[dev];
  *counter = g_counter[dev];
  return MJPBR_OK;
}

}  // namespace
}  // namespace mjpbr

extern "C" int mjpbr_refit_render_static(const MjpbrScene* scene, uint32_t seed, void* stream) {
  using namespace mjpbr;
  if (!scene) return set_error(MJPBR_ERR_ARG, "scene is NULL");
  const int64_t need = (int64_t)scene->nworld * scene->world_block_floats;
  if (need > kStaticBlockFloats) {
    return set_error(MJPBR_ERR_ARG, "static scratch holds %lld world-block floats, this scene needs %lld (nworld %d x %d)",
                     (long long)kStaticBlockFloats, (long long)need, scene->nworld, scene->world_block_floats);
  }
  MjpbrScene s = *scene;
  int rc = static_scratch(&s.world_blocks, &s.work_counter);
  if (rc) return rc;
  rc = validate_scene(&s, true);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  rc = refit_launch(s, st);
  if (rc) return rc;
  // render_pt_launch zeroes the work counter on the stream before its kernel starts
  if (s.settings.tier == MJPBR_TIER_PATH) return render_pt_launch(s, seed, st);
  return render_rt_launch(s, seed, st);
}
