// mjpbr_refit_render_static: refit + render with the per-world blocks and the path tracer's work
// counter in library-owned static device memory, so the call allocates nothing and needs no
// scratch from its caller.
//
// Who needs it: hosts that cannot hand the library device memory after start-up, e.g. a process
// that runs inside a fixed device-memory arena (a simulator or game loop that pre-reserves its
// whole budget), or a plugin whose host owns every allocation and offers none for scratch. They
// only provide the inputs and the output images; scene->world_blocks, scene->work_counter and
// scene->wave_scratch are ignored (a real-time scene set to the wavefront schedule renders with
// the grid schedule, whose images are the same).
//
// Limits: the blocks of all worlds must fit kStaticBlockFloats floats (16 MiB), i.e.
// nworld * world_block_floats <= 4,194,304, else the call fails with MJPBR_ERR_ARG before any
// work. The static buffers are shared by every call in the process on a device: calls that
// overlap in time (two streams, or two host threads without ordering) race on them. The buffers
// belong to the current device, so the stream must be one of that device (else MJPBR_ERR_ARG).
// The first call on each device (and the first after that device's context was re-created, e.g.
// by cudaDeviceReset) looks the buffers up with cudaGetSymbolAddress, so make that call before
// any stream capture.
#include <mutex>

#include "abi_internal.h"

namespace mjpbr {
namespace {

constexpr int64_t kStaticBlockFloats = int64_t(4) << 20;
constexpr int kMaxDevices = 64;

__device__ __align__(256) float g_static_blocks[kStaticBlockFloats];
__device__ __align__(256) int32_t g_static_counter[4];

using CtxGetCurrentFn = int (*)(void**);

// cuCtxGetCurrent through the runtime's driver entry point (no link against libcuda).
CtxGetCurrentFn ctx_get_current() {
  static CtxGetCurrentFn fn = [] {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      f = nullptr;
    }
    return reinterpret_cast<CtxGetCurrentFn>(f);
  }();
  return fn;
}

struct DeviceScratch {
  void* ctx;  // the context the addresses below were looked up in
  float* blocks;
  int32_t* counter;
};

std::mutex g_lookup_mutex;
DeviceScratch g_scratch[kMaxDevices];

// Device addresses of the static buffers on the current device, looked up again whenever the
// device's current context differs from the one of the cached addresses (a module reloaded after
// a context was destroyed and re-created may place the buffers elsewhere).
int static_scratch(cudaStream_t stream, float** blocks, int32_t** counter) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error(MJPBR_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return set_error(MJPBR_ERR_ARG, "device %d beyond the %d supported", dev, kMaxDevices);
  if (stream) {
    int sdev = -1;
    e = cudaStreamGetDevice(stream, &sdev);
    if (e != cudaSuccess) return set_error(MJPBR_ERR_ARG, "stream: %s", cudaGetErrorString(e));
    if (sdev != dev) {
      return set_error(MJPBR_ERR_ARG, "the stream belongs to device %d but device %d is current: the static scratch is per device", sdev,
                       dev);
    }
  }
  void* ctx = nullptr;
  CtxGetCurrentFn get = ctx_get_current();
  if (!get || get(&ctx) != 0 || !ctx) return set_error(MJPBR_ERR_CUDA, "no current CUDA context on device %d", dev);
  std::lock_guard<std::mutex> lock(g_lookup_mutex);
  DeviceScratch& d = g_scratch[dev];
  if (d.ctx != ctx || !d.blocks) {
    void* b = nullptr;
    void* c = nullptr;
    e = cudaGetSymbolAddress(&b, g_static_blocks);
    if (e != cudaSuccess) return set_error(MJPBR_ERR_CUDA, "static world blocks: %s", cudaGetErrorString(e));
    e = cudaGetSymbolAddress(&c, g_static_counter);
    if (e != cudaSuccess) return set_error(MJPBR_ERR_CUDA, "static work counter: %s", cudaGetErrorString(e));
    d.blocks = static_cast<float*>(b);
    d.counter = static_cast<int32_t*>(c);
    d.ctx = ctx;
  }
  *blocks = d.blocks;
  *counter = d.counter;
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
  // the wavefront schedules keep their queues in caller scratch: render with the grid schedule /
  // the persistent path kernel instead (the same images)
  if (s.settings.schedule == MJPBR_SCHEDULE_WAVEFRONT) s.settings.schedule = MJPBR_SCHEDULE_GRID;
  s.wave_scratch = nullptr;
  s.wave_scratch_bytes = 0;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int rc = static_scratch(st, &s.world_blocks, &s.work_counter);
  if (rc) return rc;
  rc = validate_scene(&s, true);
  if (rc) return rc;
  rc = refit_launch(s, st);
  if (rc) return rc;
  // render_pt_launch zeroes the work counter on the stream before its kernel starts
  if (s.settings.tier == MJPBR_TIER_PATH) return render_pt_launch(s, seed, st);
  return render_rt_launch(s, seed, st);
}
