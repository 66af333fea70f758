// Operation counters of the counting build (libmjpbr_count.so, compiled with MJPBR_COUNT_OPS):
// the render kernels count their ray queries, bounding-box and triangle tests, primitive tests by
// type and shading work, so that the benchmark can state the algorithmic work of a frame (the
// FP32 roofline of the real-time tier). The product library compiles the counters out.
#pragma once

#include <cstdint>

namespace mjpbr {

enum OpCount : int32_t {
  kOpRayClosest = 0,
  kOpRayAny,
  kOpBox,
  kOpTri,
  kOpPlane,
  kOpSphere,
  kOpEllipsoid,
  kOpCapsule,
  kOpCylinder,
  kOpBoxPrim,
  kOpShade,
  kOpLight,
  kOpEnv,
  kOpBackground,
  kOpPtVertex,     // path tracer: surface vertex (surface, lobes, BSDF sample, pdf and value)
  kOpPtLight,      // path tracer: next-event estimation of one light
  kOpPtEnvSample,  // path tracer: environment importance sample (CDF searches, BSDF, MIS weight)
  kOpCountN
};

// 32 copies of every counter (indexed by CTA) spread the atomics over L2.
constexpr int32_t kOpCopies = 32;

#ifdef MJPBR_COUNT_OPS
// one copy per translation unit (no relocatable device code): mjpbr_count_set sets every unit's
static __device__ unsigned long long* g_op_counts;
#define MJPBR_COUNT(k) \
  do { \
    if (g_op_counts) atomicAdd(g_op_counts + (k) * kOpCopies + (blockIdx.x & (kOpCopies - 1)), 1ull); \
  } while (0)
#else
#define MJPBR_COUNT(k) ((void)0)
#endif

}  // namespace mjpbr
