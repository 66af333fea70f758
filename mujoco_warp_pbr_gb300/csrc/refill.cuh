// Persistent ray loops with lane refill, for the traversal stages of the wavefront schedules.
//
// A warp's lanes each trace one ray of a queue as a resumable query (trace.cuh: AnyQuery,
// ClosestQuery) and take the next queue item as soon as their ray is done, instead of waiting for
// the warp's slowest ray: every trip, the idle lanes fetch items from a counter (one atomic per warp),
// then every busy lane advances its query by up to kSteps steps. The per-ray results are the
// queries' own, so they do not depend on which lane traces which ray, or when.
#pragma once

#include "trace.cuh"

namespace mjpbr {

constexpr int32_t kAnyAbort = 3;                       // a query stopped by the step bound
constexpr int32_t kMaxRaySteps = 1 << 20;              // steps of one ray: far above any traversal of a scene
constexpr uint64_t kRefillTimeLimitNs = 4000000000ull; // three orders of magnitude above the largest chunk's stage

MJ_DEV uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Runs the warp's share of `items` queue items (every lane of every warp of the launch must call
// it). fetch(item, q) sets up the query of an item and returns false when the item has no ray;
// step(q) advances the query (kAnyRunning while it runs); finish(q, result) stores a finished
// query's result (result kAnyAbort after kMaxRaySteps steps, with kErrWorkQueue in *err).
// `counter` (64-bit, zero before the launch) hands the items out. Every trip takes new items or
// advances a ray, so the loop ends; a launch still running after kRefillTimeLimitNs sets
// kErrWorkQueue and returns instead of spinning.
template <int32_t kSteps, class Query, class Fetch, class Step, class Finish>
MJ_DEV void refill_loop(int64_t items, unsigned long long* counter, Query& q, const Fetch& fetch, const Step& step, const Finish& finish,
                        int32_t* err) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  bool busy = false, exhausted = false;
  int32_t steps = 0;
  const uint64_t t_start = global_ns();
  for (;;) {
    if (__any_sync(full, global_ns() - t_start > kRefillTimeLimitNs)) {
      *err |= kErrWorkQueue;
      return;
    }
    const bool need = !busy && !exhausted;
    const unsigned m = __ballot_sync(full, need);
    if (m) {
      const int leader = __ffs(m) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(m));
      base = __shfl_sync(full, base, leader);
      if (need) {
        const int64_t item = (int64_t)base + __popc(m & ((1u << lane) - 1u));
        if (item >= items) {
          exhausted = true;
        } else if (fetch(item, q)) {
          busy = true;
          steps = 0;
        }
      }
    }
    if (__ballot_sync(full, busy) == 0) {
      if (__all_sync(full, exhausted)) return;
      continue;
    }
    if (busy) {
#pragma unroll 1
      for (int32_t k = 0; k < kSteps; ++k) {
        int32_t res = step(q);
        if (++steps > kMaxRaySteps && res == kAnyRunning) {
          *err |= kErrWorkQueue;
          res = kAnyAbort;
        }
        if (res != kAnyRunning) {
          finish(q, res);
          busy = false;
          break;
        }
      }
    }
  }
}

}  // namespace mjpbr
