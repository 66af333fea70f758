"""Autotuner of the real-time tier's launch shape, and CUDA-graph capture of a whole frame.

The real-time tier has three schedules (include/mjpbr.h, MjpbrSchedule): the megakernel as a grid
of one CTA per (camera tile, world) with 32 x 8 (RenderOrder.ROW) or 16 x 16 (TILED) pixel
tiles; the megakernel as a persistent launch whose warps pull work items of 32, 64 or 128 pixels
from a device counter (the queue's item size is its ray-sort granularity: the pixels a warp
renders back to back from one world block); and the staged wavefront (one kernel per stage over
compacted ray queues, a chunk of worlds at a time: the chunk size trades scratch memory and L2
locality against launches). Every candidate renders the same image; the autotuner times each on
the context's own scene and keeps the fastest. Results are cached per scene signature for the
process.

capture_frame() records step -> refit_bvh -> render (-> denoise) into one CUDA graph, so a
simulation loop replays the whole frame with a single launch from the host.
"""

from __future__ import annotations

import dataclasses
import time
from collections.abc import Callable
from typing import Any

import torch

from mujoco_warp_pbr_gb300 import _lib
from mujoco_warp_pbr_gb300.pbr_types import PbrRenderContext
from mujoco_warp_pbr_gb300.render import refit_bvh
from mujoco_warp_pbr_gb300.render import render
from mujoco_warp_pbr_gb300.render import scene as scene_descriptor

ROW, TILED = 0, 1
GRID, QUEUE, WAVEFRONT = 0, 1, 2


@dataclasses.dataclass(frozen=True)
class LaunchShape:
  schedule: int  # GRID, QUEUE or WAVEFRONT
  render_order: int  # grid tile shape: ROW (32 x 8) or TILED (16 x 16)
  queue_item: int  # queue work item, pixels
  wave_chunk_worlds: int = 0  # wavefront: worlds per chunk (0: about 64 M camera samples / 32 M paths)

  def describe(self) -> str:
    if self.schedule == GRID:
      return "grid 32x8" if self.render_order == ROW else "grid 16x16"
    if self.schedule == WAVEFRONT:
      return f"wavefront {self.wave_chunk_worlds or 'auto'} worlds per chunk"
    return f"queue {self.queue_item} px"


CANDIDATES = (
  LaunchShape(WAVEFRONT, TILED, 64, 0),
  LaunchShape(WAVEFRONT, TILED, 64, 64),
  LaunchShape(GRID, TILED, 64),
  LaunchShape(GRID, ROW, 64),
  LaunchShape(QUEUE, TILED, 32),
  LaunchShape(QUEUE, TILED, 64),
  LaunchShape(QUEUE, TILED, 128),
)

_cache: dict[tuple, LaunchShape] = {}


def _signature(rc: PbrRenderContext) -> tuple:
  b = rc.base
  return (
    rc.nworld,
    tuple(tuple(r) for r in b.cam_res),
    tuple(bool(v) for v in b.render_rgb),
    rc.tier,
    rc.samples_per_pixel,
    rc.shadow_samples,
    bool(rc.has_env),
    bool(rc.has_reflection),
    int(rc.world_blocks.shape[1]),
    rc.ray_direction is not None,
    torch.cuda.get_device_name(rc.device),
  )


def apply(rc: PbrRenderContext, shape: LaunchShape) -> None:
  rc.schedule = shape.schedule
  rc.render_order = shape.render_order
  rc.queue_item = shape.queue_item
  if rc.wave_chunk_worlds != shape.wave_chunk_worlds:
    rc.wave_chunk_worlds = shape.wave_chunk_worlds
    rc.wave_scratch = None  # sized again for the new chunk at the next render


def autotune(
  m: Any, d: Any, rc: PbrRenderContext, frames: int = 3, candidates: tuple[LaunchShape, ...] = CANDIDATES, use_cache: bool = True,
  timeout_ms: float = 10_000.0,
) -> dict:
  """Times every launch shape on this scene (after one warm-up frame each) and applies the
  fastest to rc. Returns {"best": description, "ms": {description: ms per frame}, "skipped":
  {description: reason}}. Shapes whose launch the library rejects or fails for this scene (the
  queue's per-warp world blocks must fit shared memory), and shapes whose warm-up frame takes
  longer than timeout_ms on the host clock, are skipped. The path-traced tier has a single
  persistent schedule: nothing to tune."""
  if rc.tier != 0:
    return {"best": "path tier: persistent tile queue", "ms": {}}
  key = _signature(rc)
  if use_cache and key in _cache:
    apply(rc, _cache[key])
    return {"best": _cache[key].describe(), "ms": {}, "cached": True}
  refit_bvh(m, d, rc)
  stream = torch.cuda.current_stream(rc.device)
  timings: dict[LaunchShape, float] = {}
  skipped: dict[str, str] = {}
  for shape in candidates:
    apply(rc, shape)
    t0 = time.perf_counter()
    try:
      render(m, d, rc)
      torch.cuda.synchronize(rc.device)
    except (ValueError, _lib.MjpbrError) as e:
      skipped[shape.describe()] = str(e)
      continue
    warm_ms = (time.perf_counter() - t0) * 1000.0
    if warm_ms > timeout_ms:
      skipped[shape.describe()] = f"warm-up frame took {warm_ms:.0f} ms (limit {timeout_ms:.0f} ms)"
      continue
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    start.record(stream)
    for i in range(frames):
      render(m, d, rc, seed=i)
    end.record(stream)
    end.synchronize()
    timings[shape] = start.elapsed_time(end) / frames
  if not timings:
    raise RuntimeError(f"no launch shape could render this scene: {skipped}")
  best = min(timings, key=timings.get)
  apply(rc, best)
  _cache[key] = best
  return {"best": best.describe(), "ms": {k.describe(): v for k, v in timings.items()}, "skipped": skipped}


def capture_frame(
  m: Any, d: Any, rc: PbrRenderContext, seed: int = 0, step: Callable[[], None] | None = None, warmup: int = 2,
  denoiser: Callable[[], None] | None = None,
) -> torch.cuda.CUDAGraph:
  """One CUDA graph of a frame: step() (e.g. the physics step, or a copy of the next poses), the
  BVH refit, the render and, for a denoised path-traced context, the filter: the a-trous passes,
  or denoiser() (e.g. the learned denoiser's kpcn.KPCN.denoise) when given. The seed is part of
  the graph. Arrays replaced by assignment after capture are not seen by the graph: capture again.
  The first calls (warm-up, outside the capture) configure the kernels and allocate workspaces."""
  s = scene_descriptor(m, d, rc)
  current = torch.cuda.current_stream(rc.device)
  side = torch.cuda.Stream(rc.device)
  side.wait_stream(current)

  def frame(stream: int) -> None:
    if step is not None:
      step()
    _lib.call("mjpbr_refit_bvh", s, stream)
    _lib.call("mjpbr_render", s, int(seed) & 0xFFFFFFFF, stream)
    if denoiser is not None:
      denoiser()
    elif rc.tier == 1 and rc.denoise:
      _lib.call("mjpbr_denoise_atrous", s, stream)

  with torch.cuda.stream(side):
    for _ in range(warmup):
      frame(side.cuda_stream)
  current.wait_stream(side)
  torch.cuda.synchronize(rc.device)
  graph = torch.cuda.CUDAGraph()
  with torch.cuda.graph(graph):
    frame(torch.cuda.current_stream(rc.device).cuda_stream)
  rc._host_cache["refit"] = True
  return graph
