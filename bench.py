"""Benchmark of the real-time render path on GB300 (one JSON line on stdout).

Workload: the seeded mesh / IBL scene at scale (4096 worlds x one 128x128 camera, 6 displaced
icospheres of 5120 triangles + 10 primitives, 1024x512 HDR environment, 512x512 albedo / ORM /
normal maps with mips, 2x2 supersampling, mirror floor of reflectance 0.3, per-world materials and
environment rotation). A step is refit_bvh + render of one frame of every world.

  value      Mpix/s from CUDA events around each step (inputs resident on the device); L2 is
             flushed (a 256 MB write) before every timed step, outside the events.
  e2e        the same metric through the public API with host buffers: every step copies the
             geom / camera / light poses from pinned host memory to the device, refits, renders,
             converts with get_rgb and copies the float images (the reference's output format) to
             pinned host memory; frames above 64 MB of images copy on a second stream while the
             next step renders (double-buffered), and the timed region ends when the last copy
             has landed.
  roofline   the frame's algorithmic HBM bytes (outputs written once, world blocks and tables
             read once) over its event-timed duration, against the measured copy bandwidth, with
             the DRAM traffic of the frame's stage kernels from an ncu launch list; the render is
             bound by traversal latency and divergence, not HBM, so this fraction is small by
             construction.
  stages_ms  the wavefront's stage split from CUDA events the library records at every stage
             boundary in the timed steps.
  roofline_fp32, rays_per_s  the real-time kernel's algorithmic FP32 work: a 256-world frame of the
             same scene rendered by the counting build (libmjpbr_count.so) counts ray queries,
             box / triangle / primitive tests and shading work; FLOPS_PER_OP of
             mujoco_warp_pbr_gb300/roofline.py turns them into FLOPs per pixel, scaled to the timed
             frame over the product kernel's render time, against the nominal FP32 peak.
  cpu_baseline  the CPU oracle (scalar C restatement of the reference's real-time tier, OpenMP
             over all host cores) on a bounded sample of the same workload.

Other workloads (--workload): primitives (16 worlds x 64², plane + 8 primitives, soft shadows;
a tens-of-microseconds frame, timed as a CUDA graph replay of refit + render),
batched (2048 worlds x 3 cameras of 64², 128² and 256², one a fisheye bundle, enable masks,
autotuned launch shape, one CUDA graph per step), path (the path-traced tier as the headline),
large_path (8192 worlds x 2 cameras x 256², 2 spp, four environments, learned denoiser, one CUDA
graph per frame). The default line also carries path_tier (1024 worlds x 128² with emissive quads
at 2 spp), learned_denoiser (learned 2 spp vs a-trous 16 spp: relative MSE and Mpix/s), batched
and large_path (at 1024 worlds).

--impl reference times the reference's own CPU implementation of the path: the reference is
Python on Warp / MuJoCo Warp (not installable here), so its CPU path is timed through the C
restatement of the oracle, on all host threads, with the same config and metric.
Multi-GPU (torchrun, N > 1): one replica of the workload per GPU, no collective on the data path
(weak scaling); rank 0 prints the aggregate.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mpix/s (real-time tier, 1 GB300)"
PATH_METRIC = "Mpix/s (path-traced tier, 1 GB300)"
UNIT = "Mpix/s"


def max_over_ranks(value: float, device=None) -> float:
  """The maximum of a per-rank value over the process group (the value itself without one):
  every timed region is reported as its slowest rank."""
  import torch
  import torch.distributed as dist

  if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
    return value
  t = torch.tensor([value], dtype=torch.float64, device=device)
  dist.all_reduce(t, op=dist.ReduceOp.MAX)
  return float(t.item())


def aggregate_rate(units_per_rank: float, ms: float, world_size: int) -> float:
  """Whole-job throughput in millions of units per second: every rank processed units_per_rank
  (replicas of the workload, weak scaling) in ms, the slowest rank's time."""
  return units_per_rank * world_size / (ms / 1000.0) / 1e6


def _peaks() -> dict:
  p = ROOT / "MEASURED_PEAKS.json"
  if p.exists():
    return json.loads(p.read_text())
  return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "fallback": True}


class ClockSampler:
  """nvidia-smi clock / throttle samples every 200 ms while the timed region runs."""

  QUERY = (
    "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
    "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"
  )

  def __init__(self, index: int):
    self.index = index
    self.proc = None
    self.lines: list[str] = []

  def __enter__(self):
    try:
      self.proc = subprocess.Popen(
        ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits", "-lms", "200"],
        stdout=subprocess.PIPE,
        stderr=subprocess.DEVNULL,
        text=True,
      )
      self.thread = threading.Thread(target=self._read, daemon=True)
      self.thread.start()
    except OSError:
      self.proc = None
    return self

  def _read(self):
    for line in self.proc.stdout:
      self.lines.append(line.strip())

  def __exit__(self, *exc):
    if self.proc is not None:
      self.proc.terminate()
      try:
        self.proc.wait(timeout=5)
      except subprocess.TimeoutExpired:
        self.proc.kill()

  def summary(self) -> dict:
    sm, smax, reasons = [], [], set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in self.lines:
      parts = [p.strip() for p in line.split(",")]
      if len(parts) < 9:
        continue
      try:
        sm.append(float(parts[1]))
        smax.append(float(parts[2]))
      except ValueError:
        continue
      for name, flag in zip(names, parts[5:9], strict=False):
        if flag.lower() == "active":
          reasons.add(name)
    if not sm:
      return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
    return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons), "samples": len(sm)}


def _world_block_bytes(rc) -> int:
  return int(rc.world_blocks.numel() * 4)


def algorithmic_bytes(rc) -> int:
  """Compulsory HBM bytes of one render launch: every output written once, the world blocks,
  textures, environment and mesh BVHs read once."""
  b = rc.base
  n = rc.nworld
  out = b.rgb_data.numel() * 4 + b.depth_data.numel() * 4 + b.seg_data.numel() * 4
  if rc.render_hdr:
    out += rc.hdr_data.numel() * 4
  inputs = _world_block_bytes(rc)
  for t in (rc.tex_data, rc.blas_nodes, rc.blas_tris):
    if t is not None:
      inputs += t.numel() * t.element_size()
  if rc.env is not None:
    inputs += rc.env.radiance_data.numel() + rc.env.prefiltered.numel() * 2
  del n
  return int(out + inputs)


def _traffic(workload: str) -> float | None:
  """DRAM bytes of one frame's render kernels from an ncu launch list (profiles/ncu_traffic.txt:
  workload, bytes per frame, kernels), or None."""
  p = ROOT / "profiles" / "ncu_traffic.txt"
  if not p.exists():
    return None
  for line in p.read_text().splitlines():
    parts = line.split("#", 1)[0].split()
    if len(parts) >= 2 and parts[0] == workload:
      try:
        return float(parts[1])
      except ValueError:
        return None
  return None


def make_scene(args):
  from mujoco_warp_pbr_gb300 import synthetic

  if args.workload == "mesh_ibl":
    return synthetic.mesh_ibl_scene(seed=args.seed, nworld=args.nworld, res=args.res)
  if args.workload == "path":
    return synthetic.path_scene(seed=args.seed, nworld=args.nworld, res=args.res, spp=args.spp)
  if args.workload == "batched":
    return synthetic.batched_scene(seed=args.seed, nworld=args.nworld)
  return synthetic.primitive_scene(seed=args.seed, nworld=args.nworld, res=args.res)


def path_tier(dev, steps: int, nworld: int = 1024, res: int = 128, spp: int = 2) -> dict:
  """Secondary line: the path-traced tier on the emissive-quad scene (device-resident, per-step
  events, L2 flushed outside them)."""
  import torch

  import mujoco_warp_pbr_gb300 as mjpbr
  from mujoco_warp_pbr_gb300 import _lib
  from mujoco_warp_pbr_gb300 import synthetic

  sc = synthetic.path_scene(seed=0, nworld=nworld, res=res, spp=spp)
  m = mjpbr.put_model(sc.mjm, device=dev)
  d = mjpbr.put_data(sc.mjm, sc.mjd, nworld=sc.nworld, device=dev)
  rc = mjpbr.create_render_context(sc.mjm, sc.nworld, data=sc.mjd, device=dev, **sc.options)
  synthetic.apply_per_world(sc, m, rc)
  stream = torch.cuda.current_stream(dev)
  flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
  scene = mjpbr.scene_descriptor(m, d, rc)
  for i in range(3):
    _lib.call("mjpbr_refit_bvh", scene, stream.cuda_stream)
    _lib.call("mjpbr_render", scene, i, stream.cuda_stream)
  torch.cuda.synchronize()
  ms = []
  for i in range(steps):
    flush.zero_()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    _lib.call("mjpbr_refit_bvh", scene, stream.cuda_stream)
    _lib.call("mjpbr_render", scene, 100 + i, stream.cuda_stream)
    e1.record(stream)
    e1.synchronize()
    ms.append(e0.elapsed_time(e1))
  assert mjpbr.check_errors(rc) == 0
  npix = sc.nworld * res * res
  avg = sum(ms) / len(ms)
  # algorithmic work: a 256-world frame of the same scene through the counting build
  from mujoco_warp_pbr_gb300 import roofline

  small = synthetic.path_scene(seed=0, nworld=min(nworld, 256), res=res, spp=spp)
  ms_ = mjpbr.put_model(small.mjm, device=dev)
  ds_ = mjpbr.put_data(small.mjm, small.mjd, nworld=small.nworld, device=dev)
  rcs = mjpbr.create_render_context(small.mjm, small.nworld, data=small.mjd, device=dev, **small.options)
  synthetic.apply_per_world(small, ms_, rcs)
  counts = roofline.count_frame(mjpbr.scene_descriptor(ms_, ds_, rcs), 100, stream.cuda_stream)
  fp32 = roofline.fp32_roofline(counts, small.nworld * res * res, npix, avg,
                               kernel="path wavefront: ptw_first_extend, ptw_extend, ptw_shade, ptw_shadow, ptw_resolve per chunk")
  return {
    "workload": sc.name,
    "value": npix / (avg / 1000.0) / 1e6,
    "unit": UNIT,
    "samples_per_s": npix * spp / (avg / 1000.0),
    "rays_per_s": fp32["rays_per_px"] * npix / (avg / 1000.0),
    "ms_per_step": avg,
    "roofline_fp32": fp32,
    "config": {"nworld": nworld, "cam_res": [res, res], "spp": spp, "max_depth": 4, "rr_depth": 2, "emissive_quads": 3},
  }


def cpu_baseline(sc, budget_s: float, nthreads: int = 0) -> dict:
  """Oracle Mpix/s on a bounded sample of worlds (grown until it runs for about budget_s)."""
  from oracle import oracle

  o = oracle.OracleScene(sc.mjm, sc.mjd, sc.nworld, sc.options, sc.per_world)
  npix = sum(w * h for w, h in o.hc.outputs["cam_res"])
  worlds = 1
  t0 = time.perf_counter()
  o.render(seed=0, worlds=(0, 1), nthreads=nthreads)
  dt = time.perf_counter() - t0
  while dt < budget_s / 4 and worlds * 2 <= sc.nworld:
    worlds *= 2
    t0 = time.perf_counter()
    o.render(seed=0, worlds=(0, worlds), nthreads=nthreads)
    dt = time.perf_counter() - t0
  cores = oracle.load().oracle_nthreads() if nthreads <= 0 else nthreads
  return {
    "value": worlds * npix / dt / 1e6,
    "unit": UNIT,
    "cores": int(cores),
    "kind": "port",
    "sample": f"{worlds} of {sc.nworld} worlds x {npix} px, {dt:.1f} s",
  }


def run_reference(args) -> None:
  """--impl reference: the reference's CPU path (C restatement) on all host threads."""
  rank = int(os.environ.get("RANK", "0"))
  if rank != 0:
    return
  sc = make_scene(args)
  from oracle import oracle

  o = oracle.OracleScene(sc.mjm, sc.mjd, sc.nworld, sc.options, sc.per_world)
  npix = sum(w * h for w, h in o.hc.outputs["cam_res"])
  # each step renders a bounded sample of the worlds (about 2 s of CPU work)
  t0 = time.perf_counter()
  o.render(seed=0, worlds=(0, 1))
  one = time.perf_counter() - t0
  worlds = int(max(1, min(sc.nworld, 2.0 / max(one, 1e-6))))
  for _ in range(args.warmup):
    o.render(seed=0, worlds=(0, min(worlds, 2)))
  times = []
  for step in range(args.steps):
    t0 = time.perf_counter()
    o.render(seed=step, worlds=(0, worlds))
    times.append(time.perf_counter() - t0)
  total = sum(times)
  value = worlds * npix * args.steps / total / 1e6
  cores = oracle.load().oracle_nthreads()
  print(
    json.dumps(
      {
        "impl": "reference",
        "metric": PATH_METRIC if args.workload == "path" else METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1000.0 * total / args.steps,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": _config(args, sc),
        "cpu_baseline": {
          "value": value,
          "unit": UNIT,
          "cores": int(cores),
          "kind": "port",
          "sample": f"{worlds} of {sc.nworld} worlds per step",
        },
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference is Python on Warp/MuJoCo Warp (not installable offline); its CPU path is timed through the oracle's C restatement",
      }
    )
  )


def _config(args, sc) -> dict:
  cfg = {
    "workload": sc.name,
    "nworld": sc.nworld,
    "cam_res": [args.res, args.res],
    "samples_per_pixel": sc.options.get("samples_per_pixel", 1) ** 2,
    "seed": args.seed,
    "l2": "flushed before every timed step (256 MB write)",
  }
  if args.workload == "mesh_ibl":
    cfg.update({"meshes": 6, "triangles_per_mesh": 5120, "primitives": 10, "env": "1024x512", "textures": "3x512^2", "mirror_floor": 0.3})
  elif args.workload == "batched":
    cfg.update(
      {
        "cam_res": [list(r) for r in sc.options["cam_res"]],
        "camera_rays": "pinhole bundles + 180 deg equidistant fisheye (camera 2)",
        "visible_primitives": "U{2..16} per world (enable masks)",
        "shadow_samples": sc.options.get("shadow_samples", 1),
        "graph": "step (pose copy) -> refit_bvh -> render, one CUDA graph",
      }
    )
  elif args.workload == "path":
    cfg.update({"tier": "path", "spp": args.spp, "max_depth": 4, "rr_depth": 2, "primitives": 8, "emissive_quads": 3})
  else:
    cfg.update({"primitives": 8, "lights": 2, "shadow_samples": sc.options.get("shadow_samples", 1),
                "graph": "refit_bvh -> render captured once (seed fixed), replayed every timed step; e2e launched eagerly"})
  return cfg


class ImageCopier:
  """get_rgb's float images (nworld, H, W, 3) of the given cameras copied to pinned host memory
  after each step. Frames above 64 MB of images are double-buffered: step i's copy runs on a second
  stream while step i + 1 renders (the render stream waits for a buffer's previous copy before
  get_rgb rewrites it); smaller frames copy on the render stream."""

  def __init__(self, torch, mjpbr, rc, cams, shapes, dev, stream):
    self.torch, self.mjpbr, self.rc, self.cams, self.stream = torch, mjpbr, rc, cams, stream
    self.d2h = sum(4 * n * h * w * 3 for n, h, w, _ in shapes)
    self.overlap = self.d2h > (64 << 20)
    nbuf = 2 if self.overlap else 1
    self.dev = [[torch.empty(sh, dtype=torch.float32, device=dev) for sh in shapes] for _ in range(nbuf)]
    self.host = [[torch.empty(sh, dtype=torch.float32).pin_memory() for sh in shapes] for _ in range(nbuf)]
    self.copy_stream = torch.cuda.Stream(dev) if self.overlap else stream
    self.copied = [torch.cuda.Event() for _ in range(nbuf)]
    for ev in self.copied:
      ev.record(self.copy_stream)
    self.i = 0

  def after_step(self) -> None:
    torch, slot = self.torch, self.i % len(self.dev)
    self.i += 1
    if self.overlap:
      self.stream.wait_event(self.copied[slot])
    for cam, td in zip(self.cams, self.dev[slot], strict=True):
      self.mjpbr.get_rgb(self.rc, cam, td)
    if not self.overlap:
      for td, th in zip(self.dev[slot], self.host[slot], strict=True):
        th.copy_(td, non_blocking=True)
      return
    ready = torch.cuda.Event()
    ready.record(self.stream)
    self.copy_stream.wait_event(ready)
    with torch.cuda.stream(self.copy_stream):
      for td, th in zip(self.dev[slot], self.host[slot], strict=True):
        th.copy_(td, non_blocking=True)
      self.copied[slot].record(self.copy_stream)

  def finish(self) -> None:
    """The render stream waits for the last copy (call before recording the end event)."""
    if self.overlap:
      self.stream.wait_stream(self.copy_stream)

  def describe(self) -> str:
    return "get_rgb float32 (nworld, H, W, 3) per RGB camera" + (", double-buffered: step i's copy overlaps step i + 1" if self.overlap else "")


def run(args) -> None:
  import torch
  import torch.distributed as dist

  import mujoco_warp_pbr_gb300 as mjpbr
  from mujoco_warp_pbr_gb300 import _lib
  from mujoco_warp_pbr_gb300 import synthetic

  world_size = int(os.environ.get("WORLD_SIZE", "1"))
  rank = int(os.environ.get("RANK", "0"))
  local_rank = int(os.environ.get("LOCAL_RANK", "0"))
  sc = make_scene(args)
  baseline = None
  if rank == 0 and not args.no_cpu_baseline:
    baseline = cpu_baseline(sc, args.cpu_budget)
  torch.cuda.set_device(local_rank)
  if world_size > 1:
    dist.init_process_group("nccl")
  dev = torch.device("cuda", local_rank)
  m = mjpbr.put_model(sc.mjm, device=dev)
  d = mjpbr.put_data(sc.mjm, sc.mjd, nworld=sc.nworld, device=dev)
  rc = mjpbr.create_render_context(sc.mjm, sc.nworld, data=sc.mjd, device=dev, **sc.options)
  synthetic.apply_per_world(sc, m, rc)
  stream = torch.cuda.current_stream(dev)
  flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)  # 256 MB > L2
  npix = sc.nworld * sum(w * h for w, h in rc.base.cam_res)

  def step(seed: int) -> None:
    mjpbr.refit_bvh(m, d, rc)
    mjpbr.render(m, d, rc, seed=seed)

  for i in range(args.warmup):
    step(i)
  torch.cuda.synchronize()
  assert mjpbr.check_errors(rc) == 0, "kernels reported an error"

  # ---- device-resident timing, per-step events, L2 flushed outside the events; the wavefront's
  # stage boundaries are recorded by the library on the same stream (mjpbr_wave_profile_begin)
  import ctypes

  from mujoco_warp_pbr_gb300.profile_frame import STAGES

  # a frame of tens of microseconds (the primitive configuration) is timed as a CUDA graph replay of
  # refit + render (seed fixed), as the reference's benchmark captures its steps in a graph: launched
  # one by one, its eight launches would be timed at the host's submission rate
  graph = None
  if args.workload == "primitives":
    scene_g = mjpbr.scene_descriptor(m, d, rc)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
      cs = torch.cuda.current_stream(dev).cuda_stream
      _lib.call("mjpbr_refit_bvh", scene_g, cs)
      _lib.call("mjpbr_render", scene_g, 1000, cs)
    graph.replay()
    torch.cuda.synchronize()
  wave = rc.tier == 0 and rc.schedule == 2 and not rc.has_transparency and graph is None
  stage_sum = dict.fromkeys(STAGES, 0.0)
  stage_buf = (ctypes.c_double * len(STAGES))()
  chunks = ctypes.c_int32(0)
  starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
  mids = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
  ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
  scene = mjpbr.scene_descriptor(m, d, rc)
  if world_size > 1:
    dist.barrier()
  torch.cuda.synchronize()
  with ClockSampler(local_rank) as clocks:
    for i in range(args.steps):
      flush.zero_()
      starts[i].record(stream)
      if graph is not None:
        mids[i].record(stream)
        graph.replay()
        ends[i].record(stream)
        continue
      _lib.call("mjpbr_refit_bvh", scene, stream.cuda_stream)
      mids[i].record(stream)
      if wave:
        _lib.call("mjpbr_wave_profile_begin")
      _lib.call("mjpbr_render", scene, 1000 + i, stream.cuda_stream)
      ends[i].record(stream)
      if wave:
        _lib.call("mjpbr_wave_profile_end", stage_buf, ctypes.byref(chunks))
        for k, name in enumerate(STAGES):
          stage_sum[name] += stage_buf[k]
    torch.cuda.synchronize()
  if world_size > 1:
    dist.barrier()
  step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends, strict=True)]
  render_ms = [s.elapsed_time(e) for s, e in zip(mids, ends, strict=True)]
  total_ms = max_over_ranks(sum(step_ms), dev)
  value = aggregate_rate(npix * args.steps, total_ms, world_size)
  assert mjpbr.check_errors(rc) == 0

  # ---- end to end through the public API with host buffers: poses in from pinned memory,
  # refit + render, get_rgb's float image (the reference's output format) back to pinned memory
  host = {name: getattr(d, name).cpu().pin_memory() for name in ("geom_xpos", "geom_xmat", "cam_xpos", "cam_xmat", "light_xpos", "light_xdir")}
  shapes = [(sc.nworld, h, w, 3) for (w, h), on in zip(rc.base.cam_res, rc.base.render_rgb) if on]
  copier = ImageCopier(torch, mjpbr, rc, [c for c, on in enumerate(rc.base.render_rgb) if on], shapes, dev, stream)
  h2d = sum(t.numel() * t.element_size() for t in host.values())
  d2h = copier.d2h

  def e2e_step(i: int, seed: int) -> None:
    for name, t in host.items():
      getattr(d, name).copy_(t, non_blocking=True)
    step(seed)
    copier.after_step()

  e2e_steps = max(3, args.steps // 2)
  for i in range(2):
    e2e_step(i, i)
  torch.cuda.synchronize()
  if world_size > 1:
    dist.barrier()
  e0 = torch.cuda.Event(enable_timing=True)
  e1 = torch.cuda.Event(enable_timing=True)
  e0.record(stream)
  for i in range(e2e_steps):
    e2e_step(i, 2000 + i)
  copier.finish()
  e1.record(stream)
  torch.cuda.synchronize()
  e2e_ms = max_over_ranks(e0.elapsed_time(e1), dev)
  e2e_value = aggregate_rate(npix * e2e_steps, e2e_ms, world_size)

  if rank == 0:
    peaks = _peaks()
    render_avg = sum(render_ms) / len(render_ms)
    alg = algorithmic_bytes(rc)
    achieved = alg / (render_avg / 1000.0) / 1e9
    peak = float(peaks.get("hbm_gbs", 6800.0))
    traffic = _traffic(sc.name)
    launches = render_launches(rc, int(chunks.value), int(scene.nlight))
    if args.workload == "path":
      kernel = "path wavefront: ptw_first_extend, ptw_extend, ptw_shade, ptw_shadow, ptw_resolve per chunk, one frame"
    elif wave:
      kernel = "wavefront render: wave_primary, wave_surface, wave_mirror, wave_mirror_surface, wave_shadow, wave_resolve per chunk, one frame"
    else:
      kernel = "rt_kernel"
    line = {
      "metric": PATH_METRIC if args.workload == "path" else METRIC,
      "value": value,
      "unit": UNIT,
      "n_gpus": world_size,
      "steps": args.steps,
      "warmup": args.warmup,
      "ms_per_step": total_ms / args.steps,
      "higher_is_better": True,
      "scaling": "weak",
      "vs_baseline": None,
      "dtype": "f32",
      "data": "synthetic (seeded scenes; no dataset)",
      "config": _config(args, sc),
      "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
              "output": copier.describe()},
      "roofline": {
        "bound": "hbm",
        "kernel": kernel,
        "achieved": achieved,
        "peak": peak,
        "unit": "GB/s",
        "frac": achieved / peak,
        "traffic": traffic,
        "algorithmic_bytes_per_launch": alg,
        "peak_source": "measured" if "fallback" not in peaks else "fallback",
      },
      "render_ms": render_avg,
      "refit_ms": (total_ms / args.steps) - render_avg,
      "rays_note": "rays_per_s: every ray query of the frame (primary, shadow, mirror), counted by the counting build",
      "gpu_launches": (1 + launches) * args.steps,
      "clocks": clocks.summary(),
      "cpu_baseline": baseline,
    }
    if wave:
      line["stages_ms"] = {k: v / args.steps for k, v in stage_sum.items()}
      line["stages_note"] = f"CUDA events the library records at the wavefront's stage boundaries in the timed steps, {int(chunks.value)} chunks of worlds per frame"
    if args.workload in ("mesh_ibl", "primitives"):
      rt = rt_fp32_roofline(args, dev, npix, render_avg)
      line["roofline_fp32"] = rt
      line["rays_per_s"] = rt["rays_per_px"] * npix / (render_avg / 1000.0)
    if args.workload == "mesh_ibl" and not args.no_path_tier:
      line["path_tier"] = path_tier(dev, max(3, args.steps // 2))
      if not args.no_learned:
        line["learned_denoiser"] = learned_denoiser(args)
    if args.workload == "mesh_ibl" and not args.no_configs:
      budget = None if args.no_cpu_baseline else 5.0
      line["batched"] = measure_batched(args, dev, 2048, 10, 3, budget)
      if WEIGHTS.exists():
        line["large_path"] = measure_large(args, dev, args.large_worlds, 3, 3, budget)
        line["large_path"]["note"] = f"{args.large_worlds} of the configuration's 8192 worlds, so the default run stays within minutes (--workload large_path runs all 8192)"
    print(json.dumps(line))
  if world_size > 1:
    dist.destroy_process_group()


def frame_chunks(m, d, rc) -> int:
  """Chunks of worlds a wavefront render of rc takes (one profiled eager render), else 0."""
  import ctypes

  import mujoco_warp_pbr_gb300 as mjpbr
  from mujoco_warp_pbr_gb300 import _lib

  if not (rc.tier == 0 and rc.schedule == 2 and not rc.has_transparency):
    return 0
  buf = (ctypes.c_double * 6)()
  chunks = ctypes.c_int32(0)
  _lib.call("mjpbr_wave_profile_begin")
  mjpbr.render(m, d, rc)
  _lib.call("mjpbr_wave_profile_end", buf, ctypes.byref(chunks))
  return int(chunks.value)


def render_launches(rc, chunks: int, nlight: int) -> int:
  """Kernels one render call launches: the wavefront's stages per chunk of worlds (primary, and
  with RGB cameras surface + resolve, mirror + mirror surface with reflections, shadow with
  shadowing lights), else the single megakernel / path kernel."""
  if not (rc.tier == 0 and rc.schedule == 2 and not rc.has_transparency):
    return 1
  rgb = any(rc.base.render_rgb)
  per = 1 + (2 if rgb else 0) + (2 if rgb and rc.has_reflection else 0)
  if rgb and rc.use_shadows and nlight > 0:
    per += 1
  return per * max(chunks, 1)


def rt_fp32_roofline(args, dev, npix: int, render_ms: float, count_worlds: int = 256) -> dict:
  """FP32 roofline of the real-time kernel: one frame of the same scene with count_worlds worlds
  rendered by the counting build (mujoco_warp_pbr_gb300/roofline.py), its operation counts per
  pixel scaled to the timed frame, over the product kernel's render time."""
  import copy

  import torch

  import mujoco_warp_pbr_gb300 as mjpbr
  from mujoco_warp_pbr_gb300 import roofline
  from mujoco_warp_pbr_gb300 import synthetic

  small = copy.copy(args)
  small.nworld = min(args.nworld, count_worlds)
  sc = make_scene(small)
  m = mjpbr.put_model(sc.mjm, device=dev)
  d = mjpbr.put_data(sc.mjm, sc.mjd, nworld=sc.nworld, device=dev)
  rc = mjpbr.create_render_context(sc.mjm, sc.nworld, data=sc.mjd, device=dev, **sc.options)
  synthetic.apply_per_world(sc, m, rc)
  scene = mjpbr.scene_descriptor(m, d, rc)
  counts = roofline.count_frame(scene, 1000, torch.cuda.current_stream(dev).cuda_stream)
  counted = sc.nworld * sum(w * h for w, h in rc.base.cam_res)
  kernel = "wavefront render (all stages)" if rc.schedule == 2 and not rc.has_transparency else "rt_kernel"
  return roofline.fp32_roofline(counts, counted, npix, render_ms, kernel=kernel)


WEIGHTS = ROOT / "mujoco_warp_pbr_gb300" / "weights" / "kpcn_path.npz"


def learned_denoiser(args) -> dict | None:
  """Learned denoiser at 2 spp against the a-trous filter at 16 spp (and plain path tracing) on a
  held-out path-traced frame: relative MSE against a converged reference and Mpix/s of each
  pipeline (render + denoise), from the committed trained weights."""
  if not WEIGHTS.exists():
    return None
  from mujoco_warp_pbr_gb300 import kpcn
  from mujoco_warp_pbr_gb300 import train_kpcn

  net = kpcn.KPCN.load(WEIGHTS)
  out = train_kpcn.evaluate(net, nworld=args.learned_worlds, res=128, ref_spp=args.learned_ref_spp, time_worlds=args.learned_time_worlds)
  out["weights"] = str(WEIGHTS.relative_to(ROOT))
  return out


def measure_large(args, dev, nworld: int, steps: int, warmup: int, cpu_budget: float | None = None) -> dict:
  """Large path-traced run: nworld worlds x 2 cameras x 256², 2 spp, depth 4, four HDR
  environments, the learned denoiser (BF16, args.chunk worlds at a time); every step is one
  CUDA-graph replay of pose copy -> refit_bvh -> path tracer -> network -> finish pass."""
  import torch

  import mujoco_warp_pbr_gb300 as mjpbr
  from mujoco_warp_pbr_gb300 import kpcn
  from mujoco_warp_pbr_gb300 import synthetic

  sc = synthetic.large_path_scene(seed=args.seed, nworld=nworld, res=256)
  baseline = cpu_baseline(sc, cpu_budget) if cpu_budget else None
  m = mjpbr.put_model(sc.mjm, device=dev)
  d = mjpbr.put_data(sc.mjm, sc.mjd, nworld=sc.nworld, device=dev)
  opts = {**sc.options, "denoise": True, "render_hdr": False}
  rc = mjpbr.create_render_context(sc.mjm, sc.nworld, data=sc.mjd, device=dev, **opts)
  synthetic.apply_per_world(sc, m, rc)
  net = kpcn.KPCN.load(WEIGHTS, device=dev)
  poses = d.geom_xpos.clone()
  poses[:, 1:, 2] += 0.01
  graph = mjpbr.capture_frame(m, d, rc, seed=7, step=lambda: d.geom_xpos.copy_(poses), denoiser=lambda: net.denoise(m, d, rc, chunk=args.chunk))
  stream = torch.cuda.current_stream(dev)
  for _ in range(warmup):
    graph.replay()
  torch.cuda.synchronize()
  assert mjpbr.check_errors(rc) == 0 and int(net.error.item()) == 0
  npix = sc.nworld * sum(w * h for w, h in rc.base.cam_res)
  e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  with ClockSampler(dev.index or 0) as clocks:
    e0.record(stream)
    for _ in range(steps):
      graph.replay()
    e1.record(stream)
    torch.cuda.synchronize()
  ms = e0.elapsed_time(e1) / steps
  # end to end: poses from pinned host memory, the graph, get_rgb's float image back to the host
  host_poses = poses.cpu().pin_memory()
  copier = ImageCopier(torch, mjpbr, rc, list(range(len(rc.base.cam_res))), [(sc.nworld, h, w, 3) for w, h in rc.base.cam_res], dev, stream)
  for _ in range(2):
    poses.copy_(host_poses, non_blocking=True)
    graph.replay()
    copier.after_step()
  copier.finish()
  torch.cuda.synchronize()
  e0.record(stream)
  for _ in range(steps):
    poses.copy_(host_poses, non_blocking=True)
    graph.replay()
    copier.after_step()
  copier.finish()
  e1.record(stream)
  torch.cuda.synchronize()
  e2e_ms = e0.elapsed_time(e1) / steps
  peaks = _peaks()
  alg = algorithmic_bytes(rc)
  return {
    "metric": PATH_METRIC,
    "value": npix / ms / 1e3,
    "unit": UNIT,
    "ms_per_step": ms,
    "steps": steps,
    "warmup": warmup,
    "dtype": "f32 path tracing, bf16 network",
    "config": {"workload": sc.name, "nworld": sc.nworld, "cameras": 2, "cam_res": [256, 256], "spp": 2, "max_depth": 4,
               "rr_depth": 2, "envs": 4, "denoiser": "learned (KPCN, BF16)", "chunk_worlds": args.chunk, "graph": "one CUDA graph per frame",
               "l2": "frame working set far above L2"},
    "e2e": {"value": npix / e2e_ms / 1e3, "unit": UNIT, "h2d_bytes_per_step": int(host_poses.numel() * 4),
            "d2h_bytes_per_step": int(copier.d2h), "output": copier.describe()},
    "roofline": {
      "bound": "hbm",
      "kernel": "whole frame graph (path tracer, network, finish pass)",
      "achieved": alg / (ms / 1000.0) / 1e9,
      "peak": float(peaks.get("hbm_gbs", 6800.0)),
      "unit": "GB/s",
      "frac": alg / (ms / 1000.0) / 1e9 / float(peaks.get("hbm_gbs", 6800.0)),
      "traffic": None,
      "algorithmic_bytes_per_launch": alg,
      "peak_source": "measured" if "fallback" not in peaks else "fallback",
    },
    "device_memory_gb": torch.cuda.max_memory_allocated(dev) / 1e9,
    # per replay: refit, path tracer, the denoiser's kernels (the pose copy is a memcpy node)
    "gpu_launches": (2 + kpcn.denoise_launches(rc, args.chunk)) * steps,
    "clocks": clocks.summary(),
    "cpu_baseline": baseline,
  }


def run_large(args) -> None:
  import torch

  torch.cuda.set_device(0)
  dev = torch.device("cuda", 0)
  out = measure_large(args, dev, args.nworld, args.steps, args.warmup, None if args.no_cpu_baseline else args.cpu_budget)
  line = {**out, "n_gpus": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "data": "synthetic (seeded scenes; no dataset)"}
  print(json.dumps(line))


def measure_batched(args, dev, nworld: int, steps: int, warmup: int, cpu_budget: float | None = None, world_size: int = 1) -> dict:
  """Batched uneven workload (three cameras of 64², 128², 256² per world, one a fisheye bundle,
  per-world enable masks): autotuned launch shape, every step one CUDA-graph replay of step (a
  copy of the next poses) -> refit_bvh -> render."""
  import copy

  import torch

  import mujoco_warp_pbr_gb300 as mjpbr
  from mujoco_warp_pbr_gb300 import synthetic

  a = copy.copy(args)
  a.workload, a.nworld = "batched", nworld
  sc = make_scene(a)
  baseline = cpu_baseline(sc, cpu_budget) if cpu_budget else None
  m = mjpbr.put_model(sc.mjm, device=dev)
  d = mjpbr.put_data(sc.mjm, sc.mjd, nworld=sc.nworld, device=dev)
  rc = mjpbr.create_render_context(sc.mjm, sc.nworld, data=sc.mjd, device=dev, **sc.options)
  synthetic.apply_per_world(sc, m, rc)
  tuned = mjpbr.autotune(m, d, rc, frames=3)
  npix = sc.nworld * sum(w * h for w, h in rc.base.cam_res)
  launches = 1 + render_launches(rc, frame_chunks(m, d, rc), int(mjpbr.scene_descriptor(m, d, rc).nlight))  # refit + render
  poses = d.geom_xpos.clone()
  poses[:, 1:, 2] += 0.01  # the "next" poses the step copies in
  graph = mjpbr.capture_frame(m, d, rc, seed=7, step=lambda: d.geom_xpos.copy_(poses))
  stream = torch.cuda.current_stream(dev)
  flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=dev)
  for _ in range(warmup):
    graph.replay()
  torch.cuda.synchronize()
  assert mjpbr.check_errors(rc) == 0
  starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
  ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
  if world_size > 1:
    import torch.distributed as dist

    dist.barrier()
  torch.cuda.synchronize()
  with ClockSampler(dev.index or 0) as clocks:
    for i in range(steps):
      flush.zero_()
      starts[i].record(stream)
      graph.replay()
      ends[i].record(stream)
    torch.cuda.synchronize()
  total_ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in zip(starts, ends, strict=True)), dev)
  value = aggregate_rate(npix * steps, total_ms, world_size)
  # end to end: next poses from pinned host memory, the graph, get_rgb's float images back
  host_poses = poses.cpu().pin_memory()
  copier = ImageCopier(torch, mjpbr, rc, list(range(len(rc.base.cam_res))), [(sc.nworld, h, w, 3) for w, h in rc.base.cam_res], dev, stream)
  for _ in range(2):
    poses.copy_(host_poses, non_blocking=True)
    graph.replay()
    copier.after_step()
  copier.finish()
  torch.cuda.synchronize()
  e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  e2e_steps = max(3, steps // 2)
  e0.record(stream)
  for _ in range(e2e_steps):
    poses.copy_(host_poses, non_blocking=True)
    graph.replay()
    copier.after_step()
  copier.finish()
  e1.record(stream)
  torch.cuda.synchronize()
  e2e_ms = max_over_ranks(e0.elapsed_time(e1), dev)
  e2e_value = aggregate_rate(npix * e2e_steps, e2e_ms, world_size)
  assert mjpbr.check_errors(rc) == 0
  peaks = _peaks()
  avg = total_ms / steps
  alg = algorithmic_bytes(rc)
  achieved = alg / (avg / 1000.0) / 1e9
  peak = float(peaks.get("hbm_gbs", 6800.0))
  cfg = _config(a, sc)
  cfg["launch_shape"] = tuned["best"]
  return {
    "metric": METRIC,
    "value": value,
    "unit": UNIT,
    "steps": steps,
    "warmup": warmup,
    "ms_per_step": avg,
    "config": cfg,
    "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(host_poses.numel() * 4),
            "d2h_bytes_per_step": int(copier.d2h), "output": copier.describe()},
    "roofline": {
      "bound": "hbm",
      "kernel": f"render ({tuned['best']}), whole graph timed",
      "achieved": achieved,
      "peak": peak,
      "unit": "GB/s",
      "frac": achieved / peak,
      "traffic": _traffic(sc.name),
      "algorithmic_bytes_per_launch": alg,
      "peak_source": "measured" if "fallback" not in peaks else "fallback",
    },
    "autotune_ms": tuned.get("ms", {}),
    "gpu_launches": launches * steps,
    "clocks": clocks.summary(),
    "cpu_baseline": baseline,
  }


def run_batched(args) -> None:
  import torch
  import torch.distributed as dist

  world_size = int(os.environ.get("WORLD_SIZE", "1"))
  rank = int(os.environ.get("RANK", "0"))
  local_rank = int(os.environ.get("LOCAL_RANK", "0"))
  torch.cuda.set_device(local_rank)
  if world_size > 1:
    dist.init_process_group("nccl")
  dev = torch.device("cuda", local_rank)
  budget = args.cpu_budget if (rank == 0 and not args.no_cpu_baseline) else None
  out = measure_batched(args, dev, args.nworld, args.steps, args.warmup, budget, world_size)
  if rank == 0:
    line = {**out, "n_gpus": world_size, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded scenes; no dataset)"}
    print(json.dumps(line))
  if world_size > 1:
    dist.destroy_process_group()


def main() -> None:
  p = argparse.ArgumentParser()
  p.add_argument("--gpus", type=int, default=1)
  p.add_argument("--steps", type=int, default=None, help="timed steps (default 20; 2000 for the 0.1 ms primitives frame, so the clock sampler sees the GPU under load)")
  p.add_argument("--warmup", type=int, default=3)
  p.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
  p.add_argument("--workload", choices=["mesh_ibl", "primitives", "path", "batched", "large_path"], default="mesh_ibl")
  p.add_argument("--chunk", type=int, default=512)
  p.add_argument("--spp", type=int, default=2)
  p.add_argument("--no-path-tier", action="store_true")
  p.add_argument("--no-learned", action="store_true")
  p.add_argument("--no-configs", action="store_true", help="leave the batched and large_path objects out of the default line")
  p.add_argument("--large-worlds", type=int, default=1024, help="worlds of the default line's large_path object")
  # quality against 4096-spp references on 64 worlds, throughput on the 1024-world path batch
  p.add_argument("--learned-worlds", type=int, default=64)
  p.add_argument("--learned-ref-spp", type=int, default=4096)
  p.add_argument("--learned-time-worlds", type=int, default=1024)
  p.add_argument("--nworld", type=int, default=None)
  p.add_argument("--res", type=int, default=None)
  p.add_argument("--seed", type=int, default=0)
  p.add_argument("--cpu-budget", type=float, default=15.0)
  p.add_argument("--no-cpu-baseline", action="store_true")
  args = p.parse_args()
  if args.nworld is None:
    args.nworld = {"mesh_ibl": 4096, "path": 1024, "batched": 2048, "large_path": 8192}.get(args.workload, 16)
  if args.res is None:
    args.res = {"mesh_ibl": 128, "path": 128, "large_path": 256}.get(args.workload, 64)
  if args.steps is None:
    args.steps = 2000 if (args.workload == "primitives" and args.impl == "gb300") else 20
  args.warmup = max(args.warmup, 3) if args.impl == "gb300" else args.warmup
  if args.impl == "reference":
    run_reference(args)
  elif args.workload == "batched":
    run_batched(args)
  elif args.workload == "large_path":
    run_large(args)
  else:
    run(args)


if __name__ == "__main__":
  main()
