"""Frame loops for profilers, and the per-stage time of the wavefront schedule.

    python -m mujoco_warp_pbr_gb300.profile_frame mesh_ibl --nworld 256 --frames 3
    python -m mujoco_warp_pbr_gb300.profile_frame mesh_ibl --nworld 512 --stages

Each frame is refit_bvh + render on the current stream, nothing else (no L2 flush, no timing, no
host copies), so a profiler's launch list holds the frame's own kernels and the DRAM counters of a
render launch count that launch's traffic only. With --stages the frames are timed instead and
the wavefront's stages are reported (wave_stage_ms: CUDA events the library records at every
stage boundary on the render stream, mjpbr_wave_profile_begin / _end). Workloads: mesh_ibl
(meshes, textures, IBL, mirror floor, 2x2 supersamples), primitives, path (path-traced tier,
2 spp), hfield (terrain), batched (three cameras of uneven size, a fisheye bundle, enable masks).
"""

from __future__ import annotations

import argparse
import ctypes
from typing import Any

import torch

import mujoco_warp_pbr_gb300 as mjpbr
from mujoco_warp_pbr_gb300 import _lib
from mujoco_warp_pbr_gb300 import synthetic

SCENES = {
  "mesh_ibl": lambda n, r: synthetic.mesh_ibl_scene(nworld=n, res=r),
  "primitives": lambda n, r: synthetic.primitive_scene(nworld=n, res=r),
  "path": lambda n, r: synthetic.path_scene(nworld=n, res=r),
  "hfield": lambda n, r: synthetic.hfield_scene(nworld=n, res=r),
  "batched": lambda n, r: synthetic.batched_scene(nworld=n),
}

# the wavefront's stages in launch order (include/mjpbr.h, mjpbr_wave_profile_end)
STAGES = ("primary", "surface", "mirror", "mirror_surface", "shadow", "resolve")


def wave_stage_ms(m: Any, d: Any, rc: Any, frames: int = 3, seed: int = 0) -> dict[str, float]:
  """Milliseconds per frame of each wavefront stage (summed over the frame's chunks of worlds)
  and of the whole render, from the CUDA events the library records at the stage boundaries
  (mjpbr_wave_profile_begin / _end). The context must use the wavefront schedule; the frames are
  rendered after one untimed frame."""
  if rc.tier != 0 or rc.schedule != 2 or rc.has_transparency:
    raise ValueError("wave_stage_ms needs a real-time context on the wavefront schedule")
  mjpbr.refit_bvh(m, d, rc)
  mjpbr.render(m, d, rc, seed=seed)
  torch.cuda.synchronize()
  stage = (ctypes.c_double * len(STAGES))()
  chunks = ctypes.c_int32(0)
  out = dict.fromkeys(STAGES, 0.0)
  start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  total = 0.0
  for f in range(frames):
    _lib.call("mjpbr_wave_profile_begin")
    start.record()
    mjpbr.render(m, d, rc, seed=seed + 1 + f)
    end.record()
    _lib.call("mjpbr_wave_profile_end", stage, ctypes.byref(chunks))
    end.synchronize()
    total += start.elapsed_time(end)
    for k, name in enumerate(STAGES):
      out[name] += stage[k]
  res = {k: v / frames for k, v in out.items()}
  res["render"] = total / frames
  res["chunks"] = int(chunks.value)
  return res


def main(argv: list[str] | None = None) -> None:
  p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
  p.add_argument("workload", choices=sorted(SCENES))
  p.add_argument("--nworld", type=int, default=256)
  p.add_argument("--res", type=int, default=128)
  p.add_argument("--frames", type=int, default=3)
  p.add_argument("--schedule", choices=["grid", "queue", "wavefront"], default=None)
  p.add_argument("--stages", action="store_true", help="time the wavefront's stages instead of looping")
  args = p.parse_args(argv)
  sc = SCENES[args.workload](args.nworld, args.res)
  m = mjpbr.put_model(sc.mjm)
  d = mjpbr.put_data(sc.mjm, sc.mjd, nworld=sc.nworld)
  opts = dict(sc.options)
  if args.schedule:
    opts["schedule"] = args.schedule
  rc = mjpbr.create_render_context(sc.mjm, sc.nworld, data=sc.mjd, **opts)
  synthetic.apply_per_world(sc, m, rc)
  npix = sc.nworld * sum(w * h for w, h in rc.base.cam_res)
  if args.stages:
    ms = wave_stage_ms(m, d, rc, frames=args.frames)
    parts = ", ".join(f"{k} {ms[k]:.2f}" for k in STAGES)
    print(f"{sc.name}: render {ms['render']:.2f} ms per frame ({npix / ms['render'] / 1e3:.1f} Mpix/s); stages (ms): {parts}")
    return
  for _ in range(args.frames):
    mjpbr.refit_bvh(m, d, rc)
    mjpbr.render(m, d, rc)
  torch.cuda.synchronize()
  status = mjpbr.check_errors(rc)
  print(f"{sc.name}: {args.frames} frames of {npix} pixels, error word {status}")
  if status != 0:
    raise SystemExit(1)


if __name__ == "__main__":
  main()
