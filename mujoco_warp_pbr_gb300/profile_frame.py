"""Renders a few frames of one seeded synthetic workload, for profilers.

    python -m mujoco_warp_pbr_gb300.profile_frame mesh_ibl --nworld 256 --frames 3

Each frame is refit_bvh + render on the current stream, nothing else (no L2 flush, no timing, no
host copies), so a profiler's launch list holds the frame's own kernels and the DRAM counters of a
render launch count that launch's traffic only. Workloads: mesh_ibl (meshes, textures, IBL, mirror
floor, 2x2 supersamples), primitives, path (path-traced tier, 2 spp), hfield (terrain).
"""

from __future__ import annotations

import argparse

import torch

import mujoco_warp_pbr_gb300 as mjpbr
from mujoco_warp_pbr_gb300 import synthetic

SCENES = {
  "mesh_ibl": lambda n, r: synthetic.mesh_ibl_scene(nworld=n, res=r),
  "primitives": lambda n, r: synthetic.primitive_scene(nworld=n, res=r),
  "path": lambda n, r: synthetic.path_scene(nworld=n, res=r),
  "hfield": lambda n, r: synthetic.hfield_scene(nworld=n, res=r),
}


def main(argv: list[str] | None = None) -> None:
  p = argparse.ArgumentParser(description=__doc__.splitlines()[0])
  p.add_argument("workload", choices=sorted(SCENES))
  p.add_argument("--nworld", type=int, default=256)
  p.add_argument("--res", type=int, default=128)
  p.add_argument("--frames", type=int, default=3)
  args = p.parse_args(argv)
  sc = SCENES[args.workload](args.nworld, args.res)
  m = mjpbr.put_model(sc.mjm)
  d = mjpbr.put_data(sc.mjm, sc.mjd, nworld=sc.nworld)
  rc = mjpbr.create_render_context(sc.mjm, sc.nworld, data=sc.mjd, **sc.options)
  synthetic.apply_per_world(sc, m, rc)
  for _ in range(args.frames):
    mjpbr.refit_bvh(m, d, rc)
    mjpbr.render(m, d, rc)
  torch.cuda.synchronize()
  status = mjpbr.check_errors(rc)
  npix = sc.nworld * sum(w * h for w, h in rc.base.cam_res)
  print(f"{sc.name}: {args.frames} frames of {npix} pixels, error word {status}")
  if status != 0:
    raise SystemExit(1)


if __name__ == "__main__":
  main()
