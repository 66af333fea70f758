"""Scenes of the reference's analytic known-answer tests, built with the synthetic Builder.

The reference expresses them as MJCF strings (its tests/test_render.py, test_ibl.py,
test_effects.py); here each is the same geometry, materials, lights and camera as arrays. The
`render` helper runs the CPU oracle (default) or the GPU library on the scene and returns one
camera's images as (nworld, H, W, ...) arrays.
"""

from __future__ import annotations

import numpy as np

from mujoco_warp_pbr_gb300 import synthetic
from mujoco_warp_pbr_gb300.synthetic import GEOM_BOX, GEOM_PLANE, GEOM_SPHERE, LIGHT_DIRECTIONAL, LIGHT_POINT, Builder
from oracle import oracle

TOP_CAMERA = {"pos": (0, 0, 2), "xyaxes": (1, 0, 0, 0, 1, 0), "fovy": 10.0}
FRONT_CAMERA = {"pos": (0, -3, 0), "xyaxes": (1, 0, 0, 0, 0, 1)}


def srgb(x):
  x = np.asarray(x, np.float64)
  return np.where(x <= 0.0031308, 12.92 * x, 1.055 * np.power(x, 1 / 2.4) - 0.055)


def plane_scene(material: dict, light: dict | None, res=(32, 32)) -> Builder:
  b = Builder()
  mat = b.material(**material)
  b.geom(GEOM_PLANE, (5, 5, 0.1), matid=mat)
  if light is not None:
    b.light(**light)
  b.camera(resolution=res, **TOP_CAMERA)
  return b


def sphere_scene(material: dict, fovy=5.0, headlight_ambient=None, res=(32, 32)) -> Builder:
  b = Builder()
  if headlight_ambient is not None:
    b.headlight_active = True
    b.headlight_ambient = headlight_ambient
    b.headlight_diffuse = (0.0, 0.0, 0.0)
    b.headlight_specular = (0.0, 0.0, 0.0)
  mat = b.material(**material)
  b.geom(GEOM_SPHERE, (0.5, 0, 0), matid=mat)
  b.camera(resolution=res, fovy=fovy, **FRONT_CAMERA)
  return b


def render(b: Builder, nworld: int = 1, seed: int = 0, per_world: dict | None = None, **options) -> dict[str, np.ndarray]:
  """Renders camera 0 with the oracle; returns rgb (float in [0,1]), hdr, depth, seg images."""
  mjm, mjd = b.build()
  options.setdefault("render_rgb", True)
  options.setdefault("render_depth", True)
  options.setdefault("render_seg", True)
  o = oracle.OracleScene(mjm, mjd, nworld, options, per_world or {})
  out = o.render(seed=seed)
  w, h = o.hc.outputs["cam_res"][0]
  npix = w * h
  rgb = oracle.unpack_rgb(out["rgb"][:, :npix]).reshape(nworld, h, w, 3) / 255.0
  return {
    "rgb": rgb,
    "hdr": out["hdr"][:, :npix].reshape(nworld, h, w, 3).copy(),
    "depth": out["depth"][:, :npix].reshape(nworld, h, w).copy(),
    "seg": out["seg"][:, :npix].reshape(nworld, h, w, 2).copy(),
    "exposure": float(o.hc.tables["exposure"][0]),
    "settings": dict(o.hc.settings),
  }


__all__ = ["GEOM_BOX", "GEOM_PLANE", "GEOM_SPHERE", "LIGHT_DIRECTIONAL", "LIGHT_POINT", "Builder", "plane_scene", "render", "sphere_scene", "srgb", "synthetic"]


def render_gpu(b: Builder, nworld: int = 1, seed: int = 0, per_world: dict | None = None, **options) -> dict[str, np.ndarray]:
  """As render(), through the public API of the GPU library."""
  import torch

  import mujoco_warp_pbr_gb300 as mjpbr

  mjm, mjd = b.build()
  options.setdefault("render_rgb", True)
  options.setdefault("render_depth", True)
  options.setdefault("render_seg", True)
  m = mjpbr.put_model(mjm)
  d = mjpbr.put_data(mjm, mjd, nworld=nworld)
  rc = mjpbr.create_render_context(mjm, nworld, data=mjd, **options)
  for name, value in (per_world or {}).items():
    owner = m if name in ("geom_rgba", "mat_emission") else rc
    setattr(owner, name, torch.as_tensor(np.asarray(value)).to(rc.device))
  mjpbr.refit_bvh(m, d, rc)
  mjpbr.render(m, d, rc, seed=seed)
  torch.cuda.synchronize()
  assert mjpbr.check_errors(rc) == 0
  w, h = rc.base.cam_res[0]
  rgb = torch.zeros((nworld, h, w, 3), device=rc.device)
  mjpbr.get_rgb(rc, 0, rgb)
  hdr = torch.zeros((nworld, h, w, 3), device=rc.device)
  if rc.render_hdr:
    mjpbr.get_hdr(rc, 0, hdr)
  seg = torch.zeros((nworld, h, w, 2), dtype=torch.int32, device=rc.device)
  mjpbr.get_segmentation(rc, 0, seg)
  depth = rc.base.depth_data[:, : w * h].reshape(nworld, h, w)
  return {
    "rgb": rgb.cpu().numpy(),
    "hdr": hdr.cpu().numpy(),
    "depth": depth.cpu().numpy(),
    "seg": seg.cpu().numpy(),
    "exposure": float(rc.exposure.reshape(-1)[0].item()),
    "settings": dict(rc._host_cache["settings"]),
  }
