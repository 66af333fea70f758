"""Shared helpers of the GPU tests: build a synthetic scene on the device and on the oracle."""

from __future__ import annotations

import numpy as np
import torch

import mujoco_warp_pbr_gb300 as mjpbr
from mujoco_warp_pbr_gb300 import synthetic
from oracle import oracle


def gpu_scene(sc: synthetic.SyntheticScene, **overrides):
  options = {**sc.options, **overrides}
  m = mjpbr.put_model(sc.mjm)
  d = mjpbr.put_data(sc.mjm, sc.mjd, nworld=sc.nworld)
  rc = mjpbr.create_render_context(sc.mjm, sc.nworld, data=sc.mjd, **options)
  synthetic.apply_per_world(sc, m, rc)
  return m, d, rc


def render_gpu(m, d, rc, seed: int = 0) -> dict[str, np.ndarray]:
  mjpbr.refit_bvh(m, d, rc)
  mjpbr.render(m, d, rc, seed=seed)
  torch.cuda.synchronize()
  assert mjpbr.check_errors(rc) == 0
  return {
    "rgb": rc.base.rgb_data.cpu().numpy().view(np.uint32),
    "depth": rc.base.depth_data.cpu().numpy(),
    "seg": rc.base.seg_data.cpu().numpy(),
    "hdr": rc.hdr_data.cpu().numpy(),
  }


def gpu_tables(rc) -> dict[str, np.ndarray]:
  t = {"dfg_lut": rc.dfg_lut.cpu().numpy()}
  if rc.tex_data is not None:
    t["tex_data"] = rc.tex_data.cpu().numpy()
  if rc.env is not None:
    t["env_data"] = rc.env.radiance_data.cpu().numpy()
    t["env_prefiltered"] = rc.env.prefiltered.cpu().numpy()
    t["env_sh"] = rc.env.sh.cpu().numpy()
    t["env_prob"] = rc.env.prob.cpu().numpy()
    t["env_marginal"] = rc.env.marginal.cpu().numpy()
    t["env_conditional"] = rc.env.conditional.cpu().numpy()
  return t


def oracle_render(sc: synthetic.SyntheticScene, seed: int = 0, tables=None, **overrides) -> dict[str, np.ndarray]:
  options = {**sc.options, **overrides}
  o = oracle.OracleScene(sc.mjm, sc.mjd, sc.nworld, options, sc.per_world, tables=tables)
  out = o.render(seed=seed)
  return {k: v.copy() for k, v in out.items()}


def rgb_diff(a: np.ndarray, b: np.ndarray) -> np.ndarray:
  return np.abs(oracle.unpack_rgb(a) - oracle.unpack_rgb(b)).max(axis=-1)
