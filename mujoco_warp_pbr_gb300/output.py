"""Per-camera views of the render outputs (mujoco_warp_pbr/_src/output.py:34-152).

Outputs are torch tensors on the context's device: get_rgb (nworld_out, H, W, 3) float32 in
[0, 1], get_depth (nworld_out, H, W) float32 depth / depth_scale clamped to [0, 1],
get_segmentation (nworld_out, H, W, 2) int32, get_hdr / get_albedo / get_normal
(nworld_out, H, W, 3) float32. nworld_out may be smaller than nworld (the first worlds).
"""

from __future__ import annotations

import torch

from mujoco_warp_pbr_gb300 import _lib
from mujoco_warp_pbr_gb300.pbr_types import PbrRenderContext


def _check(rc: PbrRenderContext, camera_index: int, out: torch.Tensor, name: str, tail: tuple[int, ...], dtype: torch.dtype) -> None:
  res = rc.base.cam_res
  if not 0 <= camera_index < len(res):
    raise ValueError(f"camera_index must be in [0, {len(res)}), got {camera_index}")
  width, height = res[camera_index]
  shape = tuple(out.shape)
  if out.dim() != 3 + len(tail) or shape[0] > rc.nworld or shape[1:3] != (height, width) or shape[3:] != tail:
    raise ValueError(f"{name} must have shape (<= {rc.nworld}, {height}, {width}{''.join(f', {t}' for t in tail)}), got {shape}")
  if out.dtype != dtype or out.device != rc.device or not out.is_contiguous():
    raise ValueError(f"{name} must be a contiguous {dtype} tensor on {rc.device}")


def _scene(rc: PbrRenderContext) -> _lib.Scene:
  cached = rc._host_cache.get("scene")
  if cached is None:
    raise ValueError("render the context before reading its outputs")
  return cached[2]


def _stream(rc: PbrRenderContext) -> int:
  return torch.cuda.current_stream(rc.device).cuda_stream


def get_rgb(rc: PbrRenderContext, camera_index: int, rgb_out: torch.Tensor) -> None:
  """Writes display RGB in [0, 1] for one camera into rgb_out (nworld, height, width, 3)."""
  _check(rc, camera_index, rgb_out, "rgb_out", (3,), torch.float32)
  if rc.base.rgb_adr[camera_index] < 0:
    raise ValueError(f"camera {camera_index} renders no RGB")
  _lib.call("mjpbr_get_rgb", _scene(rc), camera_index, rgb_out.data_ptr(), rgb_out.shape[0], _stream(rc))


def get_depth(rc: PbrRenderContext, camera_index: int, depth_scale: float, depth_out: torch.Tensor) -> None:
  """Writes planar depth / depth_scale clamped to [0, 1] for one camera."""
  _check(rc, camera_index, depth_out, "depth_out", (), torch.float32)
  if rc.base.depth_adr[camera_index] < 0:
    raise ValueError(f"camera {camera_index} renders no depth")
  _lib.call("mjpbr_get_depth", _scene(rc), camera_index, float(depth_scale), depth_out.data_ptr(), depth_out.shape[0], _stream(rc))


def get_segmentation(rc: PbrRenderContext, camera_index: int, seg_out: torch.Tensor) -> None:
  """Writes per-pixel (object id, object type) for one camera; background is (-1, -1)."""
  _check(rc, camera_index, seg_out, "seg_out", (2,), torch.int32)
  if rc.base.seg_adr[camera_index] < 0:
    raise ValueError(f"camera {camera_index} renders no segmentation")
  _lib.call("mjpbr_get_segmentation", _scene(rc), camera_index, seg_out.data_ptr(), seg_out.shape[0], _stream(rc))


def get_hdr(rc: PbrRenderContext, camera_index: int, hdr_out: torch.Tensor) -> None:
  """Writes linear HDR radiance (before exposure) for one camera. Needs render_hdr=True.

  Raises:
    ValueError: without render_hdr, for a camera index out of range or a mismatched output.
  """
  if not rc.render_hdr:
    raise ValueError("create the render context with render_hdr=True to read HDR output")
  _check(rc, camera_index, hdr_out, "hdr_out", (3,), torch.float32)
  _lib.call("mjpbr_get_image", _scene(rc), 0, camera_index, hdr_out.data_ptr(), hdr_out.shape[0], _stream(rc))


def _guides(rc: PbrRenderContext) -> None:
  if not rc.render_guides:
    raise ValueError("create the render context with render_guides=True to read the albedo / normal guides")


def get_albedo(rc: PbrRenderContext, camera_index: int, albedo_out: torch.Tensor) -> None:
  """Writes the linear base colour of each pixel's first hit (zero: background). Needs
  render_guides=True."""
  _guides(rc)
  _check(rc, camera_index, albedo_out, "albedo_out", (3,), torch.float32)
  _lib.call("mjpbr_get_image", _scene(rc), 1, camera_index, albedo_out.data_ptr(), albedo_out.shape[0], _stream(rc))


def get_normal(rc: PbrRenderContext, camera_index: int, normal_out: torch.Tensor) -> None:
  """Writes the world-space shading normal of each pixel's first hit (zero: background). Needs
  render_guides=True."""
  _guides(rc)
  _check(rc, camera_index, normal_out, "normal_out", (3,), torch.float32)
  _lib.call("mjpbr_get_image", _scene(rc), 2, camera_index, normal_out.data_ptr(), normal_out.shape[0], _stream(rc))
