"""Per-pixel camera rays (ray bundles) replacing the cameras' pinhole projection
(mujoco_warp_pbr/_src/rays.py:84-143).

Each rendering camera gets one camera-frame ray per pixel (MuJoCo's camera frame: -z forward, +y
up, +x right); ``rays[..., 0, :]`` is the origin and ``rays[..., 1, :]`` the direction (normalised
by the renderer; a zero direction marks a pixel without a ray). The render kernels place them in
each world by the camera's pose and interpolate them for sub-pixel samples.
"""

from __future__ import annotations

from collections.abc import Sequence
from typing import Any

import numpy as np
import torch

# Rays of every rendering camera: an array (nrender, height, width, 2, 3) when the cameras share a
# resolution, or one (height, width, 2, 3) array per rendering camera (NumPy or float32 torch);
# [..., 0, :] is the camera-frame origin, [..., 1, :] the direction (the reference's CameraRays
# alias, _src/rays.py:33-37).
CameraRays = np.ndarray | torch.Tensor | Sequence[np.ndarray | torch.Tensor]


def _images(camera_rays: Any) -> list[Any]:
  """The rays as one (height, width, 2, 3) array per camera (NumPy or torch)."""
  if isinstance(camera_rays, np.ndarray):
    if camera_rays.ndim != 5 or camera_rays.shape[-2:] != (2, 3):
      raise ValueError(f"camera_rays as a NumPy array must have shape (ncam, height, width, 2, 3), got {camera_rays.shape}")
    return list(camera_rays)
  if isinstance(camera_rays, torch.Tensor):
    if camera_rays.ndim == 5 and camera_rays.shape[-1] != 3:
      raise ValueError(f"camera rays must have dtype vec3 (a last dimension of 3), got shape {tuple(camera_rays.shape)}")
    if camera_rays.ndim != 5 or camera_rays.shape[-2] != 2:
      raise ValueError(f"camera_rays must have shape (ncam, height, width, 2, 3), got {tuple(camera_rays.shape)}")
    return list(camera_rays)
  if isinstance(camera_rays, Sequence):
    return list(camera_rays)
  raise TypeError(f"camera rays must be torch tensors or NumPy arrays, got {type(camera_rays).__name__}")


def _check_image(i: int, image: Any, width: int, height: int) -> None:
  if isinstance(image, np.ndarray):
    if image.ndim != 4 or image.shape[-2:] != (2, 3):
      raise ValueError(f"a camera's rays as a NumPy array must have shape (height, width, 2, 3), got {image.shape}")
  elif isinstance(image, torch.Tensor):
    if image.shape[-1:] != (3,) or image.dtype != torch.float32:
      raise ValueError(f"camera rays must have dtype vec3 (float32, last dimension 3), got {image.dtype} {tuple(image.shape)}")
  else:
    raise TypeError(f"camera rays must be torch tensors or NumPy arrays, got {type(image).__name__}")
  if tuple(image.shape[:3]) != (height, width, 2):
    raise ValueError(f"the rays of rendering camera {i} must have shape ({height}, {width}, 2) (its resolution), got {tuple(image.shape[:3])}")


def pack_camera_rays(camera_rays: Any, cam_res: Sequence[Sequence[int]]) -> tuple[np.ndarray, np.ndarray]:
  """Validated host copies: (origin, direction), each (total_rays, 3) float32, cameras in order."""
  images = _images(camera_rays)
  if len(images) != len(cam_res):
    raise ValueError(f"camera_rays must have rays for each of the {len(cam_res)} rendering cameras, got {len(images)}")
  origin, direction = [], []
  for i, (image, (width, height)) in enumerate(zip(images, cam_res)):
    _check_image(i, image, int(width), int(height))
    a = image.detach().cpu().numpy() if isinstance(image, torch.Tensor) else np.asarray(image, np.float32)
    a = a.reshape(-1, 2, 3).astype(np.float32)
    origin.append(a[:, 0])
    direction.append(a[:, 1])
  return np.ascontiguousarray(np.concatenate(origin)), np.ascontiguousarray(np.concatenate(direction))


def set_camera_rays(rc: Any, camera_rays: Any) -> None:
  """Renders the context's cameras from per-pixel rays instead of their pinhole projection.

  camera_rays: an array (nrender, height, width, 2, 3) when every rendering camera has the same
  resolution, or a sequence of one (height, width, 2, 3) array per rendering camera at its
  resolution (NumPy or float32 torch tensors); None renders the pinhole cameras again. With rays,
  depth is the distance along each ray and zfar bounds that distance; znear, fovy and intrinsics
  are not used. The rays are copied: call again after changing them.

  Raises ValueError for a camera count, resolution or dtype that does not match the context and
  TypeError for rays that are neither NumPy arrays nor torch tensors.
  """
  if camera_rays is None:
    rc.ray_origin = rc.ray_direction = rc.ray_res = None
    return
  cam_res = [tuple(int(v) for v in r) for r in rc.base.cam_res]
  origin, direction = pack_camera_rays(camera_rays, cam_res)
  total = int(rc.base.total_rays)
  if origin.shape[0] != total:
    raise ValueError(f"camera rays cover {origin.shape[0]} pixels, the rendering cameras {total}")
  if rc.ray_direction is None or rc.ray_direction.shape[0] != total:
    rc.ray_origin = torch.zeros((total, 3), dtype=torch.float32, device=rc.device)
    rc.ray_direction = torch.zeros((total, 3), dtype=torch.float32, device=rc.device)
  rc.ray_origin.copy_(torch.from_numpy(origin))
  rc.ray_direction.copy_(torch.from_numpy(direction))
  rc.ray_res = [list(r) for r in cam_res]


def pinhole_rays(width: int, height: int, fovy_deg: float) -> np.ndarray:
  """(height, width, 2, 3) camera-frame rays of a pinhole camera through the pixel centres."""
  h = np.tan(np.radians(fovy_deg) / 2.0)
  u = (np.arange(width) + 0.5) / width - 0.5
  v = (np.arange(height) + 0.5) / height - 0.5
  d = np.stack(np.broadcast_arrays(u[None, :] * 2.0 * h * width / height, -v[:, None] * 2.0 * h, -np.ones((1, 1))), axis=-1)
  d /= np.linalg.norm(d, axis=-1, keepdims=True)
  return np.stack([np.zeros_like(d), d], axis=2).astype(np.float32)


def fisheye_rays(width: int, height: int, fov_deg: float = 180.0) -> np.ndarray:
  """(height, width, 2, 3) rays of an equidistant fisheye: the angle from the optical axis grows
  linearly with the distance from the image centre, reaching fov / 2 on the inscribed circle;
  pixels outside that circle have no ray (zero direction)."""
  u = (np.arange(width) + 0.5) / width * 2.0 - 1.0
  v = 1.0 - (np.arange(height) + 0.5) / height * 2.0
  x, y = np.meshgrid(u * width / max(width, height), v * height / max(width, height))
  r = np.hypot(x, y)
  theta = r * np.radians(fov_deg) / 2.0
  phi = np.arctan2(y, x)
  d = np.stack([np.sin(theta) * np.cos(phi), np.sin(theta) * np.sin(phi), -np.cos(theta)], -1)
  d[r > 1.0] = 0.0
  return np.stack([np.zeros_like(d), d], axis=2).astype(np.float32)
