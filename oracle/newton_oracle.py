"""CPU restatement of the Newton sensor adapter's per-frame steps — TEST INFRASTRUCTURE ONLY.

Checks the two kernels of mjpbr_newton_sync_poses / mjpbr_newton_images against plain NumPy:

  * sync_poses follows newton-pbr/newton_pbr/_render.py:31-77 (_sync_poses): geom g of world w
    shows shape s = geom_shape[w][g]; its pose is body_q[shape_body[s]] * shape_transform[s] *
    offset[g] (the body factor only for shape_body[s] >= 0), and world w's camera takes
    camera_transforms[w]. Transforms are Newton's: position, then a quaternion (x, y, z, w).
    Computed in float64.
  * images follows newton-pbr/newton_pbr/sensor.py:45-86 (_copy_outputs): colour in Newton's
    0xAABBGGRR packing, depth <= 0 -> -1, ray distance = planar depth * ray_scale (float32
    product), shape index = geom_shape[w][geom] for a geom hit (object type mjOBJ_GEOM = 5) else
    0xFFFFFFFF, HDR copied.
  * ray_scale follows sensor.py:168-173: sqrt(1 + x^2 + y^2) of the pinhole ray through each
    pixel centre at unit forward distance.

Shares no code with the product package. Only tests/ use this module.
"""

from __future__ import annotations

import numpy as np

OBJ_GEOM = 5


def quat_rotate(q: np.ndarray, v: np.ndarray) -> np.ndarray:
  """Rotates v (..., 3) by unit quaternions q (..., 4) (x, y, z, w): q v q*."""
  w = q[..., 3:4]
  u = q[..., :3]
  return v * (2.0 * w * w - 1.0) + np.cross(u, v) * 2.0 * w + u * 2.0 * np.sum(u * v, axis=-1, keepdims=True)


def quat_mul(a: np.ndarray, b: np.ndarray) -> np.ndarray:
  """Hamilton product of quaternions (x, y, z, w)."""
  av, aw = a[..., :3], a[..., 3:4]
  bv, bw = b[..., :3], b[..., 3:4]
  v = aw * bv + bw * av + np.cross(av, bv)
  w = aw * bw - np.sum(av * bv, axis=-1, keepdims=True)
  return np.concatenate([v, w], axis=-1)


def transform_multiply(a: np.ndarray, b: np.ndarray) -> np.ndarray:
  """a * b for transforms (..., 7): b's frame expressed in a's parent frame."""
  return np.concatenate([a[..., :3] + quat_rotate(a[..., 3:], b[..., :3]), quat_mul(a[..., 3:], b[..., 3:])], axis=-1)


def quat_to_matrix(q: np.ndarray) -> np.ndarray:
  """Row-major rotation matrices (..., 9) of unit quaternions (x, y, z, w): columns are the
  rotated basis vectors."""
  cols = [quat_rotate(q, np.broadcast_to(e, q.shape[:-1] + (3,))) for e in np.eye(3)]
  return np.stack(cols, axis=-1).reshape(*q.shape[:-1], 9)


def sync_poses(body_q: np.ndarray | None, shape_body: np.ndarray, shape_transform: np.ndarray, geom_shape: np.ndarray, geom_offset: np.ndarray, camera_transforms: np.ndarray) -> dict[str, np.ndarray]:
  """geom_xpos (nworld, ngeom, 3), geom_xmat (nworld, ngeom, 9), cam_xpos (nworld, 3), cam_xmat
  (nworld, 9) in float64. geom_shape (1 or nworld, ngeom); geom_offset (ngeom, 7)."""
  cams = np.asarray(camera_transforms, np.float64).reshape(-1, 7)
  nworld = len(cams)
  gs = np.asarray(geom_shape).reshape(-1, np.asarray(geom_shape).shape[-1])
  if len(gs) == 1:
    gs = np.broadcast_to(gs, (nworld, gs.shape[1]))
  shape_body = np.asarray(shape_body)
  shape_transform = np.asarray(shape_transform, np.float64).reshape(-1, 7)
  geom_offset = np.asarray(geom_offset, np.float64).reshape(-1, 7)
  x = shape_transform[gs]
  body = shape_body[gs]
  if body_q is not None and len(body_q):
    bq = np.asarray(body_q, np.float64).reshape(-1, 7)
    moving = body >= 0
    x[moving] = transform_multiply(bq[body[moving]], x[moving])
  x = transform_multiply(x, np.broadcast_to(geom_offset, x.shape))
  return {
    "geom_xpos": x[..., :3],
    "geom_xmat": quat_to_matrix(x[..., 3:]),
    "cam_xpos": cams[:, :3],
    "cam_xmat": quat_to_matrix(cams[:, 3:]),
  }


def ray_scale(width: int, height: int, fovy_deg: float) -> np.ndarray:
  """(height, width) float32 ratio of ray distance to forward depth through pixel centres."""
  t = np.tan(np.radians(fovy_deg) / 2.0)
  y = (1.0 - 2.0 * (np.arange(height) + 0.5) / height) * t
  x = (2.0 * (np.arange(width) + 0.5) / width - 1.0) * t * width / height
  return np.sqrt(1.0 + x[None, :] ** 2 + y[:, None] ** 2).astype(np.float32)


def images(rgba8: np.ndarray, depth: np.ndarray, seg: np.ndarray, hdr: np.ndarray, geom_shape: np.ndarray, scale: np.ndarray) -> dict[str, np.ndarray]:
  """Newton outputs of one camera: rgba8 (nworld, H, W, 4) uint8 channels r, g, b, a; depth
  (nworld, H, W) planar; seg (nworld, H, W, 2); hdr (nworld, H, W, 3); scale (H, W) float32."""
  c = rgba8.astype(np.uint32)
  color = (c[..., 3] << 24) | (c[..., 2] << 16) | (c[..., 1] << 8) | c[..., 0]
  fwd = np.where(depth <= 0.0, np.float32(-1.0), depth).astype(np.float32)
  ray = np.where(fwd > 0.0, fwd * scale[None], fwd).astype(np.float32)
  gs = np.asarray(geom_shape)
  nworld = depth.shape[0]
  rows = np.broadcast_to(gs, (nworld, gs.shape[-1])) if gs.shape[0] == 1 else gs
  gid, kind = seg[..., 0], seg[..., 1]
  hit = (gid >= 0) & (kind == OBJ_GEOM)
  w = np.broadcast_to(np.arange(nworld)[:, None, None], gid.shape)
  index = np.full(gid.shape, 0xFFFFFFFF, np.uint32)
  index[hit] = rows[w[hit], gid[hit]].astype(np.uint32)
  return {"color": color.astype(np.uint32), "forward_depth": fwd, "depth": ray, "shape_index": index, "hdr": hdr.astype(np.float32)}
