"""A stand-in for the parts of the `newton` package the Newton adapter reads (Newton is not
installed here): GeoType, ShapeFlags, Mesh and a small ModelBuilder whose finalized Model carries
Newton's shape arrays (shape_type, shape_scale, shape_flags, shape_world, shape_body,
shape_transform, shape_source, shape_color, world_count, device, body_q) as torch tensors.

Enum members carry Newton's names; their integer values here are this stand-in's own (the
adapter maps shape types by name). Transforms are 7 floats: position, quaternion (x, y, z, w).
"""

from __future__ import annotations

import enum
import math
from typing import Any

import numpy as np
import torch


class GeoType(enum.IntEnum):
  PLANE = 0
  HFIELD = 1
  SPHERE = 2
  CAPSULE = 3
  ELLIPSOID = 4
  CYLINDER = 5
  BOX = 6
  MESH = 7
  SDF = 8
  CONE = 9
  CONVEX_MESH = 10


class ShapeFlags(enum.IntFlag):
  VISIBLE = 1
  COLLIDE_SHAPES = 2
  COLLIDE_PARTICLES = 4
  SITE = 8


class Mesh:
  def __init__(self, vertices: Any, indices: Any, normals: Any = None, uvs: Any = None, roughness: float | None = None, metallic: float | None = None, texture: Any = None):
    self.vertices = np.asarray(vertices, np.float32)
    self.indices = np.asarray(indices, np.int32).reshape(-1)
    self.normals = normals
    self.uvs = uvs
    self.roughness = roughness
    self.metallic = metallic
    self.texture = texture


def identity() -> tuple[float, ...]:
  return (0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 1.0)


def xform(pos: Any = (0.0, 0.0, 0.0), axis: Any = (0.0, 0.0, 1.0), angle: float = 0.0) -> tuple[float, ...]:
  a = np.asarray(axis, np.float64)
  a = a / np.linalg.norm(a)
  s = math.sin(angle / 2.0)
  return (*(float(p) for p in pos), float(a[0] * s), float(a[1] * s), float(a[2] * s), math.cos(angle / 2.0))


def quat_from_matrix(m: np.ndarray) -> tuple[float, float, float, float]:
  """(x, y, z, w) of a rotation matrix (columns = rotated axes), Shepperd's method."""
  m = np.asarray(m, np.float64).reshape(3, 3)
  tr = m[0, 0] + m[1, 1] + m[2, 2]
  if tr > 0:
    s = math.sqrt(tr + 1.0) * 2
    return ((m[2, 1] - m[1, 2]) / s, (m[0, 2] - m[2, 0]) / s, (m[1, 0] - m[0, 1]) / s, 0.25 * s)
  i = int(np.argmax([m[0, 0], m[1, 1], m[2, 2]]))
  j, k = (i + 1) % 3, (i + 2) % 3
  s = math.sqrt(1.0 + m[i, i] - m[j, j] - m[k, k]) * 2
  q = [0.0, 0.0, 0.0, 0.0]
  q[i] = 0.25 * s
  q[j] = (m[j, i] + m[i, j]) / s
  q[k] = (m[k, i] + m[i, k]) / s
  q[3] = (m[k, j] - m[j, k]) / s
  return tuple(q)  # type: ignore[return-value]


class Model:
  pass


class State:
  pass


class ModelBuilder:
  def __init__(self):
    self.body_q: list[tuple[float, ...]] = []
    self.shapes: list[dict[str, Any]] = []
    self.world_count = 0

  def add_body(self, xform: Any = None) -> int:
    self.body_q.append(tuple(xform) if xform is not None else identity())
    return len(self.body_q) - 1

  def _shape(self, body: int, gtype: GeoType, scale: Any, xform: Any, color: Any, source: Any = None, flags: int = ShapeFlags.VISIBLE | ShapeFlags.COLLIDE_SHAPES, opacity: float = 1.0) -> int:
    self.shapes.append(
      {"body": body, "type": int(gtype), "scale": tuple(float(s) for s in scale), "xform": tuple(xform) if xform is not None else identity(), "color": color, "source": source, "flags": int(flags), "opacity": opacity, "world": -1}
    )
    return len(self.shapes) - 1

  def add_shape_box(self, body: int, xform: Any = None, hx: float = 0.5, hy: float = 0.5, hz: float = 0.5, color: Any = None, **kw: Any) -> int:
    return self._shape(body, GeoType.BOX, (hx, hy, hz), xform, color, **kw)

  def add_shape_sphere(self, body: int, xform: Any = None, radius: float = 1.0, color: Any = None, **kw: Any) -> int:
    return self._shape(body, GeoType.SPHERE, (radius, 0.0, 0.0), xform, color, **kw)

  def add_shape_capsule(self, body: int, xform: Any = None, radius: float = 1.0, half_height: float = 0.5, color: Any = None, **kw: Any) -> int:
    return self._shape(body, GeoType.CAPSULE, (radius, half_height, 0.0), xform, color, **kw)

  def add_shape_cylinder(self, body: int, xform: Any = None, radius: float = 1.0, half_height: float = 0.5, color: Any = None, **kw: Any) -> int:
    return self._shape(body, GeoType.CYLINDER, (radius, half_height, 0.0), xform, color, **kw)

  def add_shape_cone(self, body: int, xform: Any = None, radius: float = 1.0, half_height: float = 0.5, color: Any = None, **kw: Any) -> int:
    return self._shape(body, GeoType.CONE, (radius, half_height, 0.0), xform, color, **kw)

  def add_shape_mesh(self, body: int, mesh: Mesh, xform: Any = None, scale: Any = (1.0, 1.0, 1.0), color: Any = None, **kw: Any) -> int:
    return self._shape(body, GeoType.MESH, scale, xform, color, source=mesh, **kw)

  def add_ground_plane(self, color: Any = None) -> int:
    return self._shape(-1, GeoType.PLANE, (0.0, 0.0, 0.0), None, color)

  def add_world(self, other: ModelBuilder) -> None:
    """Appends another builder's bodies and shapes as a new world."""
    offset = len(self.body_q)
    self.body_q.extend(other.body_q)
    for s in other.shapes:
      t = dict(s)
      t["body"] = s["body"] + offset if s["body"] >= 0 else -1
      t["world"] = self.world_count
      self.shapes.append(t)
    self.world_count += 1

  def replicate(self, other: ModelBuilder, n: int) -> None:
    for _ in range(n):
      self.add_world(other)

  def finalize(self, device: str = "cuda") -> Model:
    dev = torch.device(device)
    m = Model()
    sh = self.shapes
    m.device = dev
    m.world_count = max(self.world_count, 1)
    m.shape_type = torch.tensor([s["type"] for s in sh], dtype=torch.int32, device=dev)
    m.shape_scale = torch.tensor([s["scale"] for s in sh], dtype=torch.float32, device=dev).reshape(-1, 3)
    m.shape_flags = torch.tensor([s["flags"] for s in sh], dtype=torch.int32, device=dev)
    m.shape_world = torch.tensor([s["world"] for s in sh], dtype=torch.int32, device=dev)
    m.shape_body = torch.tensor([s["body"] for s in sh], dtype=torch.int32, device=dev)
    m.shape_transform = torch.tensor([s["xform"] for s in sh], dtype=torch.float32, device=dev).reshape(-1, 7)
    m.shape_source = [s["source"] for s in sh]
    colors = [s["color"] if s["color"] is not None else (0.7, 0.7, 0.7) for s in sh]
    m.shape_color = torch.tensor(colors, dtype=torch.float32, device=dev).reshape(-1, 3)
    m.shape_opacity = torch.tensor([s["opacity"] for s in sh], dtype=torch.float32, device=dev)
    m.body_q = torch.tensor(self.body_q, dtype=torch.float32, device=dev).reshape(-1, 7) if self.body_q else None

    def state() -> State:
      st = State()
      st.body_q = m.body_q.clone() if m.body_q is not None else None
      return st

    m.state = state
    return m


class _Module:
  """The stand-in as the module-like object the adapter's `newton=` argument takes."""

  GeoType = GeoType
  ShapeFlags = ShapeFlags
  Mesh = Mesh
  ModelBuilder = ModelBuilder


newton = _Module()
