"""Newton sensor adapter: renders the worlds of a Newton model through this package.

Mirrors newton_pbr (newton-pbr/newton_pbr/sensor.py, _scene.py, _render.py): `build_scene` turns
a Newton model's visible shapes into this package's host model, `SensorPbrCamera` renders one
view per world with the interface of newton.sensors.SensorCamera.update, and the per-frame work
runs in two kernels of libmjpbr (mjpbr_newton_sync_poses: geom and camera poses from Newton's
body transforms; mjpbr_newton_images: outputs in Newton's formats) around refit_bvh and render.

Newton is not a dependency. The adapter reads a Newton model and state by attribute (model:
shape_type, shape_scale, shape_flags, shape_world, shape_body, shape_transform, shape_source,
shape_color, shape_opacity, world_count, device; state: body_q) and takes Newton's enums and mesh
class (GeoType, ShapeFlags, Mesh) from the `newton` module, or from the module-like object passed
as `newton=`. Device arrays may be Warp arrays or torch tensors (anything exposing
__cuda_array_interface__); host reads use .numpy().

Differences from newton_pbr, by design:
  * No MuJoCo compiler: meshes keep Newton's vertices (no re-centring), so every geom offset is
    the identity; a mesh without normals gets area-weighted vertex normals, except at face corners
    whose face normal is more than ~37 degrees (cosine 0.8) from the vertex normal, which take
    the face normal (a crease rule like MuJoCo's default non-smooth normals).
  * Mesh textures must be image arrays: texture files are not decoded (no image decoder here).
  * Output images are torch tensors (uint32 words as torch.uint32 views of int32 storage) or any
    device array of the right shape and dtype.
"""

from __future__ import annotations

import dataclasses
import importlib
import math
import warnings
from typing import Any, Literal

import numpy as np
import torch

from mujoco_warp_pbr_gb300 import _lib
from mujoco_warp_pbr_gb300.context import create_render_context
from mujoco_warp_pbr_gb300.model import HostData
from mujoco_warp_pbr_gb300.model import HostModel
from mujoco_warp_pbr_gb300.model import put_data
from mujoco_warp_pbr_gb300.model import put_model
from mujoco_warp_pbr_gb300.render import refit_bvh
from mujoco_warp_pbr_gb300.render import render
from mujoco_warp_pbr_gb300.render import scene as scene_descriptor
from mujoco_warp_pbr_gb300.synthetic import Builder

# MuJoCo geom and light types of the host model.
_GEOM_PLANE, _GEOM_SPHERE, _GEOM_CAPSULE, _GEOM_ELLIPSOID, _GEOM_CYLINDER, _GEOM_BOX, _GEOM_MESH = 0, 2, 3, 4, 5, 6, 7
_PRIMITIVE_NAMES = {"PLANE": _GEOM_PLANE, "SPHERE": _GEOM_SPHERE, "CAPSULE": _GEOM_CAPSULE, "ELLIPSOID": _GEOM_ELLIPSOID, "CYLINDER": _GEOM_CYLINDER, "BOX": _GEOM_BOX}
_MESH_NAMES = ("MESH", "CONVEX_MESH", "CONE")
_DEFAULT_COLOR = (0.7, 0.7, 0.7)
_CONE_SEGMENTS = 32
_CREASE_COSINE = 0.8
# create_render_context options the sensor sets itself.
_RESERVED_OPTIONS = ("nworld", "cam_res", "render_rgb", "render_hdr")

LightType = Literal["directional", "point", "spot"]
_LIGHT_TYPES = {"spot": 0, "directional": 1, "point": 2}

# (ambient, diffuse, specular) RGB of MuJoCo's headlight.
Headlight = tuple[Any, Any, Any]


def srgb_to_linear(c: Any) -> np.ndarray:
  """Display (sRGB) values in [0, 1] to linear (Newton shape colours are display values)."""
  c = np.asarray(c, dtype=np.float64)
  return np.where(c <= 0.04045, c / 12.92, ((c + 0.055) / 1.055) ** 2.4)


@dataclasses.dataclass
class Light:
  """A light added to the scene (Newton models carry no lights).

  Attributes:
    type: "directional", "point" or "spot".
    pos: position [m] (point / spot).
    dir: direction the light travels (directional / spot).
    intensity: lux (directional) or candela (point / spot); 0 uses the renderer's calibrated
      fallback for MuJoCo-style scenes.
    color: linear RGB colour.
    range: falloff radius [m] (point / spot).
    cutoff: spot cone half-angle [deg].
    bulb_radius: emitter radius [m] for soft shadows.
    cast_shadow: whether the light casts ray-traced shadows.
  """

  type: LightType = "directional"
  pos: tuple = (0.0, 0.0, 3.0)
  dir: tuple = (-0.3, 0.4, -1.0)
  intensity: float = 0.0
  color: tuple = (1.0, 1.0, 1.0)
  range: float = 100.0
  cutoff: float = 45.0
  bulb_radius: float = 0.0
  cast_shadow: bool = True

  def __post_init__(self):
    if self.type not in _LIGHT_TYPES:
      raise ValueError(f"Light.type must be one of {list(_LIGHT_TYPES)}, got {self.type!r}")


def lights_from_mujoco(mjm: Any, mjd: Any) -> list[Light]:
  """The active lights of a MuJoCo model (an MjModel or a HostModel) at state mjd, to keep an
  MJCF scene's lighting when it is loaded into Newton (whose importer drops lights)."""
  names = {v: k for k, v in _LIGHT_TYPES.items()}
  xpos = np.asarray(mjd.light_xpos, dtype=np.float64).reshape(-1, 3)
  xdir = np.asarray(mjd.light_xdir, dtype=np.float64).reshape(-1, 3)
  lights = []
  for i in range(len(np.asarray(mjm.light_type))):
    kind = int(mjm.light_type[i])
    if not mjm.light_active[i] or kind not in names:
      continue
    lights.append(
      Light(
        type=names[kind],
        pos=tuple(float(v) for v in xpos[i]),
        dir=tuple(float(v) for v in xdir[i]),
        intensity=float(mjm.light_intensity[i]),
        color=tuple(float(v) for v in np.asarray(mjm.light_diffuse[i]).reshape(3)),
        range=float(mjm.light_range[i]),
        cutoff=float(mjm.light_cutoff[i]),
        bulb_radius=float(mjm.light_bulbradius[i]),
        cast_shadow=bool(mjm.light_castshadow[i]),
      )
    )
  return lights


def default_lights() -> list[Light]:
  """A key light with shadows and a dim fill, for scenes without an environment map."""
  return [
    Light("directional", dir=(-0.4, 0.5, -0.75), color=(1.0, 0.97, 0.92)),
    Light("directional", dir=(0.5, -0.3, -0.6), color=(0.25, 0.27, 0.3), cast_shadow=False),
  ]


@dataclasses.dataclass(frozen=True)
class Checkerboard:
  """Grey checkerboard texture (Newton's checkerboard material colours) on the given shapes.

  Attributes:
    shapes: indices of the textured shapes.
    resolution: texture size [px] (square).
    checker_size: size of a checker square [px].
  """

  shapes: frozenset[int]
  resolution: int = 64
  checker_size: int = 32

  def image(self) -> np.ndarray:
    cell = np.arange(self.resolution) // self.checker_size
    grey = np.where((cell[:, None] + cell[None, :]) % 2 == 0, 0x80, 0xBF).astype(np.uint8)
    return np.repeat(grey[..., None], 3, axis=-1)


@dataclasses.dataclass
class SceneMapping:
  """Host model of a Newton scene plus the Newton shape behind every geom.

  Attributes:
    mjm: host model (one world; MuJoCo field names).
    mjd: host data of world 0 at the model's initial transforms (seeds the scene BVH topology).
    geom_shape: Newton shape index of geom g in world w (one row with merge_worlds) (nrow, ngeom).
    geom_offset_pos: pose of the geom frame in the Newton shape frame (ngeom, 3); zero here.
    geom_offset_quat: (w, x, y, z) (ngeom, 4); identity here.
  """

  mjm: HostModel
  mjd: HostData
  geom_shape: np.ndarray
  geom_offset_pos: np.ndarray
  geom_offset_quat: np.ndarray


def _newton_module(newton: Any) -> Any:
  if newton is not None:
    return newton
  try:
    return importlib.import_module("newton")
  except ImportError as e:
    raise ImportError("the Newton adapter needs the newton package, or a module-like object with GeoType, ShapeFlags and Mesh passed as newton=") from e


def _host(a: Any) -> np.ndarray | None:
  if a is None:
    return None
  if isinstance(a, np.ndarray):
    return a
  if isinstance(a, torch.Tensor):
    return a.detach().cpu().numpy()
  if hasattr(a, "numpy"):
    return np.asarray(a.numpy())
  return np.asarray(a)


def _required(value: Any, name: str) -> Any:
  if value is None:
    raise ValueError(f"newton_pbr: the Newton model has no {name}; pass a finalized newton.Model")
  return value


def _quat_xyzw_to_mat(q: np.ndarray) -> np.ndarray:
  x, y, z, w = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
  return np.stack(
    [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w), 2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w), 2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
    axis=-1,
  )


def _compose(a: np.ndarray, b: np.ndarray) -> np.ndarray:
  """Newton transforms (..., 7): position, quaternion (x, y, z, w); a * b."""
  ap, aq, bp, bq = a[..., :3], a[..., 3:], b[..., :3], b[..., 3:]
  u, w = aq[..., :3], aq[..., 3:]
  t = 2.0 * np.cross(u, bp)
  p = ap + bp + w * t + np.cross(u, t)
  x1, y1, z1, w1 = aq[..., 0], aq[..., 1], aq[..., 2], aq[..., 3]
  x2, y2, z2, w2 = bq[..., 0], bq[..., 1], bq[..., 2], bq[..., 3]
  q = np.stack([w1 * x2 + x1 * w2 + y1 * z2 - z1 * y2, w1 * y2 - x1 * z2 + y1 * w2 + z1 * x2, w1 * z2 + x1 * y2 - y1 * x2 + z1 * w2, w1 * w2 - x1 * x2 - y1 * y2 - z1 * z2], axis=-1)
  return np.concatenate([p, q], axis=-1)


def crease_normals(vert: np.ndarray, face: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
  """Normals of a mesh without normals: (normals, per-corner normal indices). Corners whose face
  normal is within the crease angle of the area-weighted vertex normal use the vertex normal
  (index = vertex), the others their face's normal (index nvert + face)."""
  v = np.asarray(vert, np.float64)
  f = np.asarray(face, np.int64).reshape(-1, 3)
  fn = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
  vn = np.zeros_like(v)
  for k in range(3):
    np.add.at(vn, f[:, k], fn)
  vn /= np.maximum(np.linalg.norm(vn, axis=1, keepdims=True), 1e-12)
  fu = fn / np.maximum(np.linalg.norm(fn, axis=1, keepdims=True), 1e-12)
  cos = np.einsum("fkc,fc->fk", vn[f], fu)
  corner = np.where(cos >= _CREASE_COSINE, f, len(v) + np.arange(len(f))[:, None])
  return np.concatenate([vn, fu]).astype(np.float32), corner.astype(np.int32)


def _cone_mesh(radius: float, half_height: float) -> tuple[np.ndarray, np.ndarray]:
  """A cone along +Z: a ring of _CONE_SEGMENTS vertices at -half_height, the apex, the base centre."""
  n = _CONE_SEGMENTS
  angles = 2.0 * np.pi * np.arange(n) / n
  ring = np.stack([radius * np.cos(angles), radius * np.sin(angles), np.full(n, -half_height)], axis=1)
  vert = np.concatenate([ring, [[0.0, 0.0, half_height], [0.0, 0.0, -half_height]]])
  i = np.arange(n)
  side = np.stack([i, (i + 1) % n, np.full(n, n)], axis=1)
  base = np.stack([(i + 1) % n, i, np.full(n, n + 1)], axis=1)
  return vert, np.concatenate([side, base])


def _texture_rgba(texture: Any) -> np.ndarray | None:
  """A Newton mesh texture (image array, uint8 or float in [0, 1]) as RGBA8 (h, w, 4)."""
  if texture is None:
    return None
  if isinstance(texture, (str, bytes)) or hasattr(texture, "__fspath__"):
    raise TypeError("newton_pbr: mesh texture files are not decoded here; load the image and set the mesh's texture to the array")
  image = np.asarray(texture)
  if image.dtype != np.uint8:
    image = (np.clip(image, 0.0, 1.0) * 255.0 + 0.5).astype(np.uint8)
  if image.ndim == 2:
    image = image[..., None]
  if image.shape[-1] == 1:
    image = np.repeat(image, 3, axis=-1)
  rgba = np.full((*image.shape[:2], 4), 255, np.uint8)
  rgba[..., :3] = image[..., :3]
  return rgba


def _same_source(a: Any, b: Any) -> bool:
  if a is b:
    return True
  if a is None or b is None:
    return False
  return np.array_equal(_host(a.vertices), _host(b.vertices)) and np.array_equal(_host(a.indices), _host(b.indices))


def _check_worlds(model: Any, per_world: list[np.ndarray], shape_type: np.ndarray, shape_scale: np.ndarray, mesh_types: set[int]) -> None:
  """Raises unless every world has the same visible shapes as world 0 (type, size, mesh)."""
  first = per_world[0]
  for w, shapes in enumerate(per_world[1:], start=1):
    if len(shapes) != len(first):
      raise ValueError(f"newton_pbr needs every world to have the same visible shapes: world {w} has {len(shapes)}, world 0 {len(first)}")
    for a, b in zip(first, shapes, strict=True):
      same = shape_type[a] == shape_type[b] and np.allclose(shape_scale[a], shape_scale[b])
      if same and int(shape_type[a]) in mesh_types:
        same = _same_source(model.shape_source[a], model.shape_source[b])
      if not same:
        raise ValueError(f"newton_pbr needs every world to have the same visible shapes: shape {b} of world {w} differs from shape {a} of world 0 (type, scale or mesh)")


def build_scene(
  model: Any,
  lights: list[Light] | None,
  camera_fovy: float,
  headlight: Headlight | None = None,
  merge_worlds: bool = False,
  checkerboard: Checkerboard | None = None,
  load_textures: bool = True,
  newton: Any = None,
) -> SceneMapping:
  """Host model of a Newton model's appearance (newton-pbr/newton_pbr/_scene.py build_scene).

  The model holds one world's visible shapes plus the global ones (shape_world < 0), and every
  world must have the same visible shapes; geom_shape maps each geom to each world's shape. With
  merge_worlds it holds every world's shapes at once (geom_shape has one row). Shapes become
  geoms with their size (Newton plane extents are full sizes, MuJoCo's half sizes), sRGB colour
  made linear, opacity, and for meshes the mesh's UVs, base-colour texture and scalar metallic /
  roughness; one host mesh per (Newton mesh, scale); cones are meshed. Poses come from Newton
  every frame (SensorPbrCamera.update).

  Raises:
    ValueError: when worlds differ (without merge_worlds) or the model lacks a required array.
    TypeError: for a mesh shape without a Mesh source, or a texture given as a file.
  """
  nt = _newton_module(newton)
  geo = nt.GeoType
  primitives = {int(getattr(geo, k)): v for k, v in _PRIMITIVE_NAMES.items() if hasattr(geo, k)}
  mesh_types = {int(getattr(geo, k)) for k in _MESH_NAMES if hasattr(geo, k)}
  cone = int(geo.CONE) if hasattr(geo, "CONE") else None
  shape_world = np.asarray(_host(_required(model.shape_world, "shape_world")), np.int64)
  shape_type = np.asarray(_host(_required(model.shape_type, "shape_type")), np.int64)
  shape_scale = np.asarray(_host(_required(model.shape_scale, "shape_scale")), np.float64).reshape(-1, 3)
  shape_flags = np.asarray(_host(_required(model.shape_flags, "shape_flags")), np.int64)
  shape_xform = np.asarray(_host(_required(model.shape_transform, "shape_transform")), np.float64).reshape(-1, 7)
  shape_body = np.asarray(_host(_required(model.shape_body, "shape_body")), np.int64)
  color_arr = _host(getattr(model, "shape_color", None))
  opacity_arr = _host(getattr(model, "shape_opacity", None))
  nworld = max(int(model.world_count), 1)

  visible = (shape_flags & int(nt.ShapeFlags.VISIBLE)) != 0
  if hasattr(nt.ShapeFlags, "SITE"):
    visible &= (shape_flags & int(nt.ShapeFlags.SITE)) == 0
  skipped = sorted({geo(int(t)).name for t in shape_type[visible] if int(t) not in primitives and int(t) not in mesh_types})
  if skipped:
    warnings.warn(f"newton_pbr: shape types {skipped} are not rendered", stacklevel=3)
  renderable = visible & np.isin(shape_type, list(primitives) + list(mesh_types))
  global_shapes = np.flatnonzero(renderable & (shape_world < 0))
  per_world = [np.flatnonzero(renderable & (shape_world == w)) for w in range(nworld)]
  if merge_worlds:
    shapes0 = np.flatnonzero(renderable)
  else:
    _check_worlds(model, per_world, shape_type, shape_scale, mesh_types - ({cone} if cone is not None else set()))
    shapes0 = np.concatenate([per_world[0], global_shapes])
  checkered = set() if checkerboard is None else {int(s) for s in checkerboard.shapes}

  # Initial world-frame transforms of the shapes (the model's body_q, when it has one).
  body_q = _host(getattr(model, "body_q", None))
  initial = shape_xform.copy()
  if body_q is not None and len(shape_body):
    body_q = np.asarray(body_q, np.float64).reshape(-1, 7)
    moving = (shape_body >= 0) & (shape_body < len(body_q))
    initial[moving] = _compose(body_q[shape_body[moving]], shape_xform[moving])

  b = Builder()
  if headlight is not None:
    ambient, diffuse, specular = (tuple(float(c) for c in np.asarray(h, np.float64).reshape(3)) for h in headlight)
    b.headlight_active, b.headlight_ambient, b.headlight_diffuse, b.headlight_specular = True, ambient, diffuse, specular
  mesh_ids: dict[tuple, int] = {}
  for i, shape in enumerate(shapes0.tolist()):
    gtype = int(shape_type[shape])
    scale = shape_scale[shape]
    color = srgb_to_linear(color_arr[shape][:3] if color_arr is not None else _DEFAULT_COLOR)
    alpha = float(opacity_arr[shape]) if opacity_arr is not None else 1.0
    rgba = (*color.tolist(), alpha)
    mat: dict[str, Any] = {"rgba": rgba}
    texid: dict[int, int] = {}
    pos = initial[shape, :3]
    rot = _quat_xyzw_to_mat(initial[shape, 3:])
    if gtype in primitives:
      size = [0.5 * scale[0], 0.5 * scale[1], 0.1] if primitives[gtype] == _GEOM_PLANE else scale
      geom_type, dataid = primitives[gtype], -1
    else:
      source = None
      uv = normal = None
      if gtype == cone:
        vert, face = _cone_mesh(float(scale[0]), float(scale[1]))
      else:
        source = model.shape_source[shape]
        if not isinstance(source, nt.Mesh):
          raise TypeError(f"newton_pbr: mesh shape {shape} has no newton.Mesh source (got {type(source).__name__})")
        vert = np.asarray(_host(source.vertices), np.float64).reshape(-1, 3) * scale
        face = np.asarray(_host(source.indices), np.int64).reshape(-1, 3)
        uv = _host(getattr(source, "uvs", None))
        normal = _host(getattr(source, "normals", None))
        if uv is not None and len(uv) != len(vert):
          uv = None  # per-vertex UVs only
        if normal is not None and len(normal) != len(vert):
          normal = None
      key = ("cone" if source is None else id(source), *scale.tolist())
      if key not in mesh_ids:
        if normal is not None:
          mesh_ids[key] = b.mesh(vert, face, normal=np.asarray(normal, np.float32), texcoord=uv)
        else:
          n, corner = crease_normals(vert, face)
          mesh_ids[key] = b.mesh(vert, face, normal=n, texcoord=uv, facenormal=corner)
      geom_type, dataid, size = _GEOM_MESH, mesh_ids[key], np.zeros(3)
      if source is not None:
        if getattr(source, "roughness", None) is not None:
          mat["roughness"] = float(source.roughness)
        if getattr(source, "metallic", None) is not None:
          mat["metallic"] = float(source.metallic)
        image = _texture_rgba(getattr(source, "texture", None)) if uv is not None and load_textures else None
        if image is not None and shape not in checkered:
          texid[1] = b.texture(image)  # base-colour role; the texture replaces the shape colour
          rgba = (1.0, 1.0, 1.0, alpha)
          mat["rgba"] = rgba
    if shape in checkered and checkerboard is not None:
      rgb = checkerboard.image()
      texid[1] = b.texture(np.concatenate([rgb, np.full((*rgb.shape[:2], 1), 255, np.uint8)], axis=-1))
    matid = b.material(texid=texid or None, **mat)
    b.geom(geom_type, size, pos=pos, mat=rot, rgba=rgba, matid=matid, dataid=dataid)

  for light in lights if lights is not None else []:
    d = np.asarray(light.dir, np.float64)
    b.light(
      _LIGHT_TYPES[light.type],
      pos=light.pos,
      dir=d if np.linalg.norm(d) > 0 else (0.0, 0.0, -1.0),
      diffuse=light.color,
      intensity=light.intensity,
      range=light.range,
      cutoff=light.cutoff,
      bulbradius=light.bulb_radius,
      castshadow=light.cast_shadow,
    )
  # Placeholder camera: its pose is written from Newton's camera transforms every frame.
  b.camera(pos=(0.0, 0.0, 0.0), xyaxes=(1.0, 0.0, 0.0, 0.0, 1.0, 0.0), fovy=camera_fovy)
  mjm, mjd = b.build()
  ngeom = mjm.ngeom
  if merge_worlds:
    geom_shape = shapes0[None].astype(np.int32)
  else:
    geom_shape = np.stack([np.concatenate([per_world[w], global_shapes]) for w in range(nworld)]).astype(np.int32).reshape(nworld, ngeom)
  return SceneMapping(mjm, mjd, geom_shape, np.zeros((ngeom, 3)), np.tile([1.0, 0.0, 0.0, 0.0], (ngeom, 1)))


_DTYPES = {"f4": (torch.float32, "<f4"), "i4": (torch.int32, "<i4"), "u4": (torch.uint32, "<u4")}


def _torch_typestr(dtype: torch.dtype) -> str | None:
  for _, (t, s) in _DTYPES.items():
    if t == dtype:
      return s
  return None


def device_view(a: Any, name: str, shape: tuple[int, ...], typestrs: tuple[str, ...], device: torch.device) -> int:
  """Device pointer of a C-contiguous device array (a torch tensor or an object exposing
  __cuda_array_interface__) holding exactly `shape` elements of one of `typestrs` ("<f4" ...);
  trailing vector dimensions may be folded into the last one (a Warp transformf array of n is
  (n, 7) floats).

  Raises:
    ValueError: for another shape, element type, device or a strided array.
  """
  if isinstance(a, torch.Tensor):
    ok = a.is_cuda and a.device == device and a.is_contiguous() and _torch_typestr(a.dtype) in typestrs
    got = f"{a.dtype} {tuple(a.shape)} on {a.device}"
    ashape, ptr = tuple(a.shape), a.data_ptr()
  else:
    iface = getattr(a, "__cuda_array_interface__", None)
    if iface is None:
      raise ValueError(f"{name} must be a CUDA array (torch tensor or __cuda_array_interface__), got {type(a).__name__}")
    ashape, typestr, strides = tuple(iface["shape"]), iface["typestr"], iface.get("strides")
    contiguous = strides is None or tuple(strides) == tuple(int(np.prod(ashape[k + 1 :])) * int(typestr[-1]) for k in range(len(ashape)))
    ok = typestr in typestrs and contiguous
    got = f"{typestr} {ashape}"
    ptr = int(iface["data"][0])
  n = int(np.prod(shape))
  if not ok or int(np.prod(ashape)) != n or ashape[: len(shape) - 1] != shape[:-1]:
    raise ValueError(f"{name} must be a contiguous {'/'.join(typestrs)} CUDA array of shape {shape} on {device}, got {got}")
  return ptr


class SensorPbrCamera:
  """Physically based camera sensor for a Newton model (newton-pbr/newton_pbr/sensor.py).

  One view per world; camera transforms place a camera that looks along its local -Z axis with
  +Y up; outputs have shape (world_count, height, width) in Newton's formats: packed RGBA colour
  0xAABBGGRR (uint32), ray-distance and forward depth with -1 for no hit, shape indices with
  0xFFFFFFFF for no hit, linear HDR (world_count, height, width, 3). The pinhole image size and
  field of view are fixed at construction.

  Appearance comes from the Newton model (shape colours and opacities, mesh base-colour textures,
  scalar metallic / roughness). Newton models carry no lights: pass `envmap` for image-based
  lighting and / or `lights`; without either, default_lights() are used.

  Example::

      camera = SensorPbrCamera(model, width=128, height=128, fovy=60.0, envmap=image)
      color = camera.allocate_image_color()
      camera.update(state, camera_transforms, color_image=color)
  """

  Light = Light

  def __init__(
    self,
    model: Any,
    *,
    width: int,
    height: int,
    fovy: float = 60.0,
    lights: list[Light] | None = None,
    envmap: Any = None,
    headlight: Headlight | None = None,
    newton: Any = None,
    **render_options: Any,
  ):
    """Builds the host model and the render context.

    Args:
      model: Newton model; every world must have the same visible shapes.
      width, height: image size [px].
      fovy: vertical field of view [deg].
      lights: lights added to the scene; None uses default_lights() when no envmap is given.
      envmap: equirectangular HDR environment (path or array) lighting the scene.
      headlight: None (off) or (ambient, diffuse, specular) RGB of MuJoCo's camera headlight.
      newton: module-like object with GeoType, ShapeFlags and Mesh (default: import newton).
      **render_options: further create_render_context options (tier, samples_per_pixel,
        light_model, envmap_intensity, ...); not nworld, cam_res, render_rgb or render_hdr.

    Raises:
      TypeError: for a render option the sensor sets itself.
      ValueError: when the worlds do not have the same visible shapes.
    """
    reserved = [name for name in _RESERVED_OPTIONS if name in render_options]
    if reserved:
      raise TypeError(f"SensorPbrCamera sets {reserved} itself; remove them from the render options")
    self.model = model
    self.width = int(width)
    self.height = int(height)
    if lights is None and envmap is None:
      lights = default_lights()
    self.scene = build_scene(model, lights, fovy, headlight, newton=newton)
    self.mjm = self.scene.mjm
    self.nworld = max(int(model.world_count), 1)
    self.device = self._device(model)
    self.m = put_model(self.mjm, device=self.device)
    self.d = put_data(self.mjm, self.scene.mjd, nworld=self.nworld, device=self.device)
    if envmap is not None:
      render_options.setdefault("envmap", envmap)
    render_options.setdefault("render_depth", True)
    render_options.setdefault("render_seg", True)
    self.rc = create_render_context(
      self.mjm, nworld=self.nworld, cam_res=(self.width, self.height), render_rgb=True, render_hdr=True, data=self.scene.mjd, device=self.device, **render_options
    )
    ngeom = self.mjm.ngeom
    self.geom_shape = torch.as_tensor(self.scene.geom_shape, dtype=torch.int32).to(self.device).contiguous()
    offset = np.concatenate([self.scene.geom_offset_pos, self.scene.geom_offset_quat[:, [1, 2, 3, 0]]], axis=1).reshape(ngeom, 7)
    self.geom_offset = torch.as_tensor(offset, dtype=torch.float32).to(self.device).contiguous()
    # Ray distance / forward depth per pixel (pinhole through pixel centres).
    tan = math.tan(math.radians(fovy) / 2.0)
    ys = (1.0 - 2.0 * (np.arange(self.height) + 0.5) / self.height) * tan
    xs = (2.0 * (np.arange(self.width) + 0.5) / self.width - 1.0) * tan * self.width / self.height
    scale = np.sqrt(1.0 + xs[None, :] ** 2 + ys[:, None] ** 2)
    self.ray_scale = torch.as_tensor(scale, dtype=torch.float32).to(self.device).contiguous()
    self._no_bodies = torch.zeros(7, dtype=torch.float32, device=self.device)

  @staticmethod
  def _device(model: Any) -> torch.device:
    dev = getattr(model, "device", None)
    if dev is None:
      return torch.device("cuda", torch.cuda.current_device())
    dev = torch.device(str(dev))
    if dev.type != "cuda":
      raise ValueError(f"SensorPbrCamera renders on a CUDA device; the model is on {dev}")
    return dev if dev.index is not None else torch.device("cuda", torch.cuda.current_device())

  def _image(self, dtype: torch.dtype, tail: tuple[int, ...] = ()) -> torch.Tensor:
    shape = (self.nworld, self.height, self.width, *tail)
    if dtype == torch.uint32:  # int32 storage viewed as uint32: no uint32 kernel is needed
      return torch.zeros(shape, dtype=torch.int32, device=self.device).view(torch.uint32)
    return torch.zeros(shape, dtype=dtype, device=self.device)

  def allocate_image_color(self) -> torch.Tensor:
    """Packed RGBA colour image (Newton layout), shape (world_count, height, width) uint32."""
    return self._image(torch.uint32)

  def allocate_image_depth(self) -> torch.Tensor:
    """Depth image [m], -1 where nothing is hit, shape (world_count, height, width) float32."""
    return self._image(torch.float32)

  def allocate_image_shape_index(self) -> torch.Tensor:
    """Shape-index image, 0xFFFFFFFF where nothing is hit, shape (world_count, height, width)."""
    return self._image(torch.uint32)

  def allocate_image_color_hdr(self) -> torch.Tensor:
    """Linear HDR radiance (before exposure), shape (world_count, height, width, 3) float32."""
    return self._image(torch.float32, (3,))

  def _check_image(self, name: str, image: Any, kind: str) -> int:
    shape = (self.nworld, self.height, self.width)
    if kind == "vec3":
      return device_view(image, name, (*shape, 3), ("<f4",), self.device)
    types = ("<f4",) if kind == "f32" else ("<u4", "<i4")
    return device_view(image, name, shape, types, self.device)

  def update(
    self,
    state: Any,
    camera_transforms: Any,
    *,
    color_image: Any = None,
    depth_image: Any = None,
    forward_depth_image: Any = None,
    shape_index_image: Any = None,
    hdr_color_image: Any = None,
    seed: int = 0,
  ) -> None:
    """Renders view i = world i from camera_transforms[i] ((world_count,) transforms) on the
    current torch stream: pose kernel, refit, render, output kernel.

    Raises:
      ValueError: for camera transforms or output images of the wrong shape, dtype or device.
    """
    nworld = self.nworld
    shape = tuple(camera_transforms.shape) if hasattr(camera_transforms, "shape") else None
    if shape is None or shape[0] != nworld:
      raise ValueError(f"camera_transforms must have one transform per world ({nworld})")
    cams = device_view(camera_transforms, "camera_transforms", (nworld, 7), ("<f4",), self.device)
    ptrs = {
      "color_image": self._check_image("color_image", color_image, "u32") if color_image is not None else None,
      "depth_image": self._check_image("depth_image", depth_image, "f32") if depth_image is not None else None,
      "forward_depth_image": self._check_image("forward_depth_image", forward_depth_image, "f32") if forward_depth_image is not None else None,
      "shape_index_image": self._check_image("shape_index_image", shape_index_image, "u32") if shape_index_image is not None else None,
      "hdr_color_image": self._check_image("hdr_color_image", hdr_color_image, "vec3") if hdr_color_image is not None else None,
    }
    model = self.model
    shape_body = _required(model.shape_body, "shape_body")
    shape_xform = _required(model.shape_transform, "shape_transform")
    nshape = int(shape_body.shape[0])
    sb = device_view(shape_body, "model.shape_body", (nshape,), ("<i4",), self.device)
    sx = device_view(shape_xform, "model.shape_transform", (nshape, 7), ("<f4",), self.device)
    body_q = getattr(state, "body_q", None)
    if body_q is not None and int(body_q.shape[0]) > 0:
      nbody = int(body_q.shape[0])
      bq = device_view(body_q, "state.body_q", (nbody, 7), ("<f4",), self.device)
    else:  # a model without bodies: every shape is static
      nbody, bq = 0, self._no_bodies.data_ptr()
    stream = torch.cuda.current_stream(self.device).cuda_stream
    m, d, rc = self.m, self.d, self.rc
    _lib.call(
      "mjpbr_newton_sync_poses",
      bq, nbody, sb, sx, nshape, self.geom_shape.data_ptr(), self.geom_shape.shape[0], self.geom_offset.data_ptr(), cams,
      nworld, self.mjm.ngeom, self.mjm.ncam, 0, d.geom_xpos.data_ptr(), d.geom_xmat.data_ptr(), d.cam_xpos.data_ptr(), d.cam_xmat.data_ptr(),
      rc.error_word.data_ptr(), stream,
    )
    refit_bvh(m, d, rc)
    render(m, d, rc, seed=seed)
    _lib.call(
      "mjpbr_newton_images",
      scene_descriptor(m, d, rc), 0, self.geom_shape.data_ptr(), self.geom_shape.shape[0], self.ray_scale.data_ptr(),
      ptrs["color_image"], ptrs["depth_image"], ptrs["forward_depth_image"], ptrs["shape_index_image"], ptrs["hdr_color_image"], stream,
    )
