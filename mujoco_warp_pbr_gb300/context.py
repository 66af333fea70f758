"""create_render_context: argument checks, host-side resolution of materials, lights, cameras,
textures and environment maps, acceleration-structure builds, and device allocation.

Mirrors mujoco_warp_pbr/_src/io.py:331-634 (same keyword arguments, defaults and ValueError
messages). Work is split in two: `prepare_context` resolves everything on the host (numpy, plus the
host BVH builders of libmjpbr) and needs no GPU; `create_render_context` uploads the result and
computes the GPU tables (DFG table, mip chains, prefiltered environment stacks) with libmjpbr.
"""

from __future__ import annotations

import ctypes
import dataclasses
import enum
import math
import warnings
from collections.abc import Sequence
from typing import Any

import numpy as np
import torch

from mujoco_warp_pbr_gb300 import _lib
from mujoco_warp_pbr_gb300 import envmap as envmap_lib
from mujoco_warp_pbr_gb300 import model as model_lib
from mujoco_warp_pbr_gb300.pbr_types import LightModel
from mujoco_warp_pbr_gb300.pbr_types import Outputs
from mujoco_warp_pbr_gb300.pbr_types import PbrRenderContext
from mujoco_warp_pbr_gb300.pbr_types import RenderOrder
from mujoco_warp_pbr_gb300.pbr_types import Tier
from mujoco_warp_pbr_gb300.pbr_types import ToneMapper
from mujoco_warp_pbr_gb300.pbr_types import UnsetMaterial

# Filament's default camera: f/16, 1/125 s, ISO 100.
DEFAULT_EV100 = 14.96578428466209
DFG_LUT_SIZE = 128
DFG_LUT_SAMPLES = 1024
# Path tracer random-number layout: path depths (bounces + translucent passes) stay below this.
MAX_PATH_VERTICES = 63

_TRAVERSALS = ("software", "optix", "auto")
_MESH_BVH_FRAMES = ("auto", "mujoco")
_MESH_BVH_CONSTRUCTORS = ("cubql", "sah", "lbvh")
_MATERIAL_KEYS = ("metallic", "roughness")
_DEFAULT_SHININESS = 0.5
_DEFAULT_SPECULAR = 0.5
_DEFAULT_GEOM_RGBA = (0.5, 0.5, 0.5, 1.0)
_LUMINANCE = np.array([0.2126, 0.7152, 0.0722])

GEOM_PLANE, GEOM_HFIELD, GEOM_SPHERE, GEOM_CAPSULE, GEOM_ELLIPSOID, GEOM_CYLINDER, GEOM_BOX, GEOM_MESH, GEOM_SDF = range(9)
LIGHT_SPOT, LIGHT_DIRECTIONAL, LIGHT_POINT, LIGHT_IMAGE = range(4)
ROLE_RGB, ROLE_OCCLUSION, ROLE_ROUGHNESS, ROLE_METALLIC, ROLE_NORMAL, ROLE_OPACITY, ROLE_EMISSIVE, ROLE_RGBA, ROLE_ORM = (
  1,
  2,
  3,
  4,
  5,
  6,
  7,
  8,
  9,
)
_COLOR_ROLES = (ROLE_RGB, ROLE_RGBA, ROLE_EMISSIVE)
TEX_RGBA8, TEX_RGBA16F = 0, 1


def _enum(cls: type[enum.IntEnum], value: int, name: str) -> enum.IntEnum:
  try:
    return cls(value)
  except ValueError:
    options = ", ".join(f"{cls.__name__}.{e.name}" for e in cls)
    raise ValueError(f"{name} must be one of {options}, got {value!r}") from None


SCHEDULES = {"grid": 0, "queue": 1, "wavefront": 2}


def _schedule(schedule: str | int) -> int:
  """The real-time tier's schedule: "grid" (one CTA per camera tile and world), "queue" (a
  persistent launch whose warps pull work items from a device counter) or "wavefront" (primary,
  mirror and shadow rays and the shading as separate kernels over compacted ray queues)."""
  if isinstance(schedule, str) and schedule in SCHEDULES:
    return SCHEDULES[schedule]
  if not isinstance(schedule, str) and int(schedule) in SCHEDULES.values():
    return int(schedule)
  raise ValueError(f'schedule must be "grid", "queue" or "wavefront", got {schedule!r}')


def _check_at_least(name: str, value: int, low: int) -> None:
  if value < low:
    raise ValueError(f"{name} must be at least {low}, got {value}")


def _check_default_material(default_material: dict | None) -> None:
  for key, value in (default_material or {}).items():
    if key not in _MATERIAL_KEYS:
      raise ValueError(f"default_material keys must be among {_MATERIAL_KEYS}, got {key!r}")
    if not 0.0 <= value <= 1.0:
      raise ValueError(f"default_material[{key!r}] must be in [0, 1], got {value}")


# ------------------------------------------------------------------ materials (material.py:102-221)


def effective_geom_rgba(mjm: Any) -> np.ndarray:
  """(ngeom, 4) rgba each geom renders with: material colour where the geom keeps the default."""
  rgba = np.array(mjm.geom_rgba, dtype=np.float64).reshape(-1, 4)
  if not mjm.nmat:
    return rgba
  matid = np.asarray(mjm.geom_matid)
  inherit = (matid >= 0) & np.all(np.isclose(rgba, _DEFAULT_GEOM_RGBA), axis=1)
  rgba[inherit] = np.asarray(mjm.mat_rgba)[matid[inherit]]
  return rgba


def _heuristic(rgba: np.ndarray, shininess: float, has_material: bool) -> tuple[float, float, float]:
  r, g, b = rgba[:3]
  if not has_material:
    brightness = (r + g + b) / 3.0
    if brightness < 0.25:
      return 0.4, 0.45, 0.35
    if brightness > 0.8 or (r > 0.7 and g < 0.3):
      return 0.0, 0.4, 0.25
    return 0.0, 0.5, 0.2
  lum = float(np.dot(rgba[:3], _LUMINANCE))
  chroma = max(r, g, b) - min(r, g, b)
  metallic, roughness, reflectance = 0.0, 0.42, 0.6
  if lum > 0.75 and chroma < 0.10:
    roughness, reflectance = 0.38, 0.65
  elif lum < 0.28 and chroma < 0.12:
    roughness, reflectance = 0.28, 0.6
  elif chroma < 0.08 and 0.35 <= lum <= 0.75:
    metallic, roughness, reflectance = 0.6, 0.40, 0.7
  else:
    roughness = 0.40
  if shininess > 0.0 and shininess != _DEFAULT_SHININESS:
    roughness = float(np.clip(roughness * (1.3 - shininess), 0.06, 1.0))
  return metallic, roughness, reflectance


def resolve_geom_materials(
  mjm: Any, unset_material: int = UnsetMaterial.GLTF, default_material: dict | None = None
) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
  """(metallic, perceptual roughness, reflectance) per geom (material.py:132-182): authored values
  win; unset ones come from default_material, else GLTF (metallic 0, roughness 1 - shininess,
  reflectance = specular) or the colour HEURISTIC (ground planes matte)."""
  default_material = default_material or {}
  ngeom = len(mjm.geom_type)
  metallic = np.zeros(ngeom, np.float32)
  roughness = np.zeros(ngeom, np.float32)
  reflectance = np.zeros(ngeom, np.float32)
  rgba_all = effective_geom_rgba(mjm)
  for g in range(ngeom):
    mat = int(mjm.geom_matid[g])
    has = mat >= 0
    shininess = float(mjm.mat_shininess[mat]) if has else _DEFAULT_SHININESS
    specular = float(mjm.mat_specular[mat]) if has else _DEFAULT_SPECULAR
    am = float(mjm.mat_metallic[mat]) if has else -1.0
    ar = float(mjm.mat_roughness[mat]) if has else -1.0
    if unset_material == UnsetMaterial.HEURISTIC and am < 0.0 and ar < 0.0:
      m, r, f = _heuristic(rgba_all[g], shininess, has)
      if int(mjm.geom_type[g]) == GEOM_PLANE:
        m, r, f = 0.0, 1.0, 0.0
    else:
      m, r, f = 0.0, float(np.clip(1.0 - shininess, 0.0, 1.0)), specular
    if am < 0.0 and "metallic" in default_material:
      m = default_material["metallic"]
    if ar < 0.0 and "roughness" in default_material:
      r = default_material["roughness"]
    metallic[g] = am if am >= 0.0 else m
    roughness[g] = ar if ar >= 0.0 else r
    reflectance[g] = f
  return metallic, roughness, reflectance


@dataclasses.dataclass
class SurfaceFeatures:
  """Texture roles bound to the rendered materials, and specular anti-aliasing."""

  textures: bool
  base_color_map: bool
  normal_map: bool
  orm_map: bool
  emissive_map: bool
  opacity_map: bool
  alpha_map: bool
  specular_aa: bool


def surface_features(mjm: Any, use_textures: bool, specular_aa: bool, mats: np.ndarray) -> SurfaceFeatures:
  texid = np.asarray(mjm.mat_texid)[mats] if mjm.nmat else np.full((0, 10), -1)

  def has(*roles: int) -> bool:
    return use_textures and bool(np.any(texid[:, list(roles)] >= 0))

  f = SurfaceFeatures(
    textures=False,
    base_color_map=has(ROLE_RGB, ROLE_RGBA),
    normal_map=has(ROLE_NORMAL),
    orm_map=has(ROLE_ORM, ROLE_OCCLUSION, ROLE_ROUGHNESS, ROLE_METALLIC),
    emissive_map=has(ROLE_EMISSIVE),
    opacity_map=has(ROLE_OPACITY),
    alpha_map=False,
    specular_aa=specular_aa,
  )
  f.textures = f.base_color_map or f.normal_map or f.orm_map or f.emissive_map or f.opacity_map
  if use_textures:
    for role, channel in ((ROLE_RGBA, 3), (ROLE_OPACITY, 0)):
      for t in np.unique(texid[:, role]) if len(texid) else []:
        if t < 0:
          continue
        w, h, nc = int(mjm.tex_width[t]), int(mjm.tex_height[t]), int(mjm.tex_nchannel[t])
        data = np.asarray(mjm.tex_data)[int(mjm.tex_adr[t]) : int(mjm.tex_adr[t]) + w * h * nc].reshape(-1, nc)
        if channel < nc and np.any(data[:, channel] < 255):
          f.alpha_map = True
  return f


# ------------------------------------------------------------------ lights (io.py:223-248, lights.py:134-148)


def exposure_from_ev100(ev100: float) -> float:
  """Photometric exposure for a camera EV100 (Filament: 1 / (1.2 * 2^EV100))."""
  return 1.0 / (1.2 * math.pow(2.0, ev100))


def fallback_intensity(mjm: Any, light_xpos: np.ndarray, light_id: int, exposure: float) -> float:
  """Physical intensity of a light with intensity 0: a white Lambertian surface facing the light
  shows its diffuse colour (directional: pi / exposure lux; point / spot: that illuminance at the
  distance from the light to the model centre)."""
  illuminance = math.pi / exposure
  if int(mjm.light_type[light_id]) == LIGHT_DIRECTIONAL:
    return illuminance
  distance = float(np.linalg.norm(np.asarray(light_xpos[light_id]) - np.asarray(mjm.stat_center)))
  distance = max(distance, 0.1 * float(mjm.stat_extent), 1e-3)
  return illuminance * distance * distance


def resolve_lighting(mjm: Any, light_xpos: np.ndarray, light_model: int, ev100: float) -> tuple[float, np.ndarray, np.ndarray]:
  """(exposure, per-light physical intensity, constant ambient radiance)."""
  physical = light_model == LightModel.PHYSICAL
  exposure = exposure_from_ev100(ev100) if physical else 1.0
  nlight = len(mjm.light_type)
  intensity = np.array(mjm.light_intensity, dtype=np.float32).reshape(nlight)
  for i in range(nlight):
    if intensity[i] > 0.0:
      intensity[i] /= max(float(np.max(mjm.light_diffuse[i])), 1e-6)
    else:
      intensity[i] = fallback_intensity(mjm, light_xpos, i, exposure)
  ambient = np.zeros(3, np.float32)
  if mjm.headlight_active:
    ambient += np.asarray(mjm.headlight_ambient, np.float32)
  if physical:
    ambient /= exposure
  elif nlight:
    ambient += np.sum(np.asarray(mjm.light_ambient)[np.asarray(mjm.light_active).astype(bool)], axis=0)
  return exposure, intensity, ambient


# ------------------------------------------------------------------ geometry bounds for topology


def geom_aabbs(mjm: Any, xpos: np.ndarray, xmat: np.ndarray, mesh_bounds: np.ndarray | None) -> tuple[np.ndarray, np.ndarray]:
  """World AABBs (ngeom, 3) of every geom for one world (the build-time twin of the refit)."""
  ngeom = len(mjm.geom_type)
  lo = np.zeros((ngeom, 3))
  hi = np.zeros((ngeom, 3))
  for g in range(ngeom):
    t = int(mjm.geom_type[g])
    s = np.asarray(mjm.geom_size[g], np.float64)
    R = np.asarray(xmat[g], np.float64).reshape(3, 3)
    c = np.asarray(xpos[g], np.float64).copy()
    A = np.abs(R)
    if t == GEOM_SPHERE:
      e = np.full(3, s[0])
    elif t == GEOM_CAPSULE:
      e = A[:, 2] * s[1] + s[0]
    elif t == GEOM_ELLIPSOID:
      e = np.sqrt(((R * s[None, :]) ** 2).sum(1))
    elif t == GEOM_CYLINDER:
      e = A[:, 2] * s[1] + s[0] * np.sqrt(np.maximum(0.0, 1.0 - R[:, 2] ** 2))
    elif t == GEOM_BOX:
      e = A @ s
    elif t == GEOM_PLANE:
      sx = s[0] if s[0] > 0 else 1e6
      sy = s[1] if s[1] > 0 else 1e6
      e = A[:, 0] * sx + A[:, 1] * sy
    elif (b := blas_index(t, int(mjm.geom_dataid[g]), mjm)) >= 0 and mesh_bounds is not None:
      mb = mesh_bounds[b]
      lc = 0.5 * (mb[:3] + mb[3:])
      e = A @ (0.5 * (mb[3:] - mb[:3]))
      c = c + R @ lc
    else:
      e = np.zeros(3)
    lo[g] = c - e
    hi[g] = c + e
  return lo, hi


def geom_aabbs_all(mjm: Any, xpos: np.ndarray, xmat: np.ndarray, mesh_bounds: np.ndarray | None) -> tuple[np.ndarray, np.ndarray]:
  """geom_aabbs for every world at once: xpos (nworld, ngeom, 3), xmat (nworld, ngeom, 9) ->
  lo, hi (nworld, ngeom, 3), the same formulas vectorised over worlds and the geoms of a type."""
  xpos = np.asarray(xpos, np.float64)
  R_all = np.asarray(xmat, np.float64).reshape(xpos.shape[0], xpos.shape[1], 3, 3)
  types = np.asarray(mjm.geom_type).reshape(-1)
  size = np.asarray(mjm.geom_size, np.float64).reshape(-1, 3)
  c = xpos.copy()
  e = np.zeros_like(xpos)

  def pick(sel):
    R = R_all[:, sel]  # (nworld, n, 3, 3)
    return R, np.abs(R), size[sel][None]  # s: (1, n, 3)

  sel = types == GEOM_SPHERE
  e[:, sel] = size[sel, 0][None, :, None]
  sel = types == GEOM_CAPSULE
  R, A, sz = pick(sel)
  e[:, sel] = A[..., 2] * sz[..., 1:2] + sz[..., 0:1]
  sel = types == GEOM_ELLIPSOID
  R, A, sz = pick(sel)
  e[:, sel] = np.sqrt(((R * sz[:, :, None, :]) ** 2).sum(-1))
  sel = types == GEOM_CYLINDER
  R, A, sz = pick(sel)
  e[:, sel] = A[..., 2] * sz[..., 1:2] + sz[..., 0:1] * np.sqrt(np.maximum(0.0, 1.0 - R[..., 2] ** 2))
  sel = types == GEOM_BOX
  R, A, sz = pick(sel)
  e[:, sel] = (A * sz[:, :, None, :]).sum(-1)
  sel = types == GEOM_PLANE
  R, A, sz = pick(sel)
  sx = np.where(sz[..., 0:1] > 0, sz[..., 0:1], 1e6)
  sy = np.where(sz[..., 1:2] > 0, sz[..., 1:2], 1e6)
  e[:, sel] = A[..., 0] * sx + A[..., 1] * sy
  if mesh_bounds is not None:
    blas = np.array([blas_index(int(t), int(d), mjm) for t, d in zip(types, np.asarray(mjm.geom_dataid).reshape(-1))], np.int64)
    sel = blas >= 0
    if np.any(sel):
      R, A, _ = pick(sel)
      mb = np.asarray(mesh_bounds, np.float64)[blas[sel]]
      lc = 0.5 * (mb[:, :3] + mb[:, 3:])
      half = 0.5 * (mb[:, 3:] - mb[:, :3])
      e[:, sel] = (A * half[None, :, None, :]).sum(-1)
      c[:, sel] = c[:, sel] + (R * lc[None, :, None, :]).sum(-1)
  return c - e, c + e


def build_scene_topology(lo: np.ndarray, hi: np.ndarray) -> np.ndarray:
  """(nnode, 2) child refs of an SAH tree over the boxes (libmjpbr's host builder)."""
  lib = _lib.load()
  n = len(lo)
  lo32 = np.ascontiguousarray(lo, np.float32)
  hi32 = np.ascontiguousarray(hi, np.float32)
  out = np.zeros((lib.mjpbr_bvh_node_count(n), 2), np.int32)
  status = lib.mjpbr_build_scene_bvh(lo32.ctypes.data, hi32.ctypes.data, n, out.ctypes.data)
  if status != 0:
    raise RuntimeError("scene BVH build failed")
  return out


def scene_tree_levels(topo: np.ndarray) -> int:
  """Inner-node levels of the deepest scene tree: topo (nworld or 1, nnode, 2) child refs (>= 0 an
  inner node, < 0 a leaf or empty), nodes in pre-order (every child after its parent)."""
  topo = np.asarray(topo).reshape(-1, topo.shape[-2], 2)
  depth = np.zeros(topo.shape[:2], np.int32)
  rows = np.arange(topo.shape[0])
  for i in range(topo.shape[1]):
    for k in (0, 1):
      c = topo[:, i, k]
      inner = c >= 0
      depth[rows[inner], c[inner]] = depth[inner, i] + 1
  return int(depth.max()) + 1


def mesh_tree_levels(nodes: np.ndarray) -> int:
  """Inner-node levels of one mesh BVH: nodes (nnode, 16) float32 in the child-bounds layout of
  libmjpbr's mesh builder (child k: ref bits at 8k + 3, count bits at 8k + 7; count 0 an inner node,
  root 0)."""
  bits = np.ascontiguousarray(nodes, np.float32).view(np.int32)
  levels, frontier = 0, np.array([0])
  while frontier.size:
    levels += 1
    kids = []
    for k in (0, 1):
      ref, cnt = bits[frontier, 8 * k + 3], bits[frontier, 8 * k + 7]
      kids.append(ref[cnt == 0])
    frontier = np.concatenate(kids)
  return levels


def traversal_stack_depth(scene_levels: int, mesh_levels: int) -> int:
  """Stack entries a nearest-first traversal can hold: a node popped at stack position p sits at
  depth >= p, so at a scene leaf at most scene_levels entries wait below the mesh traversal, which
  adds at most mesh_levels + 1 (the far children of its path plus both children of its deepest
  inner node). Clamped to the 8..32 entries the kernels support."""
  need = scene_levels + mesh_levels + 1
  if need > 32:
    warnings.warn(
      f"BVHs of {scene_levels} scene and {mesh_levels} mesh levels can need {need} traversal stack entries, more than 32; "
      "a ray that overflows is reported in the error word",
      stacklevel=3,
    )
  return min(max(need, 8), 32)


def nhfield_of(mjm: Any) -> int:
  """Height fields of a model (0 for models without the hfield_* fields)."""
  nrow = getattr(mjm, "hfield_nrow", None)
  return 0 if nrow is None else int(len(np.asarray(nrow).reshape(-1)))


def blas_index(gtype: int, dataid: int, mjm: Any) -> int:
  """Triangle BVH of a geom: its mesh's (index = mesh id), a height field's (index = nmesh +
  height-field id, after every mesh), or -1 (the refit kernel's mapping)."""
  if dataid < 0:
    return -1
  if gtype in (GEOM_MESH, GEOM_SDF) and dataid < mjm.nmesh:
    return dataid
  if gtype == GEOM_HFIELD and dataid < nhfield_of(mjm):
    return mjm.nmesh + dataid
  return -1


def hfield_mesh(mjm: Any, h: int) -> tuple[np.ndarray, np.ndarray]:
  """Height field h as a closed triangle mesh in the geom frame: (vertices (nv, 3) float32, faces
  (nf, 3) int32), every face wound outwards.

  MuJoCo's height-field solid: elevation samples on an nrow x ncol grid spanning
  [-size0, size0] x [-size1, size1] (columns along x, rows along y), z = size2 * elevation, standing
  on a base at z = -size3. Faces, in this order: the top (two triangles per grid cell: (r, c),
  (r, c+1), (r+1, c+1) and (r, c), (r+1, c+1), (r+1, c), cells row by row); the four side walls (two
  triangles per border segment: top p, base q, top q and top p, base p, base q, for consecutive
  border samples p -> q walked counter-clockwise seen from +z, starting at sample (0, 0)); the base
  (a fan from the centre (0, 0, -size3) over the same segments: centre, base q, base p). Coordinates are computed in float64 and rounded
  once to float32: x = size0 (2 c / (ncol - 1) - 1), y = size1 (2 r / (nrow - 1) - 1). Replaces the
  third-party height-field mesh of MuJoCo Warp that the reference traces (traverse.py:161-164)."""
  nr, nc = int(mjm.hfield_nrow[h]), int(mjm.hfield_ncol[h])
  if nr < 2 or nc < 2:
    raise ValueError(f"height field {h}: nrow and ncol must be at least 2, got {nr} x {nc}")
  size = np.asarray(mjm.hfield_size, np.float32).reshape(-1, 4)[h].astype(np.float64)
  adr = int(mjm.hfield_adr[h])
  elev = np.asarray(mjm.hfield_data, np.float32).reshape(-1)[adr : adr + nr * nc].reshape(nr, nc).astype(np.float64)
  xs = size[0] * (2.0 * np.arange(nc) / (nc - 1) - 1.0)
  ys = size[1] * (2.0 * np.arange(nr) / (nr - 1) - 1.0)
  top = np.stack(np.broadcast_arrays(xs[None, :], ys[:, None], size[2] * elev), -1).reshape(-1, 3)
  base = top.copy()
  base[:, 2] = -size[3]
  centre = np.array([[0.0, 0.0, -size[3]]])
  vert = np.concatenate([top, base, centre]).astype(np.float32)
  nb = nr * nc  # first base vertex
  ic = 2 * nb  # the base centre

  def tid(r: np.ndarray, c: np.ndarray) -> np.ndarray:
    return r * nc + c

  r, c = np.meshgrid(np.arange(nr - 1), np.arange(nc - 1), indexing="ij")
  r, c = r.reshape(-1), c.reshape(-1)
  a, b, d, e = tid(r, c), tid(r, c + 1), tid(r + 1, c + 1), tid(r + 1, c)
  top_faces = np.stack([np.stack([a, b, d], -1), np.stack([a, d, e], -1)], 1).reshape(-1, 3)
  # border samples counter-clockwise seen from +z: along row 0, up column nc-1, back along row
  # nr-1, down column 0
  ring_r = np.concatenate([np.zeros(nc - 1, int), np.arange(nr - 1), np.full(nc - 1, nr - 1), np.arange(nr - 1, 0, -1)])
  ring_c = np.concatenate([np.arange(nc - 1), np.full(nr - 1, nc - 1), np.arange(nc - 1, 0, -1), np.zeros(nr - 1, int)])
  p = tid(ring_r, ring_c)
  q = np.roll(p, -1)
  side = np.stack([np.stack([p, q + nb, q], -1), np.stack([p, p + nb, q + nb], -1)], 1).reshape(-1, 3)
  bottom = np.stack([np.full_like(p, ic), q + nb, p + nb], -1)
  face = np.concatenate([top_faces, side, bottom]).astype(np.int32)
  return vert, face


def mesh_sources(mjm: Any) -> list[tuple[str, np.ndarray, np.ndarray]]:
  """(name, vertices, faces) of every triangle BVH: one per mesh, then one per height field."""
  vert_all = np.asarray(mjm.mesh_vert, np.float32).reshape(-1, 3)
  face_all = np.asarray(mjm.mesh_face, np.int32).reshape(-1, 3)
  sources = []
  for m in range(mjm.nmesh):
    v0, nv = int(mjm.mesh_vertadr[m]), int(mjm.mesh_vertnum[m])
    f0, nf = int(mjm.mesh_faceadr[m]), int(mjm.mesh_facenum[m])
    sources.append((f"mesh {m}", vert_all[v0 : v0 + nv], face_all[f0 : f0 + nf]))
  for h in range(nhfield_of(mjm)):
    sources.append((f"height field {h}", *hfield_mesh(mjm, h)))
  return sources


def build_mesh_bvhs(mjm: Any, sources: list[tuple[str, np.ndarray, np.ndarray]] | None = None) -> dict[str, Any]:
  """Triangle BVHs concatenated, one per mesh, then one per height field (hfield_mesh), built on
  the host with binned SAH: nodes (nnode, 16), tris (ntri, 12), root / tri_base per BVH, local
  AABBs (nmesh + nhfield, 6)."""
  lib = _lib.load()
  nodes, tris, roots, bases, bounds, nfaces, levels = [], [], [], [], [], [], []
  node_total = tri_total = 0
  sources = mesh_sources(mjm) if sources is None else sources
  for name, vert, face in sources:
    vert = np.ascontiguousarray(vert, np.float32)
    face = np.ascontiguousarray(face, np.int32)
    nv, nf = len(vert), len(face)
    cap = lib.mjpbr_bvh_node_count(nf)
    node_buf = np.zeros((cap, 16), np.float32)
    tri_buf = np.zeros((nf, 12), np.float32)
    bnd = np.zeros(6, np.float32)
    nnode = ctypes.c_int32(0)
    status = lib.mjpbr_build_mesh_bvh(
      vert.ctypes.data, nv, face.ctypes.data, nf, 4, node_buf.ctypes.data, tri_buf.ctypes.data, bnd.ctypes.data, ctypes.byref(nnode)
    )
    if status != 0:
      raise ValueError(f"{name}: BVH build failed (status {status})")
    nodes.append(node_buf[: nnode.value])
    levels.append(mesh_tree_levels(node_buf[: nnode.value]))
    tris.append(tri_buf)
    roots.append(node_total)
    bases.append(tri_total)
    bounds.append(bnd)
    nfaces.append(nf)
    node_total += nnode.value
    tri_total += nf
  return {
    "blas_nodes": np.concatenate(nodes) if nodes else None,
    "blas_tris": np.concatenate(tris) if tris else None,
    "blas_root": np.array(roots, np.int32) if roots else None,
    "blas_tri_base": np.array(bases, np.int32) if bases else None,
    "mesh_bounds": np.stack(bounds).astype(np.float32) if bounds else None,
    "mesh_nface": nfaces[: mjm.nmesh] if mjm is not None else nfaces,
    "nhfield": nhfield_of(mjm) if mjm is not None else 0,
    "mesh_levels": max(levels) if levels else 0,
  }


def device_mesh_sources(mjm: Any) -> dict[str, Any]:
  """The triangle BVH sources concatenated for the device builder (mjpbr_build_mesh_bvh_device):
  vertices, faces with source-local vertex indices, per-source vertex base / count, face base
  (nsrc + 1) and node base (node capacities mjpbr_bvh_node_count(nface) in order), plus what
  the host needs before the build: the sources' AABBs (of the vertices their faces use) and
  face counts.

  Raises:
    ValueError: for a source without faces or a face naming a vertex out of range.
  """
  sources = mesh_sources(mjm)
  nface = np.array([len(f) for _, _, f in sources], np.int64)
  nvert = np.array([len(v) for _, v, _ in sources], np.int64)
  bounds = np.zeros((len(sources), 6), np.float32)
  for i, (name, vert, face) in enumerate(sources):
    if len(face) == 0 or np.any(face < 0) or np.any(face >= len(vert)):
      raise ValueError(f"{name}: BVH build failed (a face names a vertex out of range, or there are no faces)")
    used = vert[face.reshape(-1)]
    bounds[i, :3], bounds[i, 3:] = used.min(axis=0), used.max(axis=0)
  cap = np.maximum(nface - 1, 1)
  return {
    "device_sources": {
      "vert": np.ascontiguousarray(np.concatenate([v for _, v, _ in sources]), np.float32),
      "face": np.ascontiguousarray(np.concatenate([f for _, _, f in sources]), np.int32),
      "vert_base": np.concatenate([[0], np.cumsum(nvert)[:-1]]).astype(np.int32),
      "vert_num": nvert.astype(np.int32),
      "face_base": np.concatenate([[0], np.cumsum(nface)]).astype(np.int32),
      "node_base": np.concatenate([[0], np.cumsum(cap)[:-1]]).astype(np.int32),
      "nodes": int(cap.sum()),
      "names": [n for n, _, _ in sources],
    },
    "mesh_bounds": bounds,
    "mesh_nface": [int(n) for n in nface[: mjm.nmesh]],
    "nhfield": nhfield_of(mjm),
    "mesh_levels": None,
  }


MESH_BVH_LEAF = 4  # triangles per leaf of the mesh BVHs
# With the default constructor ("cubql", the reference's GPU builder), models with at least this many
# mesh and height-field triangles build their BVHs on the GPU (linear BVHs, tens of ms for millions of
# triangles); smaller ones use the host's binned SAH, whose trees render about 5 % faster and build in
# well under 100 ms at this size. "sah" always builds on the host, "lbvh" always on the GPU.
DEVICE_BVH_FACES = 1 << 17


def total_bvh_faces(mjm: Any) -> int:
  """Triangles of every mesh and height-field BVH (hfield_mesh of r x c samples: 2 (r - 1)(c - 1)
  top triangles, and per border segment two side triangles and one of the base)."""
  n = int(np.sum(np.asarray(mjm.mesh_facenum))) if mjm.nmesh else 0
  for h in range(nhfield_of(mjm)):
    r, c = int(mjm.hfield_nrow[h]), int(mjm.hfield_ncol[h])
    n += 2 * (r - 1) * (c - 1) + 3 * (2 * (r - 1) + 2 * (c - 1))
  return n


def _source_arrays(src: dict[str, Any], i: int) -> tuple[np.ndarray, np.ndarray]:
  v0, nv = int(src["vert_base"][i]), int(src["vert_num"][i])
  f0, f1 = int(src["face_base"][i]), int(src["face_base"][i + 1])
  return src["vert"][v0 : v0 + nv], src["face"][f0:f1]


def build_mesh_bvhs_device(src: dict[str, Any], device: torch.device) -> dict[str, Any]:
  """Runs the device BVH builder over device_mesh_sources' arrays: blas_nodes / blas_tris /
  blas_root / blas_tri_base / mesh_bounds as device tensors and mesh_levels (the deepest tree's
  inner levels, read back for the traversal stack size)."""
  i32 = torch.int32

  def dev(a: np.ndarray, dtype: torch.dtype) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a)).to(device=device, dtype=dtype)

  lib = _lib.load()
  nsrc = len(src["vert_num"])
  nface = int(src["face_base"][-1])
  vert, face = dev(src["vert"], torch.float32), dev(src["face"], i32)
  vert_base, vert_num = dev(src["vert_base"], i32), dev(src["vert_num"], i32)
  face_base, node_base = dev(src["face_base"], i32), dev(src["node_base"], i32)
  nodes = torch.zeros((src["nodes"], 16), dtype=torch.float32, device=device)
  tris = torch.zeros((nface, 12), dtype=torch.float32, device=device)
  bounds = torch.zeros((nsrc, 6), dtype=torch.float32, device=device)
  nnode = torch.zeros(nsrc, dtype=i32, device=device)
  err = torch.zeros(1, dtype=i32, device=device)
  nbytes = int(lib.mjpbr_mesh_bvh_device_scratch_bytes(nsrc, nface))
  scratch = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=device)
  stream = torch.cuda.current_stream(device).cuda_stream
  _lib.call(
    "mjpbr_build_mesh_bvh_device",
    vert.data_ptr(), face.data_ptr(), vert_base.data_ptr(), vert_num.data_ptr(), face_base.data_ptr(), node_base.data_ptr(),
    nsrc, nface, MESH_BVH_LEAF, nodes.data_ptr(), tris.data_ptr(), bounds.data_ptr(), nnode.data_ptr(), scratch.data_ptr(), nbytes,
    err.data_ptr(), stream,
  )
  host_nodes = nodes.cpu().numpy()
  counts = nnode.cpu().numpy()
  if int(err.item()) != 0:
    raise ValueError("device BVH build: a face names a vertex out of range")
  base = src["node_base"]
  levels = max(mesh_tree_levels(host_nodes[base[i] : base[i] + counts[i]]) for i in range(nsrc))
  return {
    "blas_nodes": nodes,
    "blas_tris": tris,
    "blas_root": node_base,
    "blas_tri_base": face_base[:nsrc].contiguous(),
    "mesh_bounds": bounds,
    "mesh_levels": int(levels),
    "node_count": counts,
  }


# ------------------------------------------------------------------ textures (texture.py:63-101)


def srgb_to_linear(x: Any) -> np.ndarray:
  x = np.asarray(x, dtype=np.float64)
  return np.where(x <= 0.04045, x / 12.92, ((x + 0.055) / 1.055) ** 2.4)


_SRGB_TABLE = srgb_to_linear(np.arange(256) / 255.0).astype(np.float16)


def mip_count(w: int, h: int) -> int:
  """Levels of a full mip chain, at most the descriptor's MAX_MIPS (textures above 16384 texels per
  side stop at their 15th level; level-of-detail selection clamps to the last level)."""
  return min(int(math.floor(math.log2(max(w, h)))) + 1, _lib.MAX_MIPS)


@dataclasses.dataclass
class TextureSet:
  """Textures packed in one byte buffer: descriptions (host ctypes), bytes with level 0 filled."""

  desc: list[_lib.Texture]
  data: np.ndarray

  def desc_bytes(self) -> np.ndarray:
    if not self.desc:
      return np.zeros(0, np.uint8)
    return np.frombuffer(b"".join(bytes(d) for d in self.desc), dtype=np.uint8).copy()


def pack_textures(images: list[tuple[int, np.ndarray]]) -> TextureSet:
  """images: (format, (h, w, 4) level-0 array uint8 or float16). Level offsets are 16-byte aligned."""
  desc, chunks, offset = [], [], 0
  for fmt, img in images:
    h, w = img.shape[:2]
    texel = 4 if fmt == TEX_RGBA8 else 8
    d = _lib.Texture()
    d.format, d.width, d.height, d.nlevel = fmt, w, h, mip_count(w, h)
    for level in range(d.nlevel):
      lw, lh = max(w >> level, 1), max(h >> level, 1)
      d.level_offset[level] = offset
      size = lw * lh * texel
      size = (size + 15) // 16 * 16
      if level == 0:
        chunks.append((offset, np.ascontiguousarray(img).view(np.uint8).reshape(-1)))
      offset += size
    desc.append(d)
  data = np.zeros(max(offset, 16), np.uint8)
  for start, raw in chunks:
    data[start : start + raw.size] = raw
  return TextureSet(desc, data)


def texture_images(mjm: Any, used: np.ndarray) -> list[tuple[int, np.ndarray]]:
  """Level-0 images of every texture: sRGB colour roles -> linear float16, data roles -> RGBA8;
  unused or non-2D textures -> 1x1 white placeholder."""
  out = []
  mat_texid = np.asarray(mjm.mat_texid).reshape(-1, 10) if mjm.nmat else np.zeros((0, 10), np.int32)
  for t in range(mjm.ntex):
    if not used[t] or int(mjm.tex_type[t]) != 0:
      out.append((TEX_RGBA8, np.full((1, 1, 4), 255, np.uint8)))
      continue
    w, h, nc = int(mjm.tex_width[t]), int(mjm.tex_height[t]), int(mjm.tex_nchannel[t])
    raw = np.asarray(mjm.tex_data)[int(mjm.tex_adr[t]) : int(mjm.tex_adr[t]) + w * h * nc].reshape(h, w, nc)
    rgba = np.full((h, w, 4), 255, np.uint8)
    if nc == 1:
      rgba[..., :3] = raw
    else:
      rgba[..., :nc] = raw
    cs = int(mjm.tex_colorspace[t])
    srgb = cs == 2 or (cs == 0 and bool(np.isin(t, mat_texid[:, list(_COLOR_ROLES)])))
    if srgb:
      texels = np.concatenate([_SRGB_TABLE[rgba[..., :3]], (rgba[..., 3:] / 255.0).astype(np.float16)], axis=-1)
      out.append((TEX_RGBA16F, np.ascontiguousarray(texels)))
    else:
      out.append((TEX_RGBA8, rgba))
  return out


# ------------------------------------------------------------------ the host context


@dataclasses.dataclass
class HostContext:
  """Everything create_render_context resolves on the host (numpy), before any GPU work."""

  nworld: int
  options: dict[str, Any]
  outputs: dict[str, Any]
  settings: dict[str, Any]
  tables: dict[str, np.ndarray]  # per-world tables with leading dimension 1
  enabled_geom_ids: np.ndarray
  tlas_child: np.ndarray  # (1 or nworld, nnode, 2)
  world_block_floats: int
  meshes: dict[str, Any]
  textures: TextureSet | None
  environments: envmap_lib.HostEnvironments | None
  features: SurfaceFeatures


def _camera_selection(mjm: Any, cam_active: Any) -> list[int]:
  ncam = mjm.ncam
  if cam_active is None:
    return list(range(ncam))
  ids = []
  for i, v in enumerate(cam_active):
    if isinstance(v, bool) or isinstance(v, np.bool_):
      if v:
        ids.append(i)
    elif isinstance(v, (int, np.integer)):
      ids.append(int(v))
    else:
      raise ValueError(f"cam_active entries must be booleans or camera indices, got {v!r}")
  for c in ids:
    if not 0 <= c < ncam:
      raise ValueError(f"camera index {c} out of range [0, {ncam})")
  return ids


def _per_camera(value: Any, n: int, default: bool) -> list[bool]:
  if value is None:
    return [default] * n
  if isinstance(value, (bool, np.bool_)):
    return [bool(value)] * n
  value = list(value)
  if len(value) != n:
    raise ValueError(f"expected one flag per rendering camera ({n}), got {len(value)}")
  return [bool(v) for v in value]


def prepare_context(
  mjm: Any,
  nworld: int = 1,
  cam_res: list[tuple[int, int]] | tuple[int, int] | None = None,
  render_rgb: list[bool] | bool | None = None,
  render_depth: list[bool] | bool | None = None,
  render_seg: list[bool] | bool | None = None,
  enabled_geom_groups: Sequence[int] = (0, 1, 2),
  cam_active: list[bool] | list[int] | None = None,
  background_color: tuple[float, float, float, float] = (0.0, 0.0, 0.0, 1.0),
  use_fast_math: bool = True,
  use_shadows: bool = True,
  shadow_light_fraction: float = 0.0,
  enable_backface_culling: bool = True,
  enable_vertex_normals: bool = True,
  light_model: LightModel | int = LightModel.PHYSICAL,
  tone_mapper: ToneMapper | int = ToneMapper.PBR_NEUTRAL,
  ev100: float = DEFAULT_EV100,
  unset_material: UnsetMaterial | int = UnsetMaterial.GLTF,
  default_material: dict[str, float] | None = None,
  use_textures: bool = True,
  samples_per_pixel: int = 1,
  specular_aa: bool = True,
  shadow_samples: int = 1,
  max_layers: int = 4,
  enable_reflections: bool = True,
  envmap: Any = None,
  envmap_intensity: float | None = None,
  envmap_rotation: float = 0.0,
  envmap_background: bool = True,
  use_skybox: bool = True,
  render_order: RenderOrder | int = RenderOrder.TILED,
  block_dim: int | None = None,
  schedule: str | int = "wavefront",
  queue_item: int = 64,
  wave_chunk_worlds: int = 0,
  max_registers: int | None = None,
  mesh_bvh_constructor: str = "cubql",
  mesh_bvh_frame: str = "auto",
  ordered_traversal: bool | None = None,
  tier: Tier | int = Tier.REALTIME,
  path_samples: int = 64,
  max_depth: int = 4,
  rr_depth: int = 3,
  denoise: bool = False,
  denoise_iterations: int = 3,
  render_hdr: bool = False,
  traversal: str = "software",
  render_guides: bool = False,
  camera_rays: Any = None,
  data: Any = None,
) -> HostContext:
  """Host half of create_render_context (see there); needs no GPU."""
  mjm = model_lib.as_host_model(mjm)
  light_model = _enum(LightModel, light_model, "light_model")
  tone_mapper = _enum(ToneMapper, tone_mapper, "tone_mapper")
  unset_material = _enum(UnsetMaterial, unset_material, "unset_material")
  render_order = _enum(RenderOrder, render_order, "render_order")
  tier = _enum(Tier, tier, "tier")
  for name, value in (
    ("samples_per_pixel", samples_per_pixel),
    ("shadow_samples", shadow_samples),
    ("max_layers", max_layers),
    ("path_samples", path_samples),
  ):
    _check_at_least(name, value, 1)
  for name, value in (("max_depth", max_depth), ("rr_depth", rr_depth), ("denoise_iterations", denoise_iterations)):
    _check_at_least(name, value, 0)
  if tier == Tier.PATH and max_depth + 4 * max_layers >= MAX_PATH_VERTICES:
    raise ValueError(
      f"max_depth + 4 * max_layers must be below {MAX_PATH_VERTICES} for the path tracer's random "
      f"number layout, got {max_depth} + 4 * {max_layers}"
    )
  if not 0.0 <= shadow_light_fraction <= 1.0:
    raise ValueError(f"shadow_light_fraction must be in [0, 1], got {shadow_light_fraction}")
  _check_default_material(default_material)
  if denoise and tier != Tier.PATH:
    raise ValueError("denoise applies to the path-traced tier (Tier.PATH)")
  schedule = _schedule(schedule)
  if queue_item not in (32, 64, 128):
    raise ValueError(f"queue_item must be 32, 64 or 128 pixels, got {queue_item}")
  _check_at_least("wave_chunk_worlds", wave_chunk_worlds, 0)
  if mesh_bvh_frame not in _MESH_BVH_FRAMES:
    raise ValueError(f'mesh_bvh_frame must be "auto" or "mujoco", got {mesh_bvh_frame!r}')
  if mesh_bvh_constructor not in _MESH_BVH_CONSTRUCTORS:
    raise ValueError(f"mesh_bvh_constructor must be one of {_MESH_BVH_CONSTRUCTORS}, got {mesh_bvh_constructor!r}")
  if traversal not in _TRAVERSALS:
    raise ValueError(f'traversal must be "software", "optix" or "auto", got {traversal!r}')
  if block_dim is not None:
    _check_at_least("block_dim", block_dim, 1)
  if max_registers is not None:
    _check_at_least("max_registers", max_registers, 0)
  _check_at_least("nworld", nworld, 1)
  env_images = envmap_lib.envmap_images(envmap)

  light_type = np.asarray(mjm.light_type).reshape(-1)
  image_lights = np.nonzero(light_type == LIGHT_IMAGE)[0]
  if image_lights.size:
    warnings.warn(f"image lights are not supported and are ignored: {image_lights.tolist()}", stacklevel=3)
  groups = np.asarray(mjm.geom_group)
  rendered = np.isin(groups, list(enabled_geom_groups))
  if not np.any(rendered):
    raise ValueError("the model has no geoms in the enabled geom groups to render")
  if traversal != "software":
    warnings.warn(f'traversal="{traversal}" falls back to "software": the GB300 build traces on its own kernels', stacklevel=3)

  # ---- cameras and output layout
  cams = _camera_selection(mjm, cam_active)
  nrender = len(cams)
  if nrender == 0:
    raise ValueError("no active camera to render")
  if nrender > _lib.MAX_RENDER:
    raise ValueError(f"at most {_lib.MAX_RENDER} rendering cameras are supported, got {nrender}")
  if cam_res is None:
    res = [tuple(int(v) for v in np.asarray(mjm.cam_resolution)[c]) for c in cams]
  elif isinstance(cam_res, tuple) and len(cam_res) == 2 and all(isinstance(v, (int, np.integer)) for v in cam_res):
    res = [(int(cam_res[0]), int(cam_res[1]))] * nrender
  else:
    res = [(int(w), int(h)) for w, h in cam_res]
    if len(res) != nrender:
      raise ValueError(f"cam_res must have one (width, height) per rendering camera ({nrender}), got {len(res)}")
  for w, h in res:
    if w < 1 or h < 1:
      raise ValueError(f"camera resolutions must be positive, got {(w, h)}")
  rgb = _per_camera(render_rgb, nrender, True)
  depth = _per_camera(render_depth, nrender, True)
  seg = _per_camera(render_seg, nrender, False)
  npix = [w * h for w, h in res]
  ray_adr = list(np.concatenate([[0], np.cumsum(npix)[:-1]]).astype(int))

  def adr(flags: list[bool]) -> tuple[list[int], int]:
    out, total = [], 0
    for f, n in zip(flags, npix, strict=True):
      out.append(total if f else -1)
      total += n if f else 0
    return out, total

  rgb_adr, rgb_stride = adr(rgb)
  depth_adr, depth_stride = adr(depth)
  seg_adr, seg_stride = adr(seg)
  total_rays = int(sum(npix))
  if total_rays * nworld >= 2**31:
    raise ValueError(f"nworld * total_rays must stay below 2^31, got {nworld} * {total_rays}")

  # ---- data at creation (initial poses)
  host_data = data
  ngeom = len(mjm.geom_type)

  def world_arrays(w: int) -> tuple[np.ndarray, np.ndarray]:
    xpos = np.asarray(host_data.geom_xpos, np.float64)
    xmat = np.asarray(host_data.geom_xmat, np.float64)
    if xpos.ndim == 3:
      return xpos[w], xmat[w].reshape(ngeom, 9)
    return xpos, xmat.reshape(ngeom, 9)

  # ---- meshes, scene BVH topology
  if not (mjm.nmesh or nhfield_of(mjm)):
    meshes = {"mesh_nface": [], "mesh_bounds": None, "nhfield": 0}
  elif mesh_bvh_constructor == "lbvh" or (mesh_bvh_constructor == "cubql" and total_bvh_faces(mjm) >= DEVICE_BVH_FACES):
    meshes = device_mesh_sources(mjm)  # built on the GPU by upload_context
  else:
    meshes = build_mesh_bvhs(mjm)
  enabled = np.nonzero(rendered)[0].astype(np.int32)
  geom_types = np.asarray(mjm.geom_type).reshape(-1)
  supported = np.isin(geom_types[enabled], [GEOM_PLANE, GEOM_SPHERE, GEOM_CAPSULE, GEOM_ELLIPSOID, GEOM_CYLINDER, GEOM_BOX, GEOM_MESH, GEOM_SDF, GEOM_HFIELD])
  if not np.all(supported):
    bad = sorted(set(geom_types[enabled][~supported].tolist()))
    warnings.warn(f"geom types {bad} are not rendered by the GB300 build", stacklevel=3)
  per_world = host_data is not None and np.asarray(host_data.geom_xpos).ndim == 3
  if host_data is None:
    lo = np.zeros((ngeom, 3))
    hi = np.zeros((ngeom, 3))
    for g in range(ngeom):  # without poses: boxes at the origin, topology from sizes only
      lo[g], hi[g] = -1.0, 1.0
    topo = build_scene_topology(lo[enabled], hi[enabled])[None]
  elif not per_world:
    xpos, xmat = world_arrays(0)
    lo, hi = geom_aabbs(mjm, xpos, xmat, meshes.get("mesh_bounds"))
    topo = build_scene_topology(lo[enabled], hi[enabled])[None]
  else:
    xpos_all = np.asarray(host_data.geom_xpos, np.float64)
    xmat_all = np.asarray(host_data.geom_xmat, np.float64).reshape(xpos_all.shape[0], ngeom, 9)
    lo_all, hi_all = geom_aabbs_all(mjm, xpos_all[:nworld], xmat_all[:nworld], meshes.get("mesh_bounds"))
    topo = np.stack([build_scene_topology(lo_all[w][enabled], hi_all[w][enabled]) for w in range(nworld)])
  meshes["scene_levels"] = scene_tree_levels(topo)
  nbvh = len(enabled)
  nnode = topo.shape[1]
  lib = _lib.load()
  nlight = len(light_type)
  block_floats = int(lib.mjpbr_world_block_floats(nbvh, nnode, nlight, nrender))

  # ---- materials, lights, exposure
  physical = light_model == LightModel.PHYSICAL
  light_xpos0 = np.zeros((nlight, 3))
  if host_data is not None and nlight:
    lx = np.asarray(host_data.light_xpos)
    light_xpos0 = lx[0] if lx.ndim == 3 else lx
  exposure, intensity, ambient = resolve_lighting(mjm, light_xpos0, light_model, ev100)
  metallic, roughness, reflectance = resolve_geom_materials(mjm, unset_material, default_material)
  matid = np.asarray(mjm.geom_matid).reshape(-1)
  rendered_mats = np.unique(matid[rendered & (matid >= 0)])
  features = surface_features(mjm, use_textures, specular_aa and tier == Tier.REALTIME, rendered_mats)
  used_tex = np.zeros(mjm.ntex, bool)
  if features.textures:
    ids = np.asarray(mjm.mat_texid)[rendered_mats].ravel()
    used_tex[ids[ids >= 0]] = True
  textures = pack_textures(texture_images(mjm, used_tex)) if mjm.ntex else None
  alpha = effective_geom_rgba(mjm)[rendered, 3]
  has_transparency = bool(np.any((alpha > 0.0) & (alpha < 1.0))) or features.alpha_map
  mat_reflectance = np.asarray(mjm.mat_reflectance, np.float32).reshape(-1)
  has_reflection = enable_reflections and bool(len(rendered_mats) and np.any(mat_reflectance[rendered_mats] > 0.0))
  background_linear = srgb_to_linear(background_color[:3]).astype(np.float32)

  environments = envmap_lib.prepare_environments(env_images) if env_images else None
  has_env = environments is not None
  if envmap_intensity is None:
    envmap_intensity = 1.0 / exposure
  if has_env and physical:
    ambient[:] = 0.0
  env_texel_angle = 2.0 * math.pi / (environments.max_width if has_env else 1.0)

  settings = {
    "tier": int(tier),
    "render_order": int(render_order),
    "samples_per_axis": int(samples_per_pixel),
    "tone_mapper": int(tone_mapper),
    "render_hdr": int(bool(render_hdr)),
    "render_guides": int(bool(render_guides)),
    "light_model": int(light_model),
    "use_shadows": int(bool(use_shadows)),
    "shadow_samples": int(shadow_samples),
    "headlight_active": int(bool(mjm.headlight_active)),
    "has_env": int(has_env),
    "env_background": int(has_env and envmap_background),
    "textures": int(features.textures),
    "base_color_map": int(features.base_color_map),
    "normal_map": int(features.normal_map),
    "orm_map": int(features.orm_map),
    "emissive_map": int(features.emissive_map),
    "opacity_map": int(features.opacity_map),
    "specular_aa": int(features.specular_aa),
    "vertex_normals": int(bool(enable_vertex_normals)),
    "has_reflection": int(has_reflection),
    "has_transparency": int(has_transparency),
    "max_layers": int(max_layers),
    "cull_backfaces": int(bool(enable_backface_culling)),
    "path_samples": int(path_samples),
    "max_depth": int(max_depth),
    "rr_depth": int(rr_depth),
    "denoise": int(bool(denoise)),
    "stack_depth": traversal_stack_depth(scene_tree_levels(topo), int(meshes.get("mesh_levels") or 0)),
    "znear": float(getattr(mjm, "znear", 0.01)),
    "zfar": float(getattr(mjm, "zfar", 0.0)),
    "shadow_light_fraction": float(shadow_light_fraction),
    "headlight_intensity": float(math.pi),  # the MuJoCo light model ignores intensities
    "headlight_diffuse": tuple(float(c) for c in mjm.headlight_diffuse),
    "headlight_specular": tuple(float(c) for c in mjm.headlight_specular),
    "background": tuple(float(c) for c in background_linear),
    "inv_texel_angle": 1.0 / env_texel_angle,
    "denoise_sigma_color": 4.0,
    "denoise_sigma_normal": 128.0,
    "denoise_sigma_depth": 0.02,
    "denoise_sigma_albedo": 0.05,
  }
  tables = {
    "geom_metallic": metallic.reshape(1, -1),
    "geom_roughness": roughness.reshape(1, -1),
    "geom_reflectance": reflectance.reshape(1, -1),
    "mat_reflectance": (mat_reflectance if len(mat_reflectance) else np.zeros(1, np.float32)).reshape(1, -1),
    "light_intensity": (intensity if nlight else np.zeros(1, np.float32)).reshape(1, -1),
    "light_range": np.asarray(mjm.light_range if nlight else np.zeros(1), np.float32).reshape(1, -1),
    "light_bulbradius": np.asarray(mjm.light_bulbradius if nlight else np.zeros(1), np.float32).reshape(1, -1),
    "exposure": np.array([exposure], np.float32),
    "ambient_radiance": ambient.reshape(1, 3).astype(np.float32),
    "env_id": np.zeros(1, np.int32),
    "env_intensity": np.array([envmap_intensity], np.float32),
    "env_yaw": np.array([np.radians(envmap_rotation)], np.float32),
  }
  outputs = {
    "nrender": nrender,
    "cam_id_map": cams,
    "cam_res": res,
    "render_rgb": rgb,
    "render_depth": depth,
    "render_seg": seg,
    "ray_adr": ray_adr,
    "rgb_adr": rgb_adr,
    "depth_adr": depth_adr,
    "seg_adr": seg_adr,
    "rgb_stride": rgb_stride,
    "depth_stride": depth_stride,
    "seg_stride": seg_stride,
    "total_rays": total_rays,
  }
  options = {
    "light_model": int(light_model),
    "tone_mapper": int(tone_mapper),
    "use_shadows": bool(use_shadows),
    "shadow_light_fraction": float(shadow_light_fraction),
    "samples_per_pixel": int(samples_per_pixel),
    "shadow_samples": int(shadow_samples),
    "has_transparency": has_transparency,
    "max_layers": int(max_layers),
    "has_reflection": has_reflection,
    "render_order": int(render_order),
    "schedule": int(schedule),
    "queue_item": int(queue_item),
    "wave_chunk_worlds": int(wave_chunk_worlds),
    "tier": int(tier),
    "path_samples": int(path_samples),
    "max_depth": int(max_depth),
    "rr_depth": int(rr_depth),
    "denoise": bool(denoise),
    "denoise_iterations": int(denoise_iterations),
    "render_hdr": bool(render_hdr),
    "render_guides": bool(render_guides),
    "has_env": has_env,
    "env_background": bool(has_env and envmap_background),
    "env_texel_angle": env_texel_angle,
    "background_linear": tuple(float(c) for c in background_linear),
    "block_dim": block_dim,
    "max_registers": max_registers,
    "ordered_traversal": ordered_traversal,
    "traversal": "software",
    "camera_rays": camera_rays,
    "cull_backfaces": bool(enable_backface_culling),
    "vertex_normals": bool(enable_vertex_normals),
    "specular_aa": features.specular_aa,
  }
  return HostContext(
    nworld=nworld,
    options=options,
    outputs=outputs,
    settings=settings,
    tables=tables,
    enabled_geom_ids=enabled,
    tlas_child=np.ascontiguousarray(topo, np.int32),
    world_block_floats=block_floats,
    meshes=meshes,
    textures=textures,
    environments=environments,
    features=features,
  )


# ------------------------------------------------------------------ device context

_DFG_CACHE: dict[Any, torch.Tensor] = {}


def dfg_lut(device: torch.device, size: int = DFG_LUT_SIZE, nsample: int = DFG_LUT_SAMPLES) -> torch.Tensor:
  """The split-sum DFG table (size, size, 2) on the device, computed once per device."""
  key = (str(device), size, nsample)
  if key not in _DFG_CACHE:
    lut = torch.empty((size, size, 2), dtype=torch.float32, device=device)
    stream = torch.cuda.current_stream(device).cuda_stream
    _lib.call("mjpbr_dfg_lut", lut.data_ptr(), size, nsample, stream)
    _DFG_CACHE[key] = lut
  return _DFG_CACHE[key]


def upload_textures(ts: TextureSet, device: torch.device) -> tuple[torch.Tensor, torch.Tensor]:
  """Texture descriptions and bytes on the device, with the mip chains built there."""
  data = torch.from_numpy(ts.data).to(device)
  stream = torch.cuda.current_stream(device).cuda_stream
  for d in ts.desc:
    if d.nlevel > 1:
      _lib.call("mjpbr_build_mips", ctypes.byref(d), data.data_ptr(), stream)
  desc = torch.from_numpy(ts.desc_bytes()).to(device)
  return desc, data


def _dev(a: np.ndarray | None, device: torch.device) -> torch.Tensor | None:
  return None if a is None else torch.from_numpy(np.ascontiguousarray(a)).to(device)


def create_render_context(mjm: Any, nworld: int = 1, **kwargs: Any) -> PbrRenderContext:
  """Creates a PBR render context on the current CUDA device.

  Keyword arguments, defaults and errors are those of mujoco_warp_pbr.create_render_context
  (mujoco_warp_pbr/_src/io.py:331-504), plus `data`: the host data (HostData) the scene BVH
  topology is built from (default: every geom at the origin, refit each frame); `schedule`, the
  real-time tier's launch: "grid", "queue" (with `queue_item` pixels per work item) or
  "wavefront" (staged kernels over ray queues; `wave_chunk_worlds` worlds per chunk of its
  scratch, 0: about 64 M camera samples / 32 M paths per chunk); all render the same images.
  mesh_bvh_constructor places the mesh BVH build: "lbvh" on the GPU (linear BVHs), "sah" on the
  host (binned SAH), "cubql" (default) on the GPU for models of DEVICE_BVH_FACES triangles or more
  and on the host below. block_dim, max_registers, ordered_traversal, use_fast_math and
  mesh_bvh_frame are validated and recorded; the GB300 kernels choose their own launch shapes and
  traversal.

  Raises:
    ValueError: for invalid arguments, or a model with nothing to render.
  """
  device = kwargs.pop("device", None)
  hc = prepare_context(mjm, nworld, **kwargs)  # validates every argument before any device work
  device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
  return upload_context(hc, device)


def upload_context(hc: HostContext, device: torch.device) -> PbrRenderContext:
  """Device half of create_render_context: allocates every buffer and computes the GPU tables."""
  if device.type != "cuda":
    raise ValueError("the GB300 render path runs on a CUDA device")
  nworld = hc.nworld
  o = hc.outputs
  f32 = torch.float32
  rgb_stride = max(o["rgb_stride"], 1)
  out = Outputs(
    nrender=o["nrender"],
    cam_id_map=o["cam_id_map"],
    cam_res=o["cam_res"],
    render_rgb=o["render_rgb"],
    render_depth=o["render_depth"],
    render_seg=o["render_seg"],
    ray_adr=o["ray_adr"],
    rgb_adr=o["rgb_adr"],
    depth_adr=o["depth_adr"],
    seg_adr=o["seg_adr"],
    total_rays=o["total_rays"],
    rgb_data=torch.zeros((nworld, rgb_stride), dtype=torch.int32, device=device),
    depth_data=torch.zeros((nworld, max(o["depth_stride"], 1)), dtype=f32, device=device),
    seg_data=torch.zeros((nworld, max(o["seg_stride"], 1), 2), dtype=torch.int32, device=device),
    znear=hc.settings["znear"],
    zfar=hc.settings["zfar"],
  )
  op = hc.options
  hdr_pix = rgb_stride if (op["render_hdr"] or op["denoise"]) else 1
  guide_pix = rgb_stride if op["render_guides"] else 1
  aov_pix = rgb_stride if op["denoise"] else 1
  t = {k: torch.from_numpy(np.ascontiguousarray(v)).to(device) for k, v in hc.tables.items()}
  m = hc.meshes
  textures = tex_data = None
  tex_desc: list[Any] = []
  if hc.textures is not None:
    textures, tex_data = upload_textures(hc.textures, device)
    tex_desc = hc.textures.desc
  env = envmap_lib.upload_environments(hc.environments, device) if hc.environments is not None else None
  st = hc.settings
  blas = {k: _dev(m.get(k), device) for k in ("mesh_bounds", "blas_nodes", "blas_tris", "blas_root", "blas_tri_base")}
  if "device_sources" in m:
    built = build_mesh_bvhs_device(m["device_sources"], device)
    try:
      st["stack_depth"] = traversal_stack_depth(m["scene_levels"], built["mesh_levels"])
      blas = {k: built[k] for k in blas}
    except ValueError:
      # linear BVHs of degenerate meshes can be deeper than the traversal stacks: binned SAH instead
      warnings.warn("mesh_bvh_constructor='lbvh': a mesh BVH is too deep for the traversal stack; built with binned SAH on the host", stacklevel=3)
      names = m["device_sources"]["names"]
      sah = build_mesh_bvhs(None, [(n, *_source_arrays(m["device_sources"], i)) for i, n in enumerate(names)])
      st["stack_depth"] = traversal_stack_depth(m["scene_levels"], int(sah["mesh_levels"]))
      blas = {k: _dev(sah.get(k), device) for k in blas}
  rc = PbrRenderContext(
    nworld=nworld,
    base=out,
    light_model=op["light_model"],
    tone_mapper=op["tone_mapper"],
    use_shadows=op["use_shadows"],
    shadow_light_fraction=op["shadow_light_fraction"],
    geom_metallic=t["geom_metallic"],
    geom_roughness=t["geom_roughness"],
    geom_reflectance=t["geom_reflectance"],
    mat_reflectance=t["mat_reflectance"],
    light_intensity=t["light_intensity"],
    light_range=t["light_range"],
    light_bulbradius=t["light_bulbradius"],
    headlight_active=bool(st["headlight_active"]),
    headlight_diffuse=st["headlight_diffuse"],
    headlight_specular=st["headlight_specular"],
    headlight_intensity=st["headlight_intensity"],
    exposure=t["exposure"],
    ambient_radiance=t["ambient_radiance"],
    background_linear=op["background_linear"],
    has_env=op["has_env"],
    env_background=op["env_background"],
    env_id=t["env_id"],
    env_intensity=t["env_intensity"],
    env_yaw=t["env_yaw"],
    env_texel_angle=op["env_texel_angle"],
    samples_per_pixel=op["samples_per_pixel"],
    shadow_samples=op["shadow_samples"],
    has_transparency=op["has_transparency"],
    max_layers=op["max_layers"],
    has_reflection=op["has_reflection"],
    render_order=op["render_order"],
    schedule=op["schedule"],
    queue_item=op["queue_item"],
    wave_chunk_worlds=op["wave_chunk_worlds"],
    tier=op["tier"],
    path_samples=op["path_samples"],
    max_depth=op["max_depth"],
    rr_depth=op["rr_depth"],
    denoise=op["denoise"],
    denoise_iterations=op["denoise_iterations"],
    render_hdr=op["render_hdr"],
    hdr_data=torch.zeros((nworld, hdr_pix, 3), dtype=f32, device=device),
    render_guides=op["render_guides"],
    guide_albedo=torch.zeros((nworld, guide_pix, 3), dtype=f32, device=device),
    guide_normal=torch.zeros((nworld, guide_pix, 3), dtype=f32, device=device),
    cull_backfaces=op["cull_backfaces"],
    vertex_normals=op["vertex_normals"],
    specular_aa=op["specular_aa"],
    features=hc.features,
    enabled_geom_ids=_dev(hc.enabled_geom_ids, device),
    tlas_child=_dev(hc.tlas_child, device),
    world_blocks=torch.zeros((nworld, hc.world_block_floats), dtype=f32, device=device),
    world_block_floats=hc.world_block_floats,
    mesh_bounds=blas["mesh_bounds"],
    blas_nodes=blas["blas_nodes"],
    blas_tris=blas["blas_tris"],
    blas_root=blas["blas_root"],
    blas_tri_base=blas["blas_tri_base"],
    mesh_nface=list(m.get("mesh_nface", [])),
    nhfield=int(m.get("nhfield", 0)),
    textures=textures,
    tex_data=tex_data,
    tex_desc=tex_desc,
    dfg_lut=dfg_lut(device),
    dfg_size=DFG_LUT_SIZE,
    env=env,
    aov_guide=torch.zeros((nworld, aov_pix, 4), dtype=torch.int32, device=device),
    aov_emission=torch.zeros((nworld, aov_pix, 3), dtype=f32, device=device),
    denoise_buffers=(
      torch.zeros((nworld, aov_pix, 4), dtype=f32, device=device),
      torch.zeros((nworld, aov_pix, 4), dtype=f32, device=device),
    ),
    error_word=torch.zeros(1, dtype=torch.int32, device=device),
    work_counter=torch.zeros(4, dtype=torch.int32, device=device),
    device=device,
    block_dim=op["block_dim"],
    max_registers=op["max_registers"],
    ordered_traversal=op["ordered_traversal"],
  )
  rc._host_cache["settings"] = dict(hc.settings)
  if op["camera_rays"] is not None:
    from mujoco_warp_pbr_gb300.rays import set_camera_rays

    set_camera_rays(rc, op["camera_rays"])
  return rc

