"""Host model/data descriptions and their device copies.

The reference takes a mujoco.MjModel (host) plus mujoco_warp Model / Data (device). MuJoCo and
MuJoCo Warp are not dependencies of this package, so:

  * `HostModel` / `HostData` hold the MjModel / MjData fields the render path reads, under
    MuJoCo's names (numpy arrays). A real mujoco.MjModel / MjData works too: `as_host_model`
    flattens the MjModel's nested headlight / statistic / clip-plane structs, and
    create_render_context, put_model and put_data call it.
  * `put_model` / `put_data` make the device `Model` / `Data` (torch CUDA tensors with MuJoCo
    Warp's field names and batching: per-world tables have a leading dimension of 1 or nworld),
    like mujoco_warp.put_model / put_data. Objects exposing __cuda_array_interface__ (e.g. Warp
    arrays of a real mujoco_warp.Data) can be assigned to these fields directly.
"""

from __future__ import annotations

import dataclasses
from typing import Any

import numpy as np
import torch

NTEXROLE = 10


@dataclasses.dataclass
class HostModel:
  """MjModel fields used by the renderer (MuJoCo names and conventions)."""

  # geoms
  geom_type: np.ndarray  # (ngeom,) mjtGeom
  geom_size: np.ndarray  # (ngeom, 3)
  geom_rgba: np.ndarray  # (ngeom, 4)
  geom_matid: np.ndarray  # (ngeom,)
  geom_group: np.ndarray  # (ngeom,)
  geom_dataid: np.ndarray  # (ngeom,) mesh id of mesh geoms, height-field id of height fields, else -1
  # materials
  mat_rgba: np.ndarray  # (nmat, 4)
  mat_emission: np.ndarray  # (nmat,)
  mat_specular: np.ndarray  # (nmat,)
  mat_shininess: np.ndarray  # (nmat,)
  mat_reflectance: np.ndarray  # (nmat,)
  mat_metallic: np.ndarray  # (nmat,) -1: unset
  mat_roughness: np.ndarray  # (nmat,) -1: unset
  mat_texid: np.ndarray  # (nmat, 10)
  mat_texrepeat: np.ndarray  # (nmat, 2)
  mat_texuniform: np.ndarray  # (nmat,)
  # lights
  light_type: np.ndarray  # (nlight,) mjtLightType
  light_castshadow: np.ndarray
  light_active: np.ndarray
  light_attenuation: np.ndarray  # (nlight, 3)
  light_cutoff: np.ndarray
  light_exponent: np.ndarray
  light_diffuse: np.ndarray  # (nlight, 3)
  light_specular: np.ndarray
  light_ambient: np.ndarray
  light_intensity: np.ndarray  # 0: unset (calibrated fallback)
  light_range: np.ndarray
  light_bulbradius: np.ndarray
  # cameras
  cam_projection: np.ndarray  # (ncam,)
  cam_fovy: np.ndarray  # (ncam,)
  cam_sensorsize: np.ndarray  # (ncam, 2)
  cam_intrinsic: np.ndarray  # (ncam, 4)
  cam_resolution: np.ndarray  # (ncam, 2)
  # meshes (concatenated, MuJoCo layout)
  mesh_vertadr: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))
  mesh_vertnum: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))
  mesh_faceadr: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))
  mesh_facenum: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))
  mesh_normaladr: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))
  mesh_texcoordadr: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))
  mesh_vert: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 3), np.float32))
  mesh_face: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 3), np.int32))
  mesh_normal: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 3), np.float32))
  mesh_facenormal: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 3), np.int32))
  mesh_texcoord: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 2), np.float32))
  mesh_facetexcoord: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 3), np.int32))
  # height fields (MuJoCo layout: nrow x ncol elevations in [0, 1], row-major, rows along y;
  # size = x half-extent, y half-extent, elevation scale, base depth)
  hfield_size: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 4), np.float32))
  hfield_nrow: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))
  hfield_ncol: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))
  hfield_adr: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))
  hfield_data: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.float32))
  # textures (2D only; RGB or RGBA bytes concatenated in tex_data)
  tex_type: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))  # 0: 2D
  tex_width: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))
  tex_height: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))
  tex_nchannel: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))
  tex_adr: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int64))
  tex_data: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.uint8))
  tex_colorspace: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0, np.int32))  # 0 auto 1 linear 2 sRGB
  # visual
  headlight_active: bool = False
  headlight_ambient: tuple[float, float, float] = (0.1, 0.1, 0.1)
  headlight_diffuse: tuple[float, float, float] = (0.4, 0.4, 0.4)
  headlight_specular: tuple[float, float, float] = (0.5, 0.5, 0.5)
  stat_center: tuple[float, float, float] = (0.0, 0.0, 0.0)
  stat_extent: float = 1.0
  znear: float = 0.01
  zfar: float = 0.0

  @property
  def ngeom(self) -> int:
    return int(len(self.geom_type))

  @property
  def nmat(self) -> int:
    return int(len(self.mat_rgba))

  @property
  def nlight(self) -> int:
    return int(len(self.light_type))

  @property
  def ncam(self) -> int:
    return int(len(self.cam_projection))

  @property
  def nmesh(self) -> int:
    return int(len(self.mesh_vertadr))

  @property
  def nhfield(self) -> int:
    return int(len(self.hfield_nrow))

  @property
  def ntex(self) -> int:
    return int(len(self.tex_type))


def as_host_model(mjm: Any) -> Any:
  """The model as the renderer reads it: a HostModel (or any object already carrying HostModel's
  flat names) as it is; a mujoco.MjModel converted.

  An MjModel keeps the headlight, the model statistics and the clip planes in nested structs
  (mjm.vis.headlight.active / ambient / diffuse / specular, mjm.stat.center / extent,
  mjm.vis.map.znear / zfar as fractions of the extent), which the reference reads there
  (mujoco_warp_pbr/_src/io.py:242-243, lights.py:146-147); every other field has the same name in
  both. Fields a MuJoCo release lacks fall back to HostModel's defaults, or raise ValueError when
  HostModel has none.
  """
  if isinstance(mjm, HostModel) or not hasattr(mjm, "vis") or not hasattr(mjm, "stat"):
    return mjm
  values: dict[str, Any] = {}
  missing = []
  for f in dataclasses.fields(HostModel):
    if hasattr(mjm, f.name):
      values[f.name] = np.array(getattr(mjm, f.name), copy=True)
    elif f.default is dataclasses.MISSING and f.default_factory is dataclasses.MISSING:
      missing.append(f.name)
  if missing:
    raise ValueError(f"the model lacks {', '.join(missing)} (the renderer needs MuJoCo 3.3 or later)")
  hl = mjm.vis.headlight
  extent = float(mjm.stat.extent)
  values.update(
    headlight_active=bool(int(hl.active)),
    headlight_ambient=tuple(float(c) for c in hl.ambient),
    headlight_diffuse=tuple(float(c) for c in hl.diffuse),
    headlight_specular=tuple(float(c) for c in hl.specular),
    stat_center=tuple(float(c) for c in mjm.stat.center),
    stat_extent=extent,
    znear=float(mjm.vis.map.znear) * extent,
    zfar=float(mjm.vis.map.zfar) * extent,
  )
  return HostModel(**values)


@dataclasses.dataclass
class HostData:
  """MjData fields used by the renderer, for one world (or (nworld, ...) per world)."""

  geom_xpos: np.ndarray  # ([nworld,] ngeom, 3)
  geom_xmat: np.ndarray  # ([nworld,] ngeom, 9)
  cam_xpos: np.ndarray  # ([nworld,] ncam, 3)
  cam_xmat: np.ndarray  # ([nworld,] ncam, 9)
  light_xpos: np.ndarray  # ([nworld,] nlight, 3)
  light_xdir: np.ndarray  # ([nworld,] nlight, 3)


class Model:
  """Device model: torch tensors under MuJoCo Warp's names (see the module docstring)."""

  def __init__(self, **fields: Any):
    self.__dict__.update(fields)


class Data:
  """Device data: geom_xpos (nworld, ngeom, 3), geom_xmat (nworld, ngeom, 3, 3), cam_xpos,
  cam_xmat, light_xpos, light_xdir (nworld, n, 3 / 3x3)."""

  def __init__(self, nworld: int, **fields: Any):
    self.nworld = nworld
    self.__dict__.update(fields)


def _device(device: Any) -> torch.device:
  if device is None:
    return torch.device("cuda", torch.cuda.current_device()) if torch.cuda.is_available() else torch.device("cpu")
  return torch.device(device)


def _t(a: Any, dtype: torch.dtype, device: torch.device) -> torch.Tensor:
  arr = np.ascontiguousarray(a)
  if not arr.flags.writeable:  # e.g. a broadcast view: torch wants memory it may write
    arr = arr.copy()
  return torch.as_tensor(arr, dtype=dtype).to(device)


def put_model(mjm: HostModel, device: Any = None) -> Model:
  """Device copy of the model (mujoco_warp.put_model's role); per-world tables get batch 1. Takes a
  HostModel or a mujoco.MjModel (as_host_model)."""
  mjm = as_host_model(mjm)
  dev = _device(device)
  f32, i32 = torch.float32, torch.int32

  def b(a: Any, dtype: torch.dtype, tail: tuple[int, ...]) -> torch.Tensor:
    return _t(np.asarray(a).reshape((1, -1, *tail)), dtype, dev)

  return Model(
    ngeom=mjm.ngeom,
    nmat=mjm.nmat,
    nlight=mjm.nlight,
    ncam=mjm.ncam,
    nmesh=mjm.nmesh,
    geom_type=_t(mjm.geom_type, i32, dev),
    geom_dataid=b(mjm.geom_dataid, i32, ()),
    geom_matid=b(mjm.geom_matid, i32, ()),
    geom_size=b(mjm.geom_size, f32, (3,)),
    geom_rgba=b(mjm.geom_rgba, f32, (4,)),
    mat_rgba=b(mjm.mat_rgba if mjm.nmat else np.zeros((1, 4)), f32, (4,)),
    mat_emission=b(mjm.mat_emission if mjm.nmat else np.zeros(1), f32, ()),
    mat_texid=b(mjm.mat_texid if mjm.nmat else -np.ones((1, NTEXROLE)), i32, (NTEXROLE,)),
    mat_texrepeat=b(mjm.mat_texrepeat if mjm.nmat else np.ones((1, 2)), f32, (2,)),
    mat_texuniform=b(mjm.mat_texuniform if mjm.nmat else np.zeros(1), i32, ()),
    light_type=b(mjm.light_type if mjm.nlight else np.zeros(1), i32, ()),
    light_castshadow=b(mjm.light_castshadow if mjm.nlight else np.zeros(1), i32, ()),
    light_active=b(mjm.light_active if mjm.nlight else np.zeros(1), i32, ()),
    light_attenuation=b(mjm.light_attenuation if mjm.nlight else np.zeros((1, 3)), f32, (3,)),
    light_cutoff=b(mjm.light_cutoff if mjm.nlight else np.zeros(1), f32, ()),
    light_exponent=b(mjm.light_exponent if mjm.nlight else np.zeros(1), f32, ()),
    light_diffuse=b(mjm.light_diffuse if mjm.nlight else np.zeros((1, 3)), f32, (3,)),
    light_specular=b(mjm.light_specular if mjm.nlight else np.zeros((1, 3)), f32, (3,)),
    cam_projection=_t(mjm.cam_projection, i32, dev),
    cam_fovy=b(mjm.cam_fovy, f32, ()),
    cam_sensorsize=_t(np.asarray(mjm.cam_sensorsize).reshape(-1, 2), f32, dev),
    cam_intrinsic=b(mjm.cam_intrinsic, f32, (4,)),
    mesh_vertadr=_t(mjm.mesh_vertadr, i32, dev),
    mesh_faceadr=_t(mjm.mesh_faceadr, i32, dev),
    mesh_normaladr=_t(mjm.mesh_normaladr, i32, dev),
    mesh_texcoordadr=_t(mjm.mesh_texcoordadr, i32, dev),
    mesh_vert=_t(np.asarray(mjm.mesh_vert).reshape(-1, 3), f32, dev),
    mesh_face=_t(np.asarray(mjm.mesh_face).reshape(-1, 3), i32, dev),
    mesh_normal=_t(np.asarray(mjm.mesh_normal).reshape(-1, 3), f32, dev),
    mesh_facenormal=_t(np.asarray(mjm.mesh_facenormal).reshape(-1, 3), i32, dev),
    mesh_texcoord=_t(np.asarray(mjm.mesh_texcoord).reshape(-1, 2), f32, dev),
    mesh_facetexcoord=_t(np.asarray(mjm.mesh_facetexcoord).reshape(-1, 3), i32, dev),
  )


def put_data(mjm: HostModel, mjd: HostData, nworld: int = 1, device: Any = None) -> Data:
  """Device data for nworld worlds (mujoco_warp.put_data's role): a single world's arrays are
  replicated; arrays with a leading nworld dimension are copied as they are."""
  mjm = as_host_model(mjm)
  dev = _device(device)

  def per_world(a: np.ndarray, n: int, k: int) -> torch.Tensor:
    a = np.asarray(a, dtype=np.float32)
    if a.ndim == 2 or (a.ndim == 3 and a.shape[0] != nworld) or n == 0:
      a = np.broadcast_to(a.reshape(1, n, k), (nworld, n, k))
    return _t(a.reshape(nworld, n, k), torch.float32, dev)

  return Data(
    nworld,
    geom_xpos=per_world(mjd.geom_xpos, mjm.ngeom, 3),
    geom_xmat=per_world(mjd.geom_xmat, mjm.ngeom, 9),
    cam_xpos=per_world(mjd.cam_xpos, mjm.ncam, 3),
    cam_xmat=per_world(mjd.cam_xmat, mjm.ncam, 9),
    light_xpos=per_world(mjd.light_xpos, mjm.nlight, 3),
    light_xdir=per_world(mjd.light_xdir, mjm.nlight, 3),
  )
