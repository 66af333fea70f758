"""Seeded synthetic scenes: a small model builder and the benchmark workloads.

MuJoCo's XML compiler is not a dependency, so scenes are assembled directly as HostModel /
HostData arrays. Everything is drawn from numpy.random.default_rng(seed).

Workloads (the reference's configuration list, restated as concrete seeded scenes):
  * primitive_scene: ground plane + 8 primitives (spheres r~U(.05,.3), boxes half-extent
    ~U(.05,.25), capsules r~U(.03,.1) half-length~U(.05,.2), positions ~U([-1,1]^2 x [.1,.8]),
    uniform random orientations), base colour ~U(0,1)^3, roughness ~U(.05,1), metallic
    ~Bernoulli(.3), one directional + one point light (bulbradius .05, soft shadows), a flat grey
    sky (constant ambient radiance and background), 16 worlds, one 64x64 pinhole camera, fovy 45.
  * mesh_ibl_scene: 6 icospheres (subdivision 4, 5120 triangles) radially displaced by seeded
    value noise (amplitude .1) + 10 random primitives, a procedural 1024x512 equirect HDR
    (log-normal radiance, mu 0, sigma 1, plus a Gaussian sun lobe of peak 1e3), per-world
    roughness / metallic / rgba / environment rotation, seeded 512x512 albedo, ORM and
    tangent-space normal maps with mip chains, 2x2 supersampling, a mirror floor (reflectance
    .3), 4096 worlds, one 128x128 camera.
"""

from __future__ import annotations

import dataclasses
import math
from typing import Any

import numpy as np

from mujoco_warp_pbr_gb300.model import HostData
from mujoco_warp_pbr_gb300.model import HostModel

GEOM_PLANE, GEOM_HFIELD, GEOM_SPHERE, GEOM_CAPSULE, GEOM_ELLIPSOID, GEOM_CYLINDER, GEOM_BOX, GEOM_MESH = 0, 1, 2, 3, 4, 5, 6, 7
LIGHT_SPOT, LIGHT_DIRECTIONAL, LIGHT_POINT = 0, 1, 2


def quat_to_mat(q: np.ndarray) -> np.ndarray:
  """(..., 4) unit quaternions (w, x, y, z) -> (..., 9) row-major rotation matrices."""
  w, x, y, z = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
  m = np.stack(
    [
      1 - 2 * (y * y + z * z),
      2 * (x * y - z * w),
      2 * (x * z + y * w),
      2 * (x * y + z * w),
      1 - 2 * (x * x + z * z),
      2 * (y * z - x * w),
      2 * (x * z - y * w),
      2 * (y * z + x * w),
      1 - 2 * (x * x + y * y),
    ],
    axis=-1,
  )
  return m


def random_quats(rng: np.random.Generator, shape: tuple[int, ...]) -> np.ndarray:
  q = rng.normal(size=(*shape, 4))
  return q / np.linalg.norm(q, axis=-1, keepdims=True)


def look_at(pos: np.ndarray, target: np.ndarray, up: np.ndarray = np.array([0.0, 0.0, 1.0])) -> np.ndarray:
  """Camera frame (row-major 3x3, columns x right, y up, z backwards) looking from pos at target."""
  z = pos - target
  z = z / np.linalg.norm(z)
  x = np.cross(up, z)
  if np.linalg.norm(x) < 1e-9:
    x = np.array([1.0, 0.0, 0.0])
  x = x / np.linalg.norm(x)
  y = np.cross(z, x)
  return np.stack([x, y, z], axis=1).reshape(9)


@dataclasses.dataclass
class Builder:
  """Accumulates geoms, materials, lights, cameras, meshes and textures into a HostModel."""

  geoms: list[dict[str, Any]] = dataclasses.field(default_factory=list)
  mats: list[dict[str, Any]] = dataclasses.field(default_factory=list)
  lights: list[dict[str, Any]] = dataclasses.field(default_factory=list)
  cams: list[dict[str, Any]] = dataclasses.field(default_factory=list)
  meshes: list[dict[str, Any]] = dataclasses.field(default_factory=list)
  textures: list[dict[str, Any]] = dataclasses.field(default_factory=list)
  hfields: list[dict[str, Any]] = dataclasses.field(default_factory=list)
  headlight_active: bool = False
  headlight_ambient: tuple[float, float, float] = (0.0, 0.0, 0.0)
  headlight_diffuse: tuple[float, float, float] = (0.4, 0.4, 0.4)
  headlight_specular: tuple[float, float, float] = (0.5, 0.5, 0.5)

  def geom(self, type: int, size: Any, pos: Any = (0, 0, 0), mat: Any = None, rgba: Any = (0.5, 0.5, 0.5, 1.0), matid: int = -1, dataid: int = -1, group: int = 0) -> int:
    self.geoms.append(
      {
        "type": type,
        "size": np.asarray(size, float),
        "pos": np.asarray(pos, float),
        "mat": np.eye(3).reshape(9) if mat is None else np.asarray(mat, float).reshape(9),
        "rgba": np.asarray(rgba, float),
        "matid": matid,
        "dataid": dataid,
        "group": group,
      }
    )
    return len(self.geoms) - 1

  def material(self, rgba: Any = (1, 1, 1, 1), metallic: float = -1.0, roughness: float = -1.0, specular: float = 0.5, shininess: float = 0.5, reflectance: float = 0.0, emission: float = 0.0, texid: dict[int, int] | None = None, texrepeat: Any = (1, 1), texuniform: bool = False) -> int:
    ids = -np.ones(10, np.int32)
    for role, t in (texid or {}).items():
      ids[role] = t
    self.mats.append(
      {
        "rgba": np.asarray(rgba, float),
        "metallic": metallic,
        "roughness": roughness,
        "specular": specular,
        "shininess": shininess,
        "reflectance": reflectance,
        "emission": emission,
        "texid": ids,
        "texrepeat": np.asarray(texrepeat, float),
        "texuniform": int(texuniform),
      }
    )
    return len(self.mats) - 1

  def light(self, type: int, pos: Any = (0, 0, 3), dir: Any = (0, 0, -1), diffuse: Any = (0.7, 0.7, 0.7), intensity: float = 0.0, range: float = 10.0, bulbradius: float = 0.02, castshadow: bool = True, specular: Any = (0.3, 0.3, 0.3), cutoff: float = 45.0, exponent: float = 10.0) -> int:
    d = np.asarray(dir, float)
    self.lights.append(
      {
        "type": type,
        "pos": np.asarray(pos, float),
        "dir": d / np.linalg.norm(d),
        "diffuse": np.asarray(diffuse, float),
        "specular": np.asarray(specular, float),
        "intensity": intensity,
        "range": range,
        "bulbradius": bulbradius,
        "castshadow": int(castshadow),
        "cutoff": cutoff,
        "exponent": exponent,
      }
    )
    return len(self.lights) - 1

  def camera(self, pos: Any, target: Any = None, fovy: float = 45.0, resolution: tuple[int, int] = (64, 64), orthographic: bool = False, xyaxes: Any = None) -> int:
    """A camera looking from pos at target, or with MuJoCo's xyaxes (camera x and y axes)."""
    pos = np.asarray(pos, float)
    if xyaxes is not None:
      x = np.asarray(xyaxes[:3], float)
      y = np.asarray(xyaxes[3:], float)
      x = x / np.linalg.norm(x)
      y = y - x * np.dot(x, y)
      y = y / np.linalg.norm(y)
      mat = np.stack([x, y, np.cross(x, y)], axis=1).reshape(9)
    else:
      mat = look_at(pos, np.asarray(target, float))
    self.cams.append({"pos": pos, "mat": mat, "fovy": fovy, "res": resolution, "proj": int(orthographic)})
    return len(self.cams) - 1

  def mesh(self, vert: np.ndarray, face: np.ndarray, normal: np.ndarray | None = None, texcoord: np.ndarray | None = None, facenormal: np.ndarray | None = None) -> int:
    """A triangle mesh; normal: per-vertex normals (None: area-weighted vertex normals), or with
    facenormal (nface, 3) the normal index of each face corner."""
    self.meshes.append({"vert": np.asarray(vert, np.float32), "face": np.asarray(face, np.int32), "normal": normal, "texcoord": texcoord, "facenormal": facenormal})
    return len(self.meshes) - 1

  def hfield(self, elevation: np.ndarray, size: Any) -> int:
    """A height field: (nrow, ncol) elevations in [0, 1] (rows along y), size = x half-extent,
    y half-extent, elevation scale, base depth (MuJoCo's hfield size)."""
    self.hfields.append({"data": np.asarray(elevation, np.float32), "size": np.asarray(size, np.float32)})
    return len(self.hfields) - 1

  def texture(self, rgba: np.ndarray, colorspace: int = 0) -> int:
    """A 2D RGBA8 texture (h, w, 4); colorspace 0 auto (colour roles sRGB), 1 linear, 2 sRGB."""
    self.textures.append({"data": np.ascontiguousarray(rgba, np.uint8), "colorspace": colorspace})
    return len(self.textures) - 1

  def build(self) -> tuple[HostModel, HostData]:
    g, mt, lt, cm = self.geoms, self.mats, self.lights, self.cams
    nmat = len(mt)
    # meshes
    vadr, fadr, vnum, fnum, nadr, tadr = [], [], [], [], [], []
    verts, faces, normals, tcs, facenormals, facetcs = [], [], [], [], [], []
    nv = nf = nn = nt = 0
    for m in self.meshes:
      v, f = m["vert"], m["face"]
      n = m["normal"] if m["normal"] is not None else vertex_normals(v, f)
      vadr.append(nv)
      fadr.append(nf)
      vnum.append(len(v))
      fnum.append(len(f))
      nadr.append(nn)
      verts.append(v)
      faces.append(f)
      normals.append(n.astype(np.float32))
      facenormals.append(f if m.get("facenormal") is None else np.asarray(m["facenormal"], np.int32))
      if m["texcoord"] is not None:
        tadr.append(nt)
        tcs.append(np.asarray(m["texcoord"], np.float32))
        facetcs.append(f)
        nt += len(m["texcoord"])
      else:
        tadr.append(-1)
        facetcs.append(-np.ones_like(f))
      nv += len(v)
      nf += len(f)
      nn += len(n)
    # textures
    tex_adr, tex_w, tex_h, tex_data = [], [], [], []
    off = 0
    for t in self.textures:
      d = t["data"]
      tex_adr.append(off)
      tex_h.append(d.shape[0])
      tex_w.append(d.shape[1])
      tex_data.append(d.reshape(-1))
      off += d.size
    hf = self.hfields
    hf_adr = np.cumsum([0] + [h["data"].size for h in hf])[: len(hf)]
    center = np.mean([x["pos"] for x in g], axis=0) if g else np.zeros(3)
    mjm = HostModel(
      geom_type=np.array([x["type"] for x in g], np.int32),
      geom_size=np.array([x["size"] for x in g], np.float32),
      geom_rgba=np.array([x["rgba"] for x in g], np.float32),
      geom_matid=np.array([x["matid"] for x in g], np.int32),
      geom_group=np.array([x["group"] for x in g], np.int32),
      geom_dataid=np.array([x["dataid"] for x in g], np.int32),
      mat_rgba=np.array([x["rgba"] for x in mt], np.float32).reshape(nmat, 4),
      mat_emission=np.array([x["emission"] for x in mt], np.float32),
      mat_specular=np.array([x["specular"] for x in mt], np.float32),
      mat_shininess=np.array([x["shininess"] for x in mt], np.float32),
      mat_reflectance=np.array([x["reflectance"] for x in mt], np.float32),
      mat_metallic=np.array([x["metallic"] for x in mt], np.float32),
      mat_roughness=np.array([x["roughness"] for x in mt], np.float32),
      mat_texid=np.array([x["texid"] for x in mt], np.int32).reshape(nmat, 10),
      mat_texrepeat=np.array([x["texrepeat"] for x in mt], np.float32).reshape(nmat, 2),
      mat_texuniform=np.array([x["texuniform"] for x in mt], np.int32),
      light_type=np.array([x["type"] for x in lt], np.int32),
      light_castshadow=np.array([x["castshadow"] for x in lt], np.int32),
      light_active=np.ones(len(lt), np.int32),
      light_attenuation=np.tile([1.0, 0.0, 0.0], (len(lt), 1)).astype(np.float32),
      light_cutoff=np.array([x["cutoff"] for x in lt], np.float32),
      light_exponent=np.array([x["exponent"] for x in lt], np.float32),
      light_diffuse=np.array([x["diffuse"] for x in lt], np.float32).reshape(-1, 3),
      light_specular=np.array([x["specular"] for x in lt], np.float32).reshape(-1, 3),
      light_ambient=np.zeros((len(lt), 3), np.float32),
      light_intensity=np.array([x["intensity"] for x in lt], np.float32),
      light_range=np.array([x["range"] for x in lt], np.float32),
      light_bulbradius=np.array([x["bulbradius"] for x in lt], np.float32),
      cam_projection=np.array([x["proj"] for x in cm], np.int32),
      cam_fovy=np.array([x["fovy"] for x in cm], np.float32),
      cam_sensorsize=np.zeros((len(cm), 2), np.float32),
      cam_intrinsic=np.zeros((len(cm), 4), np.float32),
      cam_resolution=np.array([x["res"] for x in cm], np.int32),
      mesh_vertadr=np.array(vadr, np.int32),
      mesh_vertnum=np.array(vnum, np.int32),
      mesh_faceadr=np.array(fadr, np.int32),
      mesh_facenum=np.array(fnum, np.int32),
      mesh_normaladr=np.array(nadr, np.int32),
      mesh_texcoordadr=np.array(tadr, np.int32),
      mesh_vert=np.concatenate(verts) if verts else np.zeros((0, 3), np.float32),
      mesh_face=np.concatenate(faces) if faces else np.zeros((0, 3), np.int32),
      mesh_normal=np.concatenate(normals) if normals else np.zeros((0, 3), np.float32),
      mesh_facenormal=np.concatenate(facenormals) if facenormals else np.zeros((0, 3), np.int32),
      mesh_texcoord=np.concatenate(tcs) if tcs else np.zeros((0, 2), np.float32),
      mesh_facetexcoord=np.concatenate(facetcs) if facetcs else np.zeros((0, 3), np.int32),
      tex_type=np.zeros(len(self.textures), np.int32),
      tex_width=np.array(tex_w, np.int32),
      tex_height=np.array(tex_h, np.int32),
      tex_nchannel=np.full(len(self.textures), 4, np.int32),
      tex_adr=np.array(tex_adr, np.int64),
      tex_data=np.concatenate(tex_data) if tex_data else np.zeros(0, np.uint8),
      tex_colorspace=np.array([t["colorspace"] for t in self.textures], np.int32),
      hfield_size=np.array([h["size"] for h in hf], np.float32).reshape(-1, 4),
      hfield_nrow=np.array([h["data"].shape[0] for h in hf], np.int32),
      hfield_ncol=np.array([h["data"].shape[1] for h in hf], np.int32),
      hfield_adr=np.asarray(hf_adr, np.int32),
      hfield_data=np.concatenate([h["data"].reshape(-1) for h in hf]) if hf else np.zeros(0, np.float32),
      headlight_active=self.headlight_active,
      headlight_ambient=self.headlight_ambient,
      headlight_diffuse=self.headlight_diffuse,
      headlight_specular=self.headlight_specular,
      stat_center=tuple(float(c) for c in center),
      stat_extent=2.0,
    )
    mjd = HostData(
      geom_xpos=np.array([x["pos"] for x in g], np.float32),
      geom_xmat=np.array([x["mat"] for x in g], np.float32),
      cam_xpos=np.array([x["pos"] for x in cm], np.float32).reshape(-1, 3),
      cam_xmat=np.array([x["mat"] for x in cm], np.float32).reshape(-1, 9),
      light_xpos=np.array([x["pos"] for x in lt], np.float32).reshape(-1, 3),
      light_xdir=np.array([x["dir"] for x in lt], np.float32).reshape(-1, 3),
    )
    return mjm, mjd


def vertex_normals(vert: np.ndarray, face: np.ndarray) -> np.ndarray:
  """Area-weighted vertex normals of a triangle mesh."""
  v = np.asarray(vert, np.float64)
  f = np.asarray(face)
  fn = np.cross(v[f[:, 1]] - v[f[:, 0]], v[f[:, 2]] - v[f[:, 0]])
  n = np.zeros_like(v)
  for k in range(3):
    np.add.at(n, f[:, k], fn)
  return (n / np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-12)).astype(np.float32)


def icosphere(subdiv: int) -> tuple[np.ndarray, np.ndarray]:
  """Unit icosphere: 20 * 4^subdiv triangles (CCW, outward)."""
  t = (1.0 + 5.0**0.5) / 2.0
  v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
  f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6), (7, 1, 8),
       (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
  verts = [np.array(p, float) / np.linalg.norm(p) for p in v]
  faces = list(f)
  for _ in range(subdiv):
    cache: dict[tuple[int, int], int] = {}

    def mid(a: int, b: int) -> int:
      key = (min(a, b), max(a, b))
      if key not in cache:
        p = verts[a] + verts[b]
        verts.append(p / np.linalg.norm(p))
        cache[key] = len(verts) - 1
      return cache[key]

    new = []
    for a, b, c in faces:
      ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
      new += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
    faces = new
  return np.array(verts, np.float32), np.array(faces, np.int32)


def value_noise3(rng: np.random.Generator, points: np.ndarray, cells: int = 4) -> np.ndarray:
  """Seeded trilinear value noise in [-1, 1] on a cells^3 lattice over [-1, 1]^3."""
  lattice = rng.uniform(-1.0, 1.0, (cells + 1,) * 3)
  p = (np.clip(points, -1.0, 1.0) + 1.0) * 0.5 * cells
  i = np.minimum(p.astype(int), cells - 1)
  f = p - i
  f = f * f * (3 - 2 * f)
  out = np.zeros(len(points))
  for dx in (0, 1):
    for dy in (0, 1):
      for dz in (0, 1):
        w = (f[:, 0] if dx else 1 - f[:, 0]) * (f[:, 1] if dy else 1 - f[:, 1]) * (f[:, 2] if dz else 1 - f[:, 2])
        out += w * lattice[i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz]
  return out


def noise_image(rng: np.random.Generator, size: int, cells: int, channels: int) -> np.ndarray:
  """Seeded smooth 2D value noise (size, size, channels) in [0, 1], tileable."""
  out = np.zeros((size, size, channels))
  for c in range(channels):
    grid = rng.uniform(0, 1, (cells, cells))
    x = np.arange(size) / size * cells
    i0 = x.astype(int)
    f = x - i0
    f = f * f * (3 - 2 * f)
    i1 = (i0 + 1) % cells
    rows = grid[i0][:, i0] * (1 - f)[None, :] + grid[i0][:, i1] * f[None, :]
    rows1 = grid[i1][:, i0] * (1 - f)[None, :] + grid[i1][:, i1] * f[None, :]
    out[..., c] = rows * (1 - f)[:, None] + rows1 * f[:, None]
  return out


@dataclasses.dataclass
class SyntheticScene:
  """A seeded scene: host model and per-world data, context options and per-world tables."""

  name: str
  mjm: HostModel
  mjd: HostData
  nworld: int
  options: dict[str, Any]
  per_world: dict[str, np.ndarray]  # context / model arrays to replace after creation
  seed: int


def apply_per_world(scene: SyntheticScene, m: Any, rc: Any) -> None:
  """Assigns the scene's per-world tables to the device model and context."""
  import torch

  for name, value in scene.per_world.items():
    owner = m if name in ("geom_rgba", "mat_emission") else rc
    t = torch.as_tensor(value).to(rc.device)
    setattr(owner, name, t)


def _random_primitives(rng: np.random.Generator, n: int) -> list[tuple[int, np.ndarray]]:
  out = []
  for _ in range(n):
    kind = rng.integers(0, 3)
    if kind == 0:
      out.append((GEOM_SPHERE, np.array([rng.uniform(0.05, 0.3), 0.0, 0.0])))
    elif kind == 1:
      out.append((GEOM_BOX, rng.uniform(0.05, 0.25, 3)))
    else:
      out.append((GEOM_CAPSULE, np.array([rng.uniform(0.03, 0.1), rng.uniform(0.05, 0.2), 0.0])))
  return out


def primitive_scene(seed: int = 0, nworld: int = 16, res: int = 64, shadow_samples: int = 4) -> SyntheticScene:
  """Plain real-time tier, small primitive scene (see the module docstring)."""
  rng = np.random.default_rng(seed)
  b = Builder()
  b.geom(GEOM_PLANE, (3.0, 3.0, 0.1), rgba=(0.6, 0.6, 0.6, 1.0))
  prims = _random_primitives(rng, 8)
  for t, size in prims:
    b.geom(t, size)
  b.light(LIGHT_DIRECTIONAL, pos=(0, 0, 4), dir=(0.3, 0.2, -1.0), diffuse=(0.7, 0.7, 0.7), castshadow=True)
  b.light(LIGHT_POINT, pos=(0.5, -0.5, 2.0), diffuse=(0.5, 0.5, 0.5), range=10.0, bulbradius=0.05, castshadow=True)
  b.camera((0.0, -3.2, 2.2), (0.0, 0.0, 0.25), fovy=45.0, resolution=(res, res))
  mjm, mjd0 = b.build()
  ngeom = mjm.ngeom
  # per-world poses: the plane fixed, primitives at random positions and orientations
  xpos = np.broadcast_to(mjd0.geom_xpos, (nworld, ngeom, 3)).copy()
  xmat = np.broadcast_to(mjd0.geom_xmat, (nworld, ngeom, 9)).copy()
  xpos[:, 1:, :2] = rng.uniform(-1.0, 1.0, (nworld, ngeom - 1, 2))
  xpos[:, 1:, 2] = rng.uniform(0.1, 0.8, (nworld, ngeom - 1))
  xmat[:, 1:] = quat_to_mat(random_quats(rng, (nworld, ngeom - 1)))
  mjd = HostData(
    geom_xpos=xpos.astype(np.float32),
    geom_xmat=xmat.astype(np.float32),
    cam_xpos=np.broadcast_to(mjd0.cam_xpos, (nworld, mjm.ncam, 3)).astype(np.float32),
    cam_xmat=np.broadcast_to(mjd0.cam_xmat, (nworld, mjm.ncam, 9)).astype(np.float32),
    light_xpos=np.broadcast_to(mjd0.light_xpos, (nworld, mjm.nlight, 3)).astype(np.float32),
    light_xdir=np.broadcast_to(mjd0.light_xdir, (nworld, mjm.nlight, 3)).astype(np.float32),
  )
  rgba = np.concatenate([rng.uniform(0.0, 1.0, (nworld, ngeom, 3)), np.ones((nworld, ngeom, 1))], axis=-1)
  rgba[:, 0, :3] = 0.6
  roughness = rng.uniform(0.05, 1.0, (nworld, ngeom))
  metallic = (rng.uniform(0.0, 1.0, (nworld, ngeom)) < 0.3).astype(np.float64)
  metallic[:, 0] = 0.0
  roughness[:, 0] = 0.9
  grey = 0.5
  exposure = 1.0 / (1.2 * 2.0**14.96578428466209)
  srgb_grey = 1.055 * grey ** (1 / 2.4) - 0.055
  return SyntheticScene(
    name=f"primitives_{nworld}x{res}",
    mjm=mjm,
    mjd=mjd,
    nworld=nworld,
    options={
      "cam_res": (res, res),
      "render_rgb": True,
      "render_depth": True,
      "render_seg": True,
      "shadow_samples": shadow_samples,
      "background_color": (srgb_grey, srgb_grey, srgb_grey, 1.0),
    },
    per_world={
      "geom_rgba": rgba.astype(np.float32),
      "geom_roughness": roughness.astype(np.float32),
      "geom_metallic": metallic.astype(np.float32),
      # flat grey sky: constant display-relative radiance lighting every surface
      "ambient_radiance": np.full((1, 3), grey / exposure, np.float32),
    },
    seed=seed,
  )


def path_scene(seed: int = 0, nworld: int = 1024, res: int = 128, spp: int = 2, nquad: int = 3, ncam: int = 1) -> SyntheticScene:
  """Path-traced tier: the primitive scene plus emissive quads (thin boxes whose material emission,
  display-relative radiance, is drawn per world from U(1, 20)), next-event estimation over the
  lights, max depth 4, Russian roulette after bounce 2, `spp` jittered samples per pixel."""
  base = primitive_scene(seed=seed, nworld=nworld, res=res)
  rng = np.random.default_rng(seed + 7919)
  b = Builder()
  b.geom(GEOM_PLANE, (3.0, 3.0, 0.1), rgba=(0.6, 0.6, 0.6, 1.0))
  for t, size in _random_primitives(np.random.default_rng(seed), 8):
    b.geom(t, size)
  quads = []
  for _ in range(nquad):
    mat = b.material(rgba=(1, 1, 1, 1), roughness=1.0, specular=0.0, emission=1.0)
    pos = (rng.uniform(-1.2, 1.2), rng.uniform(-1.2, 1.2), rng.uniform(1.0, 1.6))
    quads.append(b.geom(GEOM_BOX, (rng.uniform(0.15, 0.35), rng.uniform(0.15, 0.35), 0.005), pos=pos, matid=mat, rgba=(1, 1, 1, 1)))
  b.light(LIGHT_DIRECTIONAL, pos=(0, 0, 4), dir=(0.3, 0.2, -1.0), diffuse=(0.7, 0.7, 0.7), castshadow=True)
  b.light(LIGHT_POINT, pos=(0.5, -0.5, 2.0), diffuse=(0.5, 0.5, 0.5), range=10.0, bulbradius=0.05, castshadow=True)
  b.camera((0.0, -3.2, 2.2), (0.0, 0.0, 0.25), fovy=45.0, resolution=(res, res))
  if ncam > 1:
    b.camera((2.8, 1.6, 1.8), (0.0, 0.0, 0.3), fovy=50.0, resolution=(res, res))
  mjm, mjd0 = b.build()
  ngeom, nprim = mjm.ngeom, 9
  xpos = np.broadcast_to(mjd0.geom_xpos, (nworld, ngeom, 3)).copy()
  xmat = np.broadcast_to(mjd0.geom_xmat, (nworld, ngeom, 9)).copy()
  xpos[:, :nprim] = base.mjd.geom_xpos
  xmat[:, :nprim] = base.mjd.geom_xmat
  mjd = HostData(
    geom_xpos=xpos.astype(np.float32),
    geom_xmat=xmat.astype(np.float32),
    cam_xpos=np.broadcast_to(mjd0.cam_xpos, (nworld, mjm.ncam, 3)).astype(np.float32),
    cam_xmat=np.broadcast_to(mjd0.cam_xmat, (nworld, mjm.ncam, 9)).astype(np.float32),
    light_xpos=base.mjd.light_xpos,
    light_xdir=base.mjd.light_xdir,
  )
  pw = dict(base.per_world)
  rgba = np.ones((nworld, ngeom, 4), np.float32)
  rgba[:, :nprim] = pw["geom_rgba"]
  rough = np.ones((nworld, ngeom), np.float32)
  rough[:, :nprim] = pw["geom_roughness"]
  metal = np.zeros((nworld, ngeom), np.float32)
  metal[:, :nprim] = pw["geom_metallic"]
  pw.update(
    {
      "geom_rgba": rgba,
      "geom_roughness": rough,
      "geom_metallic": metal,
      "mat_emission": rng.uniform(1.0, 20.0, (nworld, mjm.nmat)).astype(np.float32),
    }
  )
  options = dict(base.options)
  options.update({"tier": 1, "path_samples": spp, "max_depth": 4, "rr_depth": 2})
  options.pop("shadow_samples", None)
  return SyntheticScene(name=f"path_{nworld}x{res}_spp{spp}", mjm=mjm, mjd=mjd, nworld=nworld, options=options, per_world=pw, seed=seed)


def batched_scene(seed: int = 0, nworld: int = 2048, res: tuple[int, ...] = (64, 128, 256), fisheye: int = 2, nprim: int = 16) -> SyntheticScene:
  """Batched uneven workload: the primitive scene with `nprim` primitives and one camera per entry
  of `res` (square images, all looking at the scene from different places); camera `fisheye`
  renders per-pixel rays of a 180 degree equidistant fisheye, the others per-pixel pinhole rays.
  Per-world enable masks (alpha 0) leave between 2 and nprim primitives visible, uniformly."""
  from mujoco_warp_pbr_gb300 import rays

  rng = np.random.default_rng(seed)
  b = Builder()
  b.geom(GEOM_PLANE, (3.0, 3.0, 0.1), rgba=(0.6, 0.6, 0.6, 1.0))
  for t, size in _random_primitives(rng, nprim):
    b.geom(t, size)
  b.light(LIGHT_DIRECTIONAL, pos=(0, 0, 4), dir=(0.3, 0.2, -1.0), diffuse=(0.7, 0.7, 0.7), castshadow=True)
  b.light(LIGHT_POINT, pos=(0.5, -0.5, 2.0), diffuse=(0.5, 0.5, 0.5), range=10.0, bulbradius=0.05, castshadow=True)
  eyes = [(0.0, -3.2, 2.2), (2.6, -1.8, 1.6), (0.0, 0.0, 3.0), (-2.4, -2.0, 1.8)]
  for i, r in enumerate(res):
    b.camera(eyes[i % len(eyes)], (0.0, 0.0, 0.25) if i % len(eyes) != 2 else (0.0, 0.3, 0.0), fovy=45.0, resolution=(r, r))
  mjm, mjd0 = b.build()
  ngeom = mjm.ngeom
  xpos = np.broadcast_to(mjd0.geom_xpos, (nworld, ngeom, 3)).copy()
  xmat = np.broadcast_to(mjd0.geom_xmat, (nworld, ngeom, 9)).copy()
  xpos[:, 1:, :2] = rng.uniform(-1.0, 1.0, (nworld, ngeom - 1, 2))
  xpos[:, 1:, 2] = rng.uniform(0.1, 0.8, (nworld, ngeom - 1))
  xmat[:, 1:] = quat_to_mat(random_quats(rng, (nworld, ngeom - 1)))
  mjd = HostData(
    geom_xpos=xpos.astype(np.float32),
    geom_xmat=xmat.astype(np.float32),
    cam_xpos=np.broadcast_to(mjd0.cam_xpos, (nworld, mjm.ncam, 3)).astype(np.float32),
    cam_xmat=np.broadcast_to(mjd0.cam_xmat, (nworld, mjm.ncam, 9)).astype(np.float32),
    light_xpos=np.broadcast_to(mjd0.light_xpos, (nworld, mjm.nlight, 3)).astype(np.float32),
    light_xdir=np.broadcast_to(mjd0.light_xdir, (nworld, mjm.nlight, 3)).astype(np.float32),
  )
  rgba = np.concatenate([rng.uniform(0.0, 1.0, (nworld, ngeom, 3)), np.ones((nworld, ngeom, 1))], axis=-1)
  rgba[:, 0, :3] = 0.6
  # enable masks: k ~ U{2..nprim} visible primitives per world
  visible = rng.integers(2, nprim + 1, nworld)
  order = np.argsort(rng.uniform(size=(nworld, nprim)), axis=1)
  hidden = order >= visible[:, None]
  rgba[:, 1:, 3] = np.where(hidden, 0.0, 1.0)
  roughness = rng.uniform(0.05, 1.0, (nworld, ngeom))
  metallic = (rng.uniform(0.0, 1.0, (nworld, ngeom)) < 0.3).astype(np.float64)
  metallic[:, 0] = 0.0
  roughness[:, 0] = 0.9
  grey = 0.5
  exposure = 1.0 / (1.2 * 2.0**14.96578428466209)
  srgb_grey = 1.055 * grey ** (1 / 2.4) - 0.055
  bundle = [rays.fisheye_rays(r, r) if i == fisheye else rays.pinhole_rays(r, r, 45.0) for i, r in enumerate(res)]
  return SyntheticScene(
    name=f"batched_{nworld}x{'-'.join(map(str, res))}",
    mjm=mjm,
    mjd=mjd,
    nworld=nworld,
    options={
      "cam_res": [(r, r) for r in res],
      "render_rgb": True,
      "render_depth": True,
      "render_seg": True,
      "shadow_samples": 4,
      "background_color": (srgb_grey, srgb_grey, srgb_grey, 1.0),
      "camera_rays": bundle,
    },
    per_world={
      "geom_rgba": rgba.astype(np.float32),
      "geom_roughness": roughness.astype(np.float32),
      "geom_metallic": metallic.astype(np.float32),
      "ambient_radiance": np.full((1, 3), grey / exposure, np.float32),
    },
    seed=seed,
  )


def large_path_scene(seed: int = 0, nworld: int = 8192, res: int = 256, nenv: int = 4, env_width: int = 512) -> SyntheticScene:
  """Large path-traced run: the path scene with two cameras per world at res x res, per-world
  materials and emission, and `nenv` procedural HDR environments chosen per world (env_id
  uniform) with random rotation; 2 spp, depth 4."""
  sc = path_scene(seed=seed, nworld=nworld, res=res, spp=2, ncam=2)
  rng = np.random.default_rng(seed + 104729)
  sc.options["envmap"] = [procedural_env(np.random.default_rng(seed + 31 * k), env_width) for k in range(nenv)]
  sc.options["cam_res"] = [(res, res), (res, res)]
  sc.per_world["env_id"] = rng.integers(0, nenv, nworld).astype(np.int32)
  sc.per_world["env_yaw"] = rng.uniform(0.0, 2 * math.pi, nworld).astype(np.float32)
  return dataclasses.replace(sc, name=f"large_path_{nworld}x2x{res}_spp2")


def procedural_env(rng: np.random.Generator, width: int = 1024) -> np.ndarray:
  """Log-normal radiance (mu 0, sigma 1) smoothed, plus a Gaussian sun lobe of peak 1e3."""
  h = width // 2
  base = np.exp(rng.normal(0.0, 1.0, (h // 16, width // 16, 3)))
  img = np.repeat(np.repeat(base, 16, axis=0), 16, axis=1)
  theta = (np.arange(h) + 0.5) / h * np.pi
  phi = ((np.arange(width) + 0.5) / width - 0.5) * 2 * np.pi
  d = np.stack(np.broadcast_arrays(np.sin(theta)[:, None] * np.cos(phi)[None], np.sin(theta)[:, None] * np.sin(phi)[None], np.cos(theta)[:, None]), -1)
  sun = np.array([0.4, 0.3, 0.87])
  sun /= np.linalg.norm(sun)
  ang = np.arccos(np.clip(d @ sun, -1, 1))
  img = img + 1.0e3 * np.exp(-0.5 * (ang / 0.03) ** 2)[..., None]
  return img.astype(np.float32)


def hfield_scene(seed: int = 0, nworld: int = 8, res: int = 64, grid: int = 33, textured: bool = True) -> SyntheticScene:
  """Terrain: a seeded value-noise height field (grid x grid samples over 3 x 3 m, 0.5 m of relief
  on a 0.1 m base, a texture mapped over it) with five primitives resting above it, a sun and a
  soft-shadowed point light. Per world: the terrain's yaw, the primitives' poses and colours."""
  rng = np.random.default_rng(seed)
  b = Builder()
  elevation = noise_image(rng, grid - 1, 4, 1)[..., 0]
  elevation = np.concatenate([elevation, elevation[:1]], 0)
  elevation = np.concatenate([elevation, elevation[:, :1]], 1)  # (grid, grid), tileable noise closed
  hid = b.hfield(elevation, (1.5, 1.5, 0.5, 0.1))
  texid = {}
  if textured:
    albedo = noise_image(rng, 64, 8, 3) * 0.7 + 0.2
    rgba = np.concatenate([albedo, np.ones((64, 64, 1))], -1)
    texid = {1: b.texture((rgba * 255.0 + 0.5).astype(np.uint8))}
  ground = b.material(rgba=(0.5, 0.5, 0.5, 1), metallic=0.0, roughness=0.8, texid=texid, texrepeat=(2.0, 2.0))
  b.geom(GEOM_HFIELD, (1.5, 1.5, 0.3), matid=ground, dataid=hid)
  for t, size in _random_primitives(rng, 5):
    b.geom(t, size)
  b.light(LIGHT_DIRECTIONAL, pos=(0, 0, 4), dir=(0.4, 0.3, -1.0), diffuse=(0.8, 0.8, 0.8), castshadow=True)
  b.light(LIGHT_POINT, pos=(-0.6, 0.4, 1.6), diffuse=(0.4, 0.4, 0.4), range=10.0, bulbradius=0.05, castshadow=True)
  b.camera((0.0, -3.0, 2.0), (0.0, 0.0, 0.2), fovy=50.0, resolution=(res, res))
  mjm, mjd0 = b.build()
  ngeom = mjm.ngeom
  xpos = np.broadcast_to(mjd0.geom_xpos, (nworld, ngeom, 3)).copy()
  xmat = np.broadcast_to(mjd0.geom_xmat, (nworld, ngeom, 9)).copy()
  yaw = rng.uniform(0.0, 2.0 * np.pi, nworld)
  c, s_ = np.cos(yaw), np.sin(yaw)
  z, o = np.zeros(nworld), np.ones(nworld)
  xmat[:, 0] = np.stack([c, -s_, z, s_, c, z, z, z, o], -1)
  xpos[:, 1:, :2] = rng.uniform(-1.0, 1.0, (nworld, ngeom - 1, 2))
  xpos[:, 1:, 2] = rng.uniform(0.4, 0.9, (nworld, ngeom - 1))
  xmat[:, 1:] = quat_to_mat(random_quats(rng, (nworld, ngeom - 1)))
  mjd = HostData(
    geom_xpos=xpos.astype(np.float32),
    geom_xmat=xmat.astype(np.float32),
    cam_xpos=np.broadcast_to(mjd0.cam_xpos, (nworld, mjm.ncam, 3)).astype(np.float32),
    cam_xmat=np.broadcast_to(mjd0.cam_xmat, (nworld, mjm.ncam, 9)).astype(np.float32),
    light_xpos=np.broadcast_to(mjd0.light_xpos, (nworld, mjm.nlight, 3)).astype(np.float32),
    light_xdir=np.broadcast_to(mjd0.light_xdir, (nworld, mjm.nlight, 3)).astype(np.float32),
  )
  rgba = np.concatenate([rng.uniform(0.05, 0.95, (nworld, ngeom, 3)), np.ones((nworld, ngeom, 1))], axis=-1)
  rgba[:, 0] = (0.5, 0.5, 0.5, 1.0)  # the terrain keeps its material colour
  return SyntheticScene(
    name=f"hfield_{nworld}x{res}",
    mjm=mjm,
    mjd=mjd,
    nworld=nworld,
    options={"cam_res": (res, res), "render_rgb": True, "render_depth": True, "render_seg": True, "shadow_samples": 4},
    per_world={"geom_rgba": rgba.astype(np.float32)},
    seed=seed,
  )


def mesh_ibl_scene(seed: int = 0, nworld: int = 4096, res: int = 128, tex_size: int = 512, env_width: int = 1024) -> SyntheticScene:
  """Real-time tier at scale with meshes, IBL, textures and per-world randomisation."""
  rng = np.random.default_rng(seed)
  b = Builder()
  # textures: albedo (sRGB), ORM and normal (linear)
  albedo = noise_image(rng, tex_size, 8, 3) * 0.8 + 0.1
  orm = np.concatenate([0.8 + 0.2 * noise_image(rng, tex_size, 8, 1), 0.3 + 0.7 * noise_image(rng, tex_size, 16, 1), noise_image(rng, tex_size, 4, 1)], -1)
  height = noise_image(rng, tex_size, 32, 1)[..., 0]
  gy, gx = np.gradient(height * 8.0)
  n = np.stack([-gx, gy, np.ones_like(gx)], -1)
  n /= np.linalg.norm(n, axis=-1, keepdims=True)

  def u8(x: np.ndarray) -> np.ndarray:
    rgba = np.concatenate([np.clip(x, 0, 1), np.ones((*x.shape[:2], 1))], -1)
    return (rgba * 255.0 + 0.5).astype(np.uint8)

  t_albedo = b.texture(u8(albedo))
  t_orm = b.texture(u8(orm), colorspace=1)
  t_normal = b.texture(u8(n * 0.5 + 0.5), colorspace=1)
  textured = {1: t_albedo, 9: t_orm, 5: t_normal}
  floor_mat = b.material(rgba=(0.5, 0.5, 0.5, 1), metallic=0.0, roughness=0.6, reflectance=0.3, texid=textured, texrepeat=(1.0, 1.0), texuniform=True)
  mesh_mat = b.material(rgba=(0.5, 0.5, 0.5, 1), metallic=-1.0, roughness=-1.0, texid=textured, texrepeat=(2.0, 2.0))
  b.geom(GEOM_PLANE, (4.0, 4.0, 0.1), matid=floor_mat)
  v, f = icosphere(4)
  for k in range(6):
    disp = 1.0 + 0.1 * value_noise3(rng, v)
    r = rng.uniform(0.15, 0.3)
    vert = v * disp[:, None] * r
    uv = np.stack([np.arctan2(v[:, 1], v[:, 0]) / (2 * np.pi) + 0.5, np.arccos(np.clip(v[:, 2], -1, 1)) / np.pi], -1)
    mid = b.mesh(vert, f, texcoord=uv.astype(np.float32))
    b.geom(GEOM_MESH, (r, r, r), matid=mesh_mat, dataid=mid)
  for t, size in _random_primitives(rng, 10):
    b.geom(t, size)
  b.light(LIGHT_DIRECTIONAL, pos=(0, 0, 4), dir=(-0.4, -0.3, -0.87), diffuse=(0.8, 0.8, 0.8), castshadow=True)
  b.camera((0.0, -3.5, 2.4), (0.0, 0.0, 0.2), fovy=45.0, resolution=(res, res))
  mjm, mjd0 = b.build()
  ngeom = mjm.ngeom
  xpos = np.broadcast_to(mjd0.geom_xpos, (nworld, ngeom, 3)).copy()
  xmat = np.broadcast_to(mjd0.geom_xmat, (nworld, ngeom, 9)).copy()
  xpos[:, 1:, :2] = rng.uniform(-1.3, 1.3, (nworld, ngeom - 1, 2))
  xpos[:, 1:, 2] = rng.uniform(0.25, 0.9, (nworld, ngeom - 1))
  xmat[:, 1:] = quat_to_mat(random_quats(rng, (nworld, ngeom - 1)))
  mjd = HostData(
    geom_xpos=xpos.astype(np.float32),
    geom_xmat=xmat.astype(np.float32),
    cam_xpos=np.broadcast_to(mjd0.cam_xpos, (nworld, mjm.ncam, 3)).astype(np.float32),
    cam_xmat=np.broadcast_to(mjd0.cam_xmat, (nworld, mjm.ncam, 9)).astype(np.float32),
    light_xpos=np.broadcast_to(mjd0.light_xpos, (nworld, mjm.nlight, 3)).astype(np.float32),
    light_xdir=np.broadcast_to(mjd0.light_xdir, (nworld, mjm.nlight, 3)).astype(np.float32),
  )
  rgba = np.concatenate([rng.uniform(0.05, 0.95, (nworld, ngeom, 3)), np.ones((nworld, ngeom, 1))], axis=-1)
  rgba[:, 0] = (0.5, 0.5, 0.5, 1.0)  # floor keeps its material colour
  roughness = rng.uniform(0.05, 1.0, (nworld, ngeom))
  metallic = rng.uniform(0.0, 1.0, (nworld, ngeom))
  roughness[:, 0] = 0.6
  metallic[:, 0] = 0.0
  env = procedural_env(rng, env_width)
  return SyntheticScene(
    name=f"mesh_ibl_{nworld}x{res}",
    mjm=mjm,
    mjd=mjd,
    nworld=nworld,
    options={
      "cam_res": (res, res),
      "render_rgb": True,
      "render_depth": True,
      "render_seg": True,
      "samples_per_pixel": 2,
      "envmap": env,
    },
    per_world={
      "geom_rgba": rgba.astype(np.float32),
      "geom_roughness": roughness.astype(np.float32),
      "geom_metallic": metallic.astype(np.float32),
      "env_yaw": rng.uniform(0.0, 2 * math.pi, nworld).astype(np.float32),
    },
    seed=seed,
  )
