"""Host preparation of a scene for the CPU oracle — TEST INFRASTRUCTURE, independent of the product.

A restatement of what the reference resolves on the host when it creates a render context, so that
the oracle's inputs do not come from the product's own host code (mujoco_warp_pbr_gb300.context):

  materials      mujoco_warp_pbr/_src/material.py:90-182 (effective rgba, GLTF / HEURISTIC rules)
  features       mujoco_warp_pbr/_src/material.py:185-221 (texture roles, alpha maps)
  lighting       mujoco_warp_pbr/_src/io.py:223-248, lights.py:134-148 (exposure, intensities,
                 fallback intensity, ambient)
  flags          mujoco_warp_pbr/_src/io.py:288-300 (translucency, reflection)
  textures       mujoco_warp_pbr/_src/texture.py:40-101 (sRGB colour roles to linear float16,
                 data roles RGBA8, 1x1 placeholders)
  environments   mujoco_warp_pbr/_src/envmap.py:143-150, 224-249, 365-380, 409-432, 517-567
                 (downsampling, SH9 irradiance, sampling tables, shared table resolution)
  output layout  MuJoCo Warp's create_render_context as called at mujoco_warp_pbr/_src/io.py:510-527
                 (active cameras, per-output pixel addresses), third party; restated from its use

Models are read by MjModel field names (duck typing: HostModel or a MuJoCo MjModel's flat fields);
the environment's MJCF skybox (io.py:267-285) is not restated: the oracle's scenes carry explicit
environment images. The settings are the MjpbrSettings fields of include/mjpbr.h.
"""

from __future__ import annotations

import dataclasses
import math
from typing import Any

import numpy as np

from oracle import scene_struct as ss

# include/mjpbr.h enums
GEOM_PLANE, GEOM_HFIELD, GEOM_MESH, GEOM_SDF = 0, 1, 7, 8
LIGHT_DIRECTIONAL = 1
LIGHT_MODEL_PHYSICAL = 0
UNSET_GLTF, UNSET_HEURISTIC = 0, 1
TIER_REALTIME = 0
TEX_RGBA8, TEX_RGBA16F = 0, 1
ROLE_RGB, ROLE_OCCLUSION, ROLE_ROUGHNESS, ROLE_METALLIC, ROLE_NORMAL, ROLE_OPACITY, ROLE_EMISSIVE, ROLE_RGBA, ROLE_ORM = range(1, 10)
COLOR_ROLES = [ROLE_RGB, ROLE_RGBA, ROLE_EMISSIVE]

# reference constants (material.py:62-63,90; color.py:32; io.py:54; envmap.py)
DEFAULT_SHININESS = 0.5
DEFAULT_SPECULAR = 0.5
DEFAULT_GEOM_RGBA = (0.5, 0.5, 0.5, 1.0)
LUMINANCE_WEIGHTS = (0.2126, 0.7152, 0.0722)
DEFAULT_EV100 = 14.96578428466209
MAX_RADIANCE_WIDTH = 2048
PREFILTER_WIDTH = 256
PREFILTER_LEVELS = 8
CDF_WIDTH = 256
DENOISE_SIGMAS = {"denoise_sigma_color": 4.0, "denoise_sigma_normal": 128.0, "denoise_sigma_depth": 0.02, "denoise_sigma_albedo": 0.05}


def srgb_to_linear(x: Any) -> np.ndarray:
  """The sRGB EOTF (color.py:96-99)."""
  x = np.asarray(x, dtype=np.float64)
  return np.where(x <= 0.04045, x / 12.92, ((x + 0.055) / 1.055) ** 2.4)


SRGB_TABLE = srgb_to_linear(np.arange(256) / 255.0).astype(np.float16)


# ------------------------------------------------------------------ materials


def effective_geom_rgba(mjm: Any) -> np.ndarray:
  rgba = np.array(mjm.geom_rgba, dtype=np.float64).reshape(-1, 4)
  if not mjm.nmat:
    return rgba
  matid = np.asarray(mjm.geom_matid).reshape(-1)
  inherit = (matid >= 0) & np.all(np.isclose(rgba, DEFAULT_GEOM_RGBA), axis=1)
  rgba[inherit] = np.asarray(mjm.mat_rgba).reshape(-1, 4)[matid[inherit]]
  return rgba


def heuristic(rgba: np.ndarray, shininess: float, has_material: bool) -> tuple[float, float, float]:
  r, g, b = rgba[:3]
  if not has_material:
    brightness = (r + g + b) / 3.0
    if brightness < 0.25:
      return 0.4, 0.45, 0.35
    if brightness > 0.8 or (r > 0.7 and g < 0.3):
      return 0.0, 0.4, 0.25
    return 0.0, 0.5, 0.2
  lum = float(np.dot(rgba[:3], LUMINANCE_WEIGHTS))
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
  if shininess > 0.0 and shininess != DEFAULT_SHININESS:
    roughness = float(np.clip(roughness * (1.3 - shininess), 0.06, 1.0))
  return metallic, roughness, reflectance


def resolve_materials(mjm: Any, unset_material: int, default_material: dict | None) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
  default_material = default_material or {}
  ngeom = len(np.asarray(mjm.geom_type).reshape(-1))
  out = np.zeros((3, ngeom), np.float32)
  rgba_all = effective_geom_rgba(mjm)
  gtype = np.asarray(mjm.geom_type).reshape(-1)
  for g in range(ngeom):
    mat = int(np.asarray(mjm.geom_matid).reshape(-1)[g])
    has = mat >= 0
    shininess = float(np.asarray(mjm.mat_shininess)[mat]) if has else DEFAULT_SHININESS
    specular = float(np.asarray(mjm.mat_specular)[mat]) if has else DEFAULT_SPECULAR
    am = float(np.asarray(mjm.mat_metallic)[mat]) if has else -1.0
    ar = float(np.asarray(mjm.mat_roughness)[mat]) if has else -1.0
    if unset_material == UNSET_HEURISTIC and am < 0.0 and ar < 0.0:
      m, r, f = heuristic(rgba_all[g], shininess, has)
      if int(gtype[g]) == GEOM_PLANE:
        m, r, f = 0.0, 1.0, 0.0
    else:
      m, r, f = 0.0, float(np.clip(1.0 - shininess, 0.0, 1.0)), specular
    if am < 0.0 and "metallic" in default_material:
      m = default_material["metallic"]
    if ar < 0.0 and "roughness" in default_material:
      r = default_material["roughness"]
    out[0, g] = am if am >= 0.0 else m
    out[1, g] = ar if ar >= 0.0 else r
    out[2, g] = f
  return out[0], out[1], out[2]


def surface_features(mjm: Any, use_textures: bool, specular_aa: bool, mats: np.ndarray) -> dict[str, bool]:
  texid = np.asarray(mjm.mat_texid).reshape(-1, 10)[mats] if mjm.nmat else np.full((0, 10), -1)

  def has(*roles: int) -> bool:
    return use_textures and bool(np.any(texid[:, list(roles)] >= 0))

  f = {
    "base_color_map": has(ROLE_RGB, ROLE_RGBA),
    "normal_map": has(ROLE_NORMAL),
    "orm_map": has(ROLE_ORM, ROLE_OCCLUSION, ROLE_ROUGHNESS, ROLE_METALLIC),
    "emissive_map": has(ROLE_EMISSIVE),
    "opacity_map": has(ROLE_OPACITY),
    "specular_aa": bool(specular_aa),
  }
  f["textures"] = any(f[k] for k in ("base_color_map", "normal_map", "orm_map", "emissive_map", "opacity_map"))
  f["alpha_map"] = False
  if use_textures:
    for role, channel in ((ROLE_RGBA, 3), (ROLE_OPACITY, 0)):
      for t in np.unique(texid[:, role]) if len(texid) else []:
        if t < 0:
          continue
        w, h, nc = int(mjm.tex_width[t]), int(mjm.tex_height[t]), int(mjm.tex_nchannel[t])
        data = np.asarray(mjm.tex_data)[int(mjm.tex_adr[t]) : int(mjm.tex_adr[t]) + w * h * nc].reshape(-1, nc)
        if channel < nc and np.any(data[:, channel] < 255):
          f["alpha_map"] = True
  return f


# ------------------------------------------------------------------ lighting


def exposure_from_ev100(ev100: float) -> float:
  return 1.0 / (1.2 * math.pow(2.0, ev100))


def resolve_lighting(mjm: Any, light_xpos: np.ndarray, light_model: int, ev100: float) -> tuple[float, np.ndarray, np.ndarray]:
  physical = light_model == LIGHT_MODEL_PHYSICAL
  exposure = exposure_from_ev100(ev100) if physical else 1.0
  ltype = np.asarray(mjm.light_type).reshape(-1)
  nlight = len(ltype)
  intensity = np.array(mjm.light_intensity, dtype=np.float32).reshape(nlight)
  diffuse = np.asarray(mjm.light_diffuse, np.float64).reshape(-1, 3)
  for i in range(nlight):
    if intensity[i] > 0.0:
      intensity[i] /= max(float(np.max(diffuse[i])), 1e-6)
      continue
    illuminance = math.pi / exposure
    if int(ltype[i]) == LIGHT_DIRECTIONAL:
      intensity[i] = illuminance
    else:
      distance = float(np.linalg.norm(np.asarray(light_xpos[i], np.float64) - np.asarray(mjm.stat_center, np.float64)))
      distance = max(distance, 0.1 * float(mjm.stat_extent), 1e-3)
      intensity[i] = illuminance * distance * distance
  ambient = np.zeros(3, np.float32)
  if mjm.headlight_active:
    ambient += np.asarray(mjm.headlight_ambient, np.float32)
  if physical:
    ambient /= exposure
  elif nlight:
    ambient += np.sum(np.asarray(mjm.light_ambient, np.float32).reshape(-1, 3)[np.asarray(mjm.light_active).astype(bool)], axis=0)
  return exposure, intensity, ambient


# ------------------------------------------------------------------ textures


def texture_images(mjm: Any, used: np.ndarray) -> list[tuple[int, np.ndarray]]:
  out = []
  mat_texid = np.asarray(mjm.mat_texid).reshape(-1, 10) if mjm.nmat else np.zeros((0, 10), np.int32)
  for t in range(mjm.ntex):
    if not used[t] or int(mjm.tex_type[t]) != 0:
      out.append((TEX_RGBA8, np.full((1, 1, 4), 255, np.uint8)))
      continue
    w, h, nc = int(mjm.tex_width[t]), int(mjm.tex_height[t]), int(mjm.tex_nchannel[t])
    data = np.asarray(mjm.tex_data)[int(mjm.tex_adr[t]) : int(mjm.tex_adr[t]) + w * h * nc].reshape(h, w, nc)
    rgba = np.full((h, w, 4), 255, dtype=np.uint8)
    if nc == 1:
      rgba[..., :3] = data
    else:
      rgba[..., :nc] = data
    cs = int(mjm.tex_colorspace[t])  # 0 auto, 1 linear, 2 sRGB
    srgb = cs == 2 or (cs == 0 and bool(np.isin(t, mat_texid[:, COLOR_ROLES])))
    if srgb:
      out.append((TEX_RGBA16F, np.concatenate([SRGB_TABLE[rgba[..., :3]], (rgba[..., 3:] / 255.0).astype(np.float16)], axis=-1)))
    else:
      out.append((TEX_RGBA8, rgba))
  return out


# ------------------------------------------------------------------ environments


def downsample(image: np.ndarray, max_width: int) -> np.ndarray:
  while image.shape[1] > max_width:
    h, w = image.shape[0] // 2 * 2, image.shape[1] // 2 * 2
    image = image[:h, :w].reshape(h // 2, 2, w // 2, 2, -1).mean(axis=(1, 3))
  return image


def downsampled_shape(shape: tuple[int, ...], max_width: int) -> tuple[int, int]:
  h, w = shape[0], shape[1]
  while w > max_width:
    h, w = h // 2, w // 2
  return h, w


def resize_nearest(image: np.ndarray, shape: tuple[int, int]) -> np.ndarray:
  h, w = shape
  ys = (np.arange(h) + 0.5) / h * image.shape[0]
  xs = (np.arange(w) + 0.5) / w * image.shape[1]
  return image[ys.astype(int)][:, xs.astype(int)]


def sh9_irradiance(image: np.ndarray) -> np.ndarray:
  """SH9 Lambertian radiance of an equirect image in float64 (envmap.py:224-249)."""
  h, w, _ = image.shape
  theta = (np.arange(h) + 0.5) / h * np.pi
  phi = ((np.arange(w) + 0.5) / w - 0.5) * 2.0 * np.pi
  st, ct = np.sin(theta)[:, None], np.cos(theta)[:, None]
  x, y, z = st * np.cos(phi)[None], st * np.sin(phi)[None], np.broadcast_to(ct, (h, w))
  basis = np.stack(
    [np.full((h, w), 0.282095), 0.488603 * y, 0.488603 * z, 0.488603 * x, 1.092548 * x * y, 1.092548 * y * z,
     0.315392 * (3.0 * z * z - 1.0), 1.092548 * x * z, 0.546274 * (x * x - y * y)]
  )
  solid_angle = (2.0 * np.pi / w) * (np.pi / h) * np.broadcast_to(st, (h, w))
  coeffs = np.einsum("khw,hwc->kc", basis * solid_angle, image.astype(np.float64))
  band = np.array([np.pi, 2 * np.pi / 3, 2 * np.pi / 3, 2 * np.pi / 3] + [np.pi / 4] * 5)
  return (coeffs * band[:, None] / np.pi).astype(np.float32)


def sampling_tables(image: np.ndarray) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
  """Cell probabilities, marginal and conditional CDFs (envmap.py:409-432)."""
  small = downsample(np.asarray(image, dtype=np.float64)[..., :3], CDF_WIDTH)
  h = small.shape[0]
  lum = small @ np.array(LUMINANCE_WEIGHTS)
  sin_theta = np.sin((np.arange(h) + 0.5) / h * np.pi)[:, None]
  weight = lum * sin_theta + 1e-6 * max(float(lum.mean()), 1e-12)
  prob = weight / weight.sum()
  row = prob.sum(axis=1)
  marginal = np.concatenate([[0.0], np.cumsum(row)])
  conditional = np.concatenate([np.zeros((h, 1)), np.cumsum(prob, axis=1) / np.maximum(row[:, None], 1e-30)], axis=1)
  marginal[-1] = 1.0
  conditional[:, -1] = 1.0
  return prob.astype(np.float32), marginal.astype(np.float32), conditional.astype(np.float32)


@dataclasses.dataclass
class Environments:
  radiance: list[np.ndarray]  # (h, w, 4) float16 level 0 per map
  sh: np.ndarray  # (nenv, 9, 3)
  prob: np.ndarray
  marginal: np.ndarray
  conditional: np.ndarray
  prefilter_levels: int
  prefilter_height: int
  prefilter_width: int
  max_width: float

  @property
  def nenv(self) -> int:
    return len(self.radiance)


def build_environments(images: list[np.ndarray]) -> Environments:
  radiance, shs, widths, tables = [], [], [], []
  for im in images:
    small = downsample(np.asarray(im, dtype=np.float32)[..., :3], MAX_RADIANCE_WIDTH)
    h, w, _ = small.shape
    widths.append(w)
    radiance.append(np.concatenate([small, np.ones((h, w, 1), np.float32)], axis=-1).astype(np.float16))
    shs.append(sh9_irradiance(small))
  shape = None
  for im in images:
    if shape is not None and downsampled_shape(im.shape, CDF_WIDTH) != shape:
      im = resize_nearest(im, shape)
    table = sampling_tables(im)
    shape = shape or table[0].shape
    tables.append(table)
  pw = min(PREFILTER_WIDTH, min(widths))
  return Environments(
    radiance=radiance,
    sh=np.stack(shs).astype(np.float32),
    prob=np.stack([t[0] for t in tables]),
    marginal=np.stack([t[1] for t in tables]),
    conditional=np.stack([t[2] for t in tables]),
    prefilter_levels=PREFILTER_LEVELS,
    prefilter_height=max(pw // 2, 1),
    prefilter_width=pw,
    max_width=float(max(widths)),
  )


def environment_images(envmap: Any) -> list[np.ndarray]:
  """The scene's explicit environment images (arrays; the oracle's scenes pass no file paths)."""
  if envmap is None:
    return []
  items = envmap if isinstance(envmap, (list, tuple)) else [envmap]
  return [np.asarray(np.asarray(im)[..., :3], np.float32) for im in items]


# ------------------------------------------------------------------ the prepared scene


@dataclasses.dataclass
class Prepared:
  outputs: dict[str, Any]
  settings: dict[str, Any]
  tables: dict[str, np.ndarray]
  enabled_geom_ids: np.ndarray
  textures: list[tuple[int, np.ndarray]]
  environments: Environments | None
  mesh_nface: np.ndarray


def _per_camera(value: Any, n: int, default: bool) -> list[bool]:
  if value is None:
    return [default] * n
  if isinstance(value, (bool, np.bool_)):
    return [bool(value)] * n
  return [bool(v) for v in value]


def output_layout(mjm: Any, cam_res: Any, render_rgb: Any, render_depth: Any, render_seg: Any, cam_active: Any) -> dict[str, Any]:
  """Active cameras and the per-output pixel addresses of MuJoCo Warp's render context: each
  output packs the images of the cameras that render it one after another (address -1 for the
  others), the ray addresses cover every camera."""
  cams = []
  for i, v in enumerate(range(mjm.ncam) if cam_active is None else cam_active):
    if isinstance(v, (bool, np.bool_)):
      if v:
        cams.append(i)  # a flag per model camera
    else:
      cams.append(int(v))  # a camera index
  n = len(cams)
  if cam_res is None:
    res = [tuple(int(v) for v in np.asarray(mjm.cam_resolution)[c]) for c in cams]
  elif isinstance(cam_res, tuple) and len(cam_res) == 2 and all(isinstance(v, (int, np.integer)) for v in cam_res):
    res = [(int(cam_res[0]), int(cam_res[1]))] * n
  else:
    res = [(int(w), int(h)) for w, h in cam_res]
  flags = {"render_rgb": _per_camera(render_rgb, n, True), "render_depth": _per_camera(render_depth, n, True),
           "render_seg": _per_camera(render_seg, n, False)}
  npix = [w * h for w, h in res]
  out: dict[str, Any] = {"nrender": n, "cam_id_map": cams, "cam_res": res, **flags}
  out["ray_adr"] = [int(sum(npix[:c])) for c in range(n)]
  out["total_rays"] = int(sum(npix))
  for key, name in (("render_rgb", "rgb"), ("render_depth", "depth"), ("render_seg", "seg")):
    adr, total = [], 0
    for on, p in zip(flags[key], npix, strict=True):
      adr.append(total if on else -1)
      total += p if on else 0
    out[f"{name}_adr"] = adr
    out[f"{name}_stride"] = total
  return out


def prepare(mjm: Any, mjd: Any, nworld: int, options: dict[str, Any]) -> Prepared:
  """The oracle's scene inputs for create_render_context keyword arguments `options`."""
  o = dict(options)
  light_model = int(o.get("light_model", LIGHT_MODEL_PHYSICAL))
  physical = light_model == LIGHT_MODEL_PHYSICAL
  tier = int(o.get("tier", TIER_REALTIME))
  groups = np.asarray(mjm.geom_group).reshape(-1)
  rendered = np.isin(groups, list(o.get("enabled_geom_groups", (0, 1, 2))))
  outputs = output_layout(mjm, o.get("cam_res"), o.get("render_rgb"), o.get("render_depth"), o.get("render_seg"), o.get("cam_active"))

  ltype = np.asarray(mjm.light_type).reshape(-1)
  nlight = len(ltype)
  light_xpos0 = np.zeros((nlight, 3))
  if mjd is not None and nlight:
    lx = np.asarray(mjd.light_xpos)
    light_xpos0 = lx[0] if lx.ndim == 3 else lx
  exposure, intensity, ambient = resolve_lighting(mjm, light_xpos0, light_model, float(o.get("ev100", DEFAULT_EV100)))
  metallic, roughness, reflectance = resolve_materials(mjm, int(o.get("unset_material", UNSET_GLTF)), o.get("default_material"))
  matid = np.asarray(mjm.geom_matid).reshape(-1)
  rendered_mats = np.unique(matid[rendered & (matid >= 0)])
  use_textures = bool(o.get("use_textures", True))
  f = surface_features(mjm, use_textures, bool(o.get("specular_aa", True)) and tier == TIER_REALTIME, rendered_mats)
  used = np.zeros(mjm.ntex, bool)
  if f["textures"]:
    ids = np.asarray(mjm.mat_texid).reshape(-1, 10)[rendered_mats].ravel()
    used[ids[ids >= 0]] = True
  textures = texture_images(mjm, used) if mjm.ntex else []
  alpha = effective_geom_rgba(mjm)[rendered, 3]
  has_transparency = bool(np.any((alpha > 0.0) & (alpha < 1.0))) or f["alpha_map"]
  mat_reflectance = np.asarray(mjm.mat_reflectance, np.float32).reshape(-1)
  has_reflection = bool(o.get("enable_reflections", True)) and bool(len(rendered_mats) and np.any(mat_reflectance[rendered_mats] > 0.0))
  background = srgb_to_linear(tuple(o.get("background_color", (0.0, 0.0, 0.0, 1.0)))[:3]).astype(np.float32)

  images = environment_images(o.get("envmap"))
  env = build_environments(images) if images else None
  has_env = env is not None
  env_intensity = o.get("envmap_intensity")
  if env_intensity is None:
    env_intensity = 1.0 / exposure
  if has_env and physical:
    ambient[:] = 0.0
  texel_angle = 2.0 * math.pi / (env.max_width if has_env else 1.0)

  settings = {
    "tier": tier,
    "render_order": int(o.get("render_order", 1)),
    "samples_per_axis": int(o.get("samples_per_pixel", 1)),
    "tone_mapper": int(o.get("tone_mapper", 0)),
    "render_hdr": int(bool(o.get("render_hdr", False))),
    "render_guides": int(bool(o.get("render_guides", False))),
    "light_model": light_model,
    "use_shadows": int(bool(o.get("use_shadows", True))),
    "shadow_samples": int(o.get("shadow_samples", 1)),
    "headlight_active": int(bool(mjm.headlight_active)),
    "has_env": int(has_env),
    "env_background": int(has_env and bool(o.get("envmap_background", True))),
    **{k: int(f[k]) for k in ("textures", "base_color_map", "normal_map", "orm_map", "emissive_map", "opacity_map", "specular_aa")},
    "vertex_normals": int(bool(o.get("enable_vertex_normals", True))),
    "has_reflection": int(has_reflection),
    "has_transparency": int(has_transparency),
    "max_layers": int(o.get("max_layers", 4)),
    "cull_backfaces": int(bool(o.get("enable_backface_culling", True))),
    "path_samples": int(o.get("path_samples", 64)),
    "max_depth": int(o.get("max_depth", 4)),
    "rr_depth": int(o.get("rr_depth", 3)),
    "denoise": int(bool(o.get("denoise", False))),
    "znear": float(getattr(mjm, "znear", 0.01)),
    "zfar": float(getattr(mjm, "zfar", 0.0)),
    "shadow_light_fraction": float(o.get("shadow_light_fraction", 0.0)),
    "headlight_intensity": float(math.pi),
    "headlight_diffuse": tuple(float(c) for c in mjm.headlight_diffuse),
    "headlight_specular": tuple(float(c) for c in mjm.headlight_specular),
    "background": tuple(float(c) for c in background),
    "inv_texel_angle": 1.0 / texel_angle,
    **DENOISE_SIGMAS,
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
    "env_intensity": np.array([env_intensity], np.float32),
    "env_yaw": np.array([np.radians(float(o.get("envmap_rotation", 0.0)))], np.float32),
  }
  return Prepared(
    outputs=outputs,
    settings=settings,
    tables=tables,
    enabled_geom_ids=np.nonzero(rendered)[0].astype(np.int32),
    textures=textures,
    environments=env,
    mesh_nface=np.asarray(getattr(mjm, "mesh_facenum", []), np.int32).reshape(-1),
  )


# ------------------------------------------------------------------ packing


def mip_count(w: int, h: int) -> int:
  """Full mip chain length, at most the texture descriptor's MJPBR_MAX_MIPS levels."""
  return min(int(math.floor(math.log2(max(w, h)))) + 1, ss.MAX_MIPS)


def pack_textures(images: list[tuple[int, np.ndarray]], texture_type: Any) -> tuple[list[Any], np.ndarray]:
  """MjpbrTexture descriptions and one byte buffer with every level 0 in place (levels 16-byte
  aligned, row-major, mip sizes max(1, size >> level))."""
  desc, offset, chunks = [], 0, []
  for fmt, img in images:
    h, w = img.shape[:2]
    texel = 4 if fmt == TEX_RGBA8 else 8
    d = texture_type()
    d.format, d.width, d.height, d.nlevel = fmt, w, h, mip_count(w, h)
    for level in range(d.nlevel):
      d.level_offset[level] = offset
      if level == 0:
        chunks.append((offset, np.ascontiguousarray(img).view(np.uint8).reshape(-1)))
      offset += (max(w >> level, 1) * max(h >> level, 1) * texel + 15) // 16 * 16
    desc.append(d)
  data = np.zeros(max(offset, 16), np.uint8)
  for start, raw in chunks:
    data[start : start + raw.size] = raw
  return desc, data


def desc_bytes(desc: list[Any]) -> np.ndarray:
  return np.frombuffer(b"".join(bytes(d) for d in desc), dtype=np.uint8).copy() if desc else np.zeros(0, np.uint8)


def pack_camera_rays(camera_rays: Any, cam_res: list[tuple[int, int]]) -> tuple[np.ndarray, np.ndarray]:
  """(origin, direction) (total_rays, 3) float32: every rendering camera's (h, w, 2, 3) rays in
  camera order, pixels row-major."""
  images = list(camera_rays) if not (isinstance(camera_rays, np.ndarray) and camera_rays.ndim == 5) else list(camera_rays)
  origin, direction = [], []
  for im, (w, h) in zip(images, cam_res, strict=True):
    a = np.asarray(im.cpu() if hasattr(im, "cpu") else im, np.float32).reshape(h * w, 2, 3)
    origin.append(a[:, 0])
    direction.append(a[:, 1])
  return np.ascontiguousarray(np.concatenate(origin)), np.ascontiguousarray(np.concatenate(direction))
