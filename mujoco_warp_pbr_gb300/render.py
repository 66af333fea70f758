"""render / refit_bvh: the host side of one frame.

`render(m, d, rc, seed)` mirrors mujoco_warp_pbr.render (mujoco_warp_pbr/_src/render.py:431-460);
`refit_bvh(m, d, rc)` stands in for mujoco_warp.refit_bvh(m, d, rc.base), which reference users
call after physics moved the geometry. Each builds (or reuses) the MjpbrScene descriptor and makes
one libmjpbr call on the current torch stream, asynchronously: both can be captured into a CUDA
graph. The descriptor is rebuilt only when an array of m, d or rc was replaced (identity check,
like the reference's launch-input cache, mujoco_warp_pbr/_src/launch.py:89-115).
"""

from __future__ import annotations

import warnings
from typing import Any

import numpy as np
import torch

from mujoco_warp_pbr_gb300 import _lib
from mujoco_warp_pbr_gb300 import _scene
from mujoco_warp_pbr_gb300.pbr_types import PbrRenderContext

_MODEL_FIELDS = (
  "geom_type",
  "geom_dataid",
  "geom_matid",
  "geom_size",
  "geom_rgba",
  "mat_rgba",
  "mat_emission",
  "mat_texid",
  "mat_texrepeat",
  "mat_texuniform",
  "light_type",
  "light_castshadow",
  "light_active",
  "light_attenuation",
  "light_cutoff",
  "light_exponent",
  "light_diffuse",
  "light_specular",
  "cam_projection",
  "cam_fovy",
  "cam_sensorsize",
  "cam_intrinsic",
  "mesh_vertadr",
  "mesh_faceadr",
  "mesh_normaladr",
  "mesh_texcoordadr",
  "mesh_vert",
  "mesh_face",
  "mesh_normal",
  "mesh_facenormal",
  "mesh_texcoord",
  "mesh_facetexcoord",
)
_DATA_FIELDS = ("geom_xpos", "geom_xmat", "cam_xpos", "cam_xmat", "light_xpos", "light_xdir")
_CONTEXT_TABLES = (
  "geom_metallic",
  "geom_roughness",
  "geom_reflectance",
  "mat_reflectance",
  "light_intensity",
  "light_range",
  "light_bulbradius",
  "exposure",
  "ambient_radiance",
  "env_id",
  "env_intensity",
  "env_yaw",
)
_INT_FIELDS = {
  "geom_type",
  "geom_dataid",
  "geom_matid",
  "mat_texid",
  "mat_texuniform",
  "light_type",
  "light_castshadow",
  "light_active",
  "cam_projection",
  "mesh_vertadr",
  "mesh_faceadr",
  "mesh_normaladr",
  "mesh_texcoordadr",
  "mesh_face",
  "mesh_facenormal",
  "mesh_facetexcoord",
  "env_id",
}


def as_tensor(value: Any, name: str, device: torch.device) -> torch.Tensor:
  """A contiguous float32 / int32 tensor on `device` for a model, data or context array."""
  dtype = torch.int32 if name in _INT_FIELDS else torch.float32
  if isinstance(value, torch.Tensor):
    t = value
  elif hasattr(value, "__cuda_array_interface__"):
    t = torch.as_tensor(value, device=device)
  else:
    t = torch.as_tensor(np.asarray(value))
  if t.dtype == torch.bool:
    t = t.to(torch.int32)
  if t.dtype != dtype:
    t = t.to(dtype)
  if t.device != device:
    t = t.to(device)
  return t.contiguous()


def _batched(t: torch.Tensor, inner: int) -> torch.Tensor:
  """A batched table viewed as (nbatch, inner...) with nbatch its leading dimension."""
  if t.dim() == 0:
    return t.reshape(1)
  return t


def scene_fields(m: Any, d: Any, rc: PbrRenderContext) -> dict[str, Any]:
  """MjpbrScene fields (tensors and ints) of a frame; the tensors must stay alive."""
  dev = rc.device
  f: dict[str, Any] = {}
  for name in _MODEL_FIELDS:
    v = getattr(m, name, None)
    f[name] = None if v is None or (hasattr(v, "numel") and v.numel() == 0) else as_tensor(v, name, dev)
  for name in _DATA_FIELDS:
    v = getattr(d, name, None)
    f[name] = None if v is None or (hasattr(v, "numel") and v.numel() == 0) else as_tensor(v, name, dev)
  for name in _CONTEXT_TABLES:
    f[name] = as_tensor(getattr(rc, name), name, dev)
  # batched tables must carry their batch dimension first
  for name in ("exposure", "env_id", "env_intensity", "env_yaw"):
    f[name] = f[name].reshape(-1)
  f["ambient_radiance"] = f["ambient_radiance"].reshape(-1, 3)
  ngeom = int(f["geom_type"].shape[0])
  nworld = int(d.nworld)
  if nworld != rc.nworld:
    raise ValueError(f"data has {nworld} worlds, the render context {rc.nworld}")
  b = rc.base
  st = dict(rc._host_cache["settings"])
  st.update(
    {
      "render_order": int(rc.render_order),
      "schedule": int(rc.schedule),
      "queue_item": int(rc.queue_item),
      "samples_per_axis": int(rc.samples_per_pixel),
      "tone_mapper": int(rc.tone_mapper),
      "render_hdr": int(bool(rc.render_hdr)),
      "light_model": int(rc.light_model),
      "use_shadows": int(bool(rc.use_shadows)),
      "shadow_samples": int(rc.shadow_samples),
      "has_reflection": int(bool(rc.has_reflection)),
      "has_transparency": int(bool(rc.has_transparency)),
      "max_layers": int(rc.max_layers),
      "shadow_light_fraction": float(rc.shadow_light_fraction),
      "has_env": int(bool(rc.has_env)),
      "env_background": int(bool(rc.env_background)),
      "tier": int(rc.tier),
      "path_samples": int(rc.path_samples),
      "max_depth": int(rc.max_depth),
      "rr_depth": int(rc.rr_depth),
      "denoise": int(bool(rc.denoise)),
      "denoise_sigma_color": float(rc.denoise_sigma_color),
      "denoise_sigma_normal": float(rc.denoise_sigma_normal),
      "denoise_sigma_depth": float(rc.denoise_sigma_depth),
      "denoise_sigma_albedo": float(rc.denoise_sigma_albedo),
    }
  )
  env = rc.env
  f.update(
    {
      "nworld": nworld,
      "ngeom": ngeom,
      "nmat": int(f["mat_rgba"].shape[1]) if f["mat_rgba"] is not None else 0,
      "nlight": int(f["light_xpos"].shape[1]) if f["light_xpos"] is not None else 0,
      "ncam": int(f["cam_projection"].shape[0]),
      "nmesh": len(rc.mesh_nface),
      "nhfield": int(rc.nhfield),
      "ntex": len(rc.tex_desc),
      "nenv": env.nenv if env is not None else 0,
      "nrender": b.nrender,
      "total_rays": b.total_rays,
      "cam_id_map": b.cam_id_map,
      "cam_res": b.cam_res,
      "render_rgb": [int(v) for v in b.render_rgb],
      "render_depth": [int(v) for v in b.render_depth],
      "render_seg": [int(v) for v in b.render_seg],
      "ray_adr": b.ray_adr,
      "rgb_adr": b.rgb_adr,
      "depth_adr": b.depth_adr,
      "seg_adr": b.seg_adr,
      "rgb_stride": int(b.rgb_data.shape[1]),
      "depth_stride": int(b.depth_data.shape[1]),
      "seg_stride": int(b.seg_data.shape[1]),
      "rgb_data": b.rgb_data,
      "depth_data": b.depth_data,
      "seg_data": b.seg_data,
      "hdr_data": rc.hdr_data if (rc.render_hdr or rc.denoise) else None,
      "guide_albedo": rc.guide_albedo if rc.render_guides else None,
      "guide_normal": rc.guide_normal if rc.render_guides else None,
      "nbvh_geom": int(rc.enabled_geom_ids.shape[0]),
      "nnode": int(rc.tlas_child.shape[1]),
      "enabled_geom_ids": rc.enabled_geom_ids,
      "tlas_child": rc.tlas_child,
      "mesh_bounds": rc.mesh_bounds,
      "world_blocks": rc.world_blocks,
      "world_block_floats": rc.world_block_floats,
      "blas_nodes": rc.blas_nodes,
      "blas_tris": rc.blas_tris,
      "blas_root": rc.blas_root,
      "blas_tri_base": rc.blas_tri_base,
      "textures": rc.textures,
      "tex_data": rc.tex_data,
      "dfg_lut": rc.dfg_lut,
      "dfg_size": rc.dfg_size,
      "aov_guide": rc.aov_guide,
      "aov_emission": rc.aov_emission,
      "denoise_buffers": rc.denoise_buffers,
      "denoise_iterations": int(rc.denoise_iterations),
      "error_word": rc.error_word,
      "work_counter": rc.work_counter,
      "wave_scratch": rc.wave_scratch,
      "wave_scratch_bytes": int(rc.wave_scratch.numel()) if rc.wave_scratch is not None else 0,
      "settings": st,
    }
  )
  if env is not None:
    f.update(
      {
        "prefilter_levels": env.levels,
        "prefilter_height": env.height,
        "prefilter_width": env.width,
        "env_prefiltered": env.prefiltered,
        "env_radiance": env.radiance_desc,
        "env_data": env.radiance_data,
        "env_sh": env.sh,
        "cdf_height": int(env.prob.shape[1]),
        "cdf_width": int(env.prob.shape[2]),
        "env_prob": env.prob,
        "env_marginal": env.marginal,
        "env_conditional": env.conditional,
      }
    )
  if rc.ray_direction is not None:
    f["ray_origin"] = rc.ray_origin
    f["ray_direction"] = rc.ray_direction
    f["bundle_res"] = rc.ray_res
  return f


def _sources(m: Any, d: Any, rc: PbrRenderContext) -> tuple:
  public = [v for k, v in vars(rc).items() if not k.startswith("_")]
  return (*vars(m).values(), *vars(d).values(), *public, *vars(rc.base).values())


def scene(m: Any, d: Any, rc: PbrRenderContext) -> _lib.Scene:
  """The (cached) MjpbrScene of a frame."""
  sources = _sources(m, d, rc)
  ids = tuple(map(id, sources))
  cached = rc._host_cache.get("scene")
  if cached is not None and cached[1] == ids:
    return cached[2]
  _check_env_id(rc)
  _warn_ignored_overrides(m, rc)
  fields = scene_fields(m, d, rc)
  struct = _scene.fill_scene(fields)
  if _ensure_wave_scratch(rc, struct):
    sources = _sources(m, d, rc)
    ids = tuple(map(id, sources))
    fields = scene_fields(m, d, rc)
    struct = _scene.fill_scene(fields)
  # the cache holds the sources and the converted tensors so their addresses stay valid
  rc._host_cache["scene"] = (sources, ids, struct, fields)
  return struct


# camera samples (real-time tier) or paths (path tier) per chunk of the wavefront schedules when
# wave_chunk_worlds is 0: queues of about 21 GB (mesh / IBL scene, two lights) and 13 GB (path
# scene), a few per cent faster than chunks of a quarter of that (fewer launches and launch tails)
WAVE_CHUNK_SAMPLES = 1 << 26
# worlds one launch of the real-time kernels covers (CUDA's gridDim.y limit; more take more launches)
MAX_GRID_WORLDS = 65535
WAVE_CHUNK_PATHS = 1 << 25


def _ensure_wave_scratch(rc: PbrRenderContext, struct: _lib.Scene) -> bool:
  """Allocates (or grows) the wavefront schedule's scratch for a context using it: wave_chunk_worlds
  worlds per chunk, or about WAVE_CHUNK_SAMPLES camera samples (real-time tier) / WAVE_CHUNK_PATHS
  paths (path tier). Returns True when rc.wave_scratch changed."""
  if rc.schedule != 2 or (rc.tier == 0 and rc.has_transparency):
    return False
  lib = _lib.load()
  per_world = lib.mjpbr_wave_scratch_bytes(struct, 1) - lib.mjpbr_wave_scratch_bytes(struct, 0)
  pixels = sum(w * h for (w, h), on in zip(rc.base.cam_res, rc.base.render_rgb) if on)
  if rc.tier == 0:
    chunk_units, units = WAVE_CHUNK_SAMPLES, pixels * int(rc.samples_per_pixel) ** 2
  else:
    chunk_units, units = WAVE_CHUNK_PATHS, pixels * int(rc.path_samples)
  chunk = rc.wave_chunk_worlds or max(1, chunk_units // max(units, 1))
  chunk = min(chunk, int(rc.base.rgb_data.shape[0]))
  if rc.tier == 0:
    chunk = min(chunk, MAX_GRID_WORLDS)  # the real-time stages put a chunk's worlds in grid y
  need = int(lib.mjpbr_wave_scratch_bytes(struct, chunk))
  if need < 0 or per_world < 0:
    raise ValueError("the wavefront schedule cannot render this scene")
  if rc.wave_scratch is not None and rc.wave_scratch.numel() >= need:
    return False
  rc.wave_scratch = torch.empty(need, dtype=torch.uint8, device=rc.device)
  return True


def _warn_ignored_overrides(m: Any, rc: PbrRenderContext) -> None:
  """UserWarning when a replaced array needs a flag that is off: translucent m.geom_rgba without
  rc.has_transparency, positive rc.mat_reflectance without rc.has_reflection (both flags are
  derived from the model at creation; mujoco_warp_pbr/_src/launch.py:59-86). Each array is
  checked once, when it first appears; the arrays of the first render are not checked; nothing
  is checked while a graph is being captured."""
  if torch.cuda.is_available() and torch.cuda.is_current_stream_capturing():
    return
  checks = (
    ("geom_rgba", getattr(m, "geom_rgba", None), rc.has_transparency, "has_transparency",
     lambda a: bool(np.any((a[..., 3] > 0.0) & (a[..., 3] < 1.0)))),
    ("mat_reflectance", rc.mat_reflectance, rc.has_reflection, "has_reflection", lambda a: bool(np.any(a > 0.0))),
  )
  for name, array, enabled, flag, needs in checks:
    key = "seen_" + name
    seen = rc._host_cache.get(key)
    rc._host_cache[key] = array
    if array is None or seen is None or seen is array or enabled:
      continue
    if isinstance(array, torch.Tensor):
      values = array.detach().cpu().numpy()
    elif hasattr(array, "__cuda_array_interface__"):
      values = torch.as_tensor(array, device=rc.device).cpu().numpy()
    else:
      values = np.asarray(array)
    if values.size and needs(values):
      warnings.warn(f"the replaced {name} is ignored by the renderer: set rc.{flag} = True to render it", stacklevel=4)


def _check_env_id(rc: PbrRenderContext) -> None:
  """ValueError if a replaced env_id selects a missing map (checked once per array, not while
  capturing a graph; mujoco_warp_pbr/_src/kernel_inputs.py:480-490)."""
  env_id = rc.env_id
  if rc._host_cache.get("env_id") is env_id or torch.cuda.is_current_stream_capturing():
    return
  nenv = rc.env.nenv if rc.env is not None else 1
  ids = env_id.detach().cpu().numpy()
  if ids.size and (ids.min() < 0 or ids.max() >= nenv):
    raise ValueError(f"env_id must be in [0, {nenv}) (one per environment map), got values in [{ids.min()}, {ids.max()}]")
  rc._host_cache["env_id"] = env_id


def _stream(rc: PbrRenderContext) -> int:
  return torch.cuda.current_stream(rc.device).cuda_stream


def refit_bvh(m: Any, d: Any, rc: PbrRenderContext) -> None:
  """Refits every world's scene BVH to the current geom poses and packs the per-world blocks the
  render kernels read (one kernel). Call after the geometry, cameras or lights moved."""
  _lib.call("mjpbr_refit_bvh", scene(m, d, rc), _stream(rc))
  rc._host_cache["refit"] = True


def render(m: Any, d: Any, rc: PbrRenderContext, seed: int = 0, denoise: bool = True) -> None:
  """Renders the current frame into the context's output buffers (one kernel for the real-time
  tier, one persistent kernel for the path-traced tier). The image is a deterministic function of
  the seed. The per-world blocks come from the last refit_bvh; the first render of a context
  refits once itself. A path-traced context created with denoise=True then runs the a-trous
  filter (the reference's _src/render.py:431-460 dispatch and _src/pathtrace.py:426-438);
  denoise=False leaves the noisy image and the filter's inputs for a
  later denoise() call."""
  s = scene(m, d, rc)
  stream = _stream(rc)
  if not rc._host_cache.get("refit"):
    _lib.call("mjpbr_refit_bvh", s, stream)
    rc._host_cache["refit"] = True
  _lib.call("mjpbr_render", s, int(seed) & 0xFFFFFFFF, stream)
  if rc.tier == 1 and rc.denoise and denoise:
    _lib.call("mjpbr_denoise_atrous", s, stream)


def denoise(m: Any, d: Any, rc: PbrRenderContext) -> None:
  """Filters the path tracer's demodulated image into the RGB (and HDR) outputs
  (denoise.py:214-248): denoise_iterations a-trous passes, the last one remodulating, tone
  mapping and encoding."""
  if not (rc.tier == 1 and rc.denoise):
    raise ValueError("denoise applies to a path-traced context created with denoise=True")
  _lib.call("mjpbr_denoise_atrous", scene(m, d, rc), _stream(rc))


def check_errors(rc: PbrRenderContext) -> int:
  """Synchronises and returns (then clears) the error bits kernels reported (0: none).

  Bit 1: a traversal stack overflowed. Bit 2: the work queue was inconsistent. Bit 4: a bounded
  wait gave up. Bit 8: the Newton adapter's pose step met a shape or body index out of range."""
  value = int(rc.error_word.item())
  rc.error_word.zero_()
  return value
