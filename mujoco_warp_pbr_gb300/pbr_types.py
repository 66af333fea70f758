"""Enums and the render context of the GB300 render path.

The enums and the PbrRenderContext fields mirror mujoco_warp_pbr/_src/types.py:29-322 (same
names, values and batching convention: a table whose first dimension is a batch dimension is
indexed with worldid % shape[0]; replace it with a tensor of leading size nworld to vary it per
world). Arrays are torch CUDA tensors.
"""

from __future__ import annotations

import dataclasses
import enum
from typing import Any

import torch


class LightModel(enum.IntEnum):
  """How MuJoCo light parameters are interpreted (PHYSICAL: lux / candela with EV100 exposure;
  MUJOCO: MuJoCo's OpenGL attenuation and colours, exposure 1)."""

  PHYSICAL = 0
  MUJOCO = 1


class Tier(enum.IntEnum):
  """REALTIME: primary ray, shadows, split-sum IBL, mirror, layers. PATH: path tracing."""

  REALTIME = 0
  PATH = 1


class ToneMapper(enum.IntEnum):
  PBR_NEUTRAL = 0
  ACES = 1
  CLAMP = 2


class RenderOrder(enum.IntEnum):
  """Assignment of pixels to threads; images are identical for every order.

  ROW: a warp covers 32 pixels of one row. TILED: a warp covers an 8 x 4 pixel block of a
  16 x 16 CTA tile. WORLD: accepted for compatibility, rendered as TILED.
  """

  ROW = 0
  TILED = 1
  WORLD = 2


class UnsetMaterial(enum.IntEnum):
  """Resolution of material fields MuJoCo leaves unset (-1): GLTF or colour HEURISTIC."""

  GLTF = 0
  HEURISTIC = 1


@dataclasses.dataclass
class Outputs:
  """Output buffers and their layout (MuJoCo Warp's RenderContext fields).

  Attributes:
    nrender: rendering cameras.
    cam_id_map: model camera of each rendering camera.
    cam_res: (width, height) per rendering camera.
    render_rgb, render_depth, render_seg: per rendering camera.
    ray_adr: first pixel of each camera among total_rays.
    rgb_adr, depth_adr, seg_adr: first pixel of each camera in the buffers (-1: not rendered).
    total_rays: pixels per world over all rendering cameras.
    rgb_data: (nworld, npix_rgb) packed RGBA8 (int32 storage, R in the low byte).
    depth_data: (nworld, npix_depth) float32 planar depth.
    seg_data: (nworld, npix_seg, 2) int32 (geom id, mjOBJ_GEOM) or (-1, -1).
  """

  nrender: int
  cam_id_map: list[int]
  cam_res: list[tuple[int, int]]
  render_rgb: list[bool]
  render_depth: list[bool]
  render_seg: list[bool]
  ray_adr: list[int]
  rgb_adr: list[int]
  depth_adr: list[int]
  seg_adr: list[int]
  total_rays: int
  rgb_data: torch.Tensor
  depth_data: torch.Tensor
  seg_data: torch.Tensor
  znear: float = 0.01
  zfar: float = 0.0


@dataclasses.dataclass
class PbrRenderContext:
  """Context for physically based rendering of nworld worlds (see the module docstring).

  Per-world tables (leading dimension 1 until replaced by one of size nworld):
    geom_metallic, geom_roughness, geom_reflectance (*, ngeom); mat_reflectance (*, nmat);
    light_intensity, light_range, light_bulbradius (*, nlight); exposure (*,);
    ambient_radiance (*, 3); env_id (*,) int32; env_intensity (*,); env_yaw (*,) radians.
  Flags derived at creation (set them when a replaced array introduces the feature):
    has_transparency, has_reflection.
  """

  nworld: int
  base: Outputs
  light_model: int
  tone_mapper: int
  use_shadows: bool
  shadow_light_fraction: float
  geom_metallic: torch.Tensor
  geom_roughness: torch.Tensor
  geom_reflectance: torch.Tensor
  mat_reflectance: torch.Tensor
  light_intensity: torch.Tensor
  light_range: torch.Tensor
  light_bulbradius: torch.Tensor
  headlight_active: bool
  headlight_diffuse: tuple[float, float, float]
  headlight_specular: tuple[float, float, float]
  headlight_intensity: float
  exposure: torch.Tensor
  ambient_radiance: torch.Tensor
  background_linear: tuple[float, float, float]
  has_env: bool
  env_background: bool
  env_id: torch.Tensor
  env_intensity: torch.Tensor
  env_yaw: torch.Tensor
  env_texel_angle: float
  samples_per_pixel: int
  shadow_samples: int
  has_transparency: bool
  max_layers: int
  has_reflection: bool
  render_order: int
  tier: int
  path_samples: int
  max_depth: int
  rr_depth: int
  denoise: bool
  denoise_iterations: int
  render_hdr: bool
  hdr_data: torch.Tensor
  render_guides: bool
  guide_albedo: torch.Tensor
  guide_normal: torch.Tensor
  cull_backfaces: bool
  vertex_normals: bool
  specular_aa: bool
  features: Any
  # scene BVH and acceleration structures
  enabled_geom_ids: torch.Tensor
  tlas_child: torch.Tensor
  world_blocks: torch.Tensor
  world_block_floats: int
  mesh_bounds: torch.Tensor | None
  blas_nodes: torch.Tensor | None
  blas_tris: torch.Tensor | None
  blas_root: torch.Tensor | None
  blas_tri_base: torch.Tensor | None
  mesh_nface: list[int]
  # textures, tables and environment maps
  textures: torch.Tensor | None
  tex_data: torch.Tensor | None
  tex_desc: list[Any]
  dfg_lut: torch.Tensor
  dfg_size: int
  env: Any
  # path tier
  aov_guide: torch.Tensor
  aov_emission: torch.Tensor
  denoise_buffers: tuple[torch.Tensor, torch.Tensor]
  error_word: torch.Tensor
  work_counter: torch.Tensor
  device: torch.device
  denoise_sigma_color: float = 4.0
  denoise_sigma_normal: float = 128.0
  denoise_sigma_depth: float = 0.02
  denoise_sigma_albedo: float = 0.05
  ray_origin: torch.Tensor | None = None
  ray_direction: torch.Tensor | None = None
  ray_res: list[tuple[int, int]] | None = None
  # real-time tier schedule (MJPBR_SCHEDULE_GRID 0 / QUEUE 1 / WAVEFRONT 2), the queue's work item
  # size in pixels and the wavefront's worlds per chunk (0: automatic); set by
  # create_render_context or mujoco_warp_pbr_gb300.autotune
  schedule: int = 0
  queue_item: int = 64
  wave_chunk_worlds: int = 0
  # the wavefront schedule's ray queues and records (uint8, allocated at the first render that
  # needs them, sized by mjpbr_wave_scratch_bytes)
  wave_scratch: torch.Tensor | None = None
  # accepted for compatibility with the reference's signature; the GB300 kernels choose their own
  block_dim: int | None = None
  max_registers: int | None = None
  ordered_traversal: bool | None = None
  traversal: str = "software"
  nhfield: int = 0  # height-field BVHs after the meshes' in blas_root / blas_tri_base / mesh_bounds
  _host_cache: dict[str, Any] = dataclasses.field(default_factory=dict)
