"""GB300-native (sm_103a) batched physically based render path for MuJoCo worlds.

A drop-in for mujoco_warp_pbr's render surface: create_render_context / render / refit_bvh /
get_rgb / get_depth / get_segmentation (+ get_hdr / get_albedo / get_normal / load_hdr). The
compute runs in hand-written CUDA kernels of libmjpbr.so behind a C ABI (include/mjpbr.h); this
package is the host side. There is no CPU fallback: without the built library, rendering raises.
"""

from mujoco_warp_pbr_gb300.autotune import autotune as autotune
from mujoco_warp_pbr_gb300.autotune import capture_frame as capture_frame
from mujoco_warp_pbr_gb300.envmap import load_hdr as load_hdr
from mujoco_warp_pbr_gb300.context import create_render_context as create_render_context
from mujoco_warp_pbr_gb300.context import resolve_geom_materials as resolve_geom_materials
from mujoco_warp_pbr_gb300.model import Data as Data
from mujoco_warp_pbr_gb300.model import HostData as HostData
from mujoco_warp_pbr_gb300.model import HostModel as HostModel
from mujoco_warp_pbr_gb300.model import Model as Model
from mujoco_warp_pbr_gb300.model import put_data as put_data
from mujoco_warp_pbr_gb300.model import put_model as put_model
from mujoco_warp_pbr_gb300.output import get_albedo as get_albedo
from mujoco_warp_pbr_gb300.output import get_depth as get_depth
from mujoco_warp_pbr_gb300.output import get_hdr as get_hdr
from mujoco_warp_pbr_gb300.output import get_normal as get_normal
from mujoco_warp_pbr_gb300.output import get_rgb as get_rgb
from mujoco_warp_pbr_gb300.output import get_segmentation as get_segmentation
from mujoco_warp_pbr_gb300.rays import CameraRays as CameraRays
from mujoco_warp_pbr_gb300.rays import set_camera_rays as set_camera_rays
from mujoco_warp_pbr_gb300.render import check_errors as check_errors
from mujoco_warp_pbr_gb300.render import denoise as denoise
from mujoco_warp_pbr_gb300.render import refit_bvh as refit_bvh
from mujoco_warp_pbr_gb300.render import render as render
from mujoco_warp_pbr_gb300.render import scene as scene_descriptor
from mujoco_warp_pbr_gb300.pbr_types import LightModel as LightModel
from mujoco_warp_pbr_gb300.pbr_types import PbrRenderContext as PbrRenderContext
from mujoco_warp_pbr_gb300.pbr_types import RenderOrder as RenderOrder
from mujoco_warp_pbr_gb300.pbr_types import Tier as Tier
from mujoco_warp_pbr_gb300.pbr_types import ToneMapper as ToneMapper
from mujoco_warp_pbr_gb300.pbr_types import UnsetMaterial as UnsetMaterial

__all__ = [
  "CameraRays",
  "Data",
  "HostData",
  "HostModel",
  "LightModel",
  "Model",
  "PbrRenderContext",
  "RenderOrder",
  "Tier",
  "ToneMapper",
  "UnsetMaterial",
  "autotune",
  "capture_frame",
  "check_errors",
  "create_render_context",
  "denoise",
  "get_albedo",
  "get_depth",
  "get_hdr",
  "get_normal",
  "get_rgb",
  "get_segmentation",
  "load_hdr",
  "put_data",
  "put_model",
  "refit_bvh",
  "render",
  "resolve_geom_materials",
  "scene_descriptor",
  "set_camera_rays",
]
