"""ctypes binding of libmjpbr.so (include/mjpbr.h).

The structures below mirror the C declarations field by field; `check_layout()` compares their
sizes and offsets with the library's own `mjpbr_struct_layout`. Loading fails loudly when the
library is missing: there is no fallback path.
"""

from __future__ import annotations

import ctypes
import threading
from pathlib import Path

LIBRARY = Path(__file__).resolve().parent / "libmjpbr.so"
ABI_VERSION = 3
MAX_RENDER = 16
NTEXROLE = 10
MAX_MIPS = 15

OK = 0
ERR_ARG = 1
ERR_CUDA = 2
ERR_DEVICE = 3
ERR_UNSUPPORTED = 4

c_i32 = ctypes.c_int32
c_f32 = ctypes.c_float
c_vp = ctypes.c_void_p


class F32B(ctypes.Structure):
  """mjpbr_f32b: batched float table (pointer, leading batch size)."""

  _fields_ = [("ptr", c_vp), ("nbatch", c_i32), ("pad_", c_i32)]


class I32B(ctypes.Structure):
  """mjpbr_i32b: batched int32 table."""

  _fields_ = [("ptr", c_vp), ("nbatch", c_i32), ("pad_", c_i32)]


KPCN_LAYERS = 15


class KpcnWeights(ctypes.Structure):
  """MjpbrKpcnWeights."""

  _fields_ = [("weight", c_vp * KPCN_LAYERS), ("bias", c_vp * KPCN_LAYERS)]


class Texture(ctypes.Structure):
  """MjpbrTexture."""

  _fields_ = [
    ("format", c_i32),
    ("width", c_i32),
    ("height", c_i32),
    ("nlevel", c_i32),
    ("level_offset", ctypes.c_int64 * MAX_MIPS),
    ("pad_", c_i32 * 2),
  ]


class Settings(ctypes.Structure):
  """MjpbrSettings."""

  _fields_ = [
    (name, c_i32)
    for name in (
      "tier",
      "render_order",
      "samples_per_axis",
      "tone_mapper",
      "render_hdr",
      "render_guides",
      "light_model",
      "use_shadows",
      "shadow_samples",
      "headlight_active",
      "has_env",
      "env_background",
      "textures",
      "base_color_map",
      "normal_map",
      "orm_map",
      "emissive_map",
      "opacity_map",
      "specular_aa",
      "vertex_normals",
      "has_reflection",
      "has_transparency",
      "max_layers",
      "cull_backfaces",
      "path_samples",
      "max_depth",
      "rr_depth",
      "denoise",
      "schedule",
      "queue_item",
      "stack_depth",
    )
  ] + [
    ("znear", c_f32),
    ("zfar", c_f32),
    ("shadow_light_fraction", c_f32),
    ("headlight_intensity", c_f32),
    ("headlight_diffuse", c_f32 * 3),
    ("headlight_specular", c_f32 * 3),
    ("background", c_f32 * 3),
    ("inv_texel_angle", c_f32),
    ("denoise_sigma_color", c_f32),
    ("denoise_sigma_normal", c_f32),
    ("denoise_sigma_depth", c_f32),
    ("denoise_sigma_albedo", c_f32),
  ]


_CAM = c_i32 * MAX_RENDER
_CAM2 = (c_i32 * 2) * MAX_RENDER


class Scene(ctypes.Structure):
  """MjpbrScene: everything one render reads and writes (device pointers)."""

  _fields_ = [
    ("abi_version", c_i32),
    ("nworld", c_i32),
    ("ngeom", c_i32),
    ("nmat", c_i32),
    ("nlight", c_i32),
    ("ncam", c_i32),
    ("nmesh", c_i32),
    ("ntex", c_i32),
    ("nenv", c_i32),
    # model
    ("geom_type", c_vp),
    ("geom_dataid", I32B),
    ("geom_matid", I32B),
    ("geom_size", F32B),
    ("geom_rgba", F32B),
    ("mat_rgba", F32B),
    ("mat_emission", F32B),
    ("mat_texid", I32B),
    ("mat_texrepeat", F32B),
    ("mat_texuniform", I32B),
    ("light_type", I32B),
    ("light_castshadow", I32B),
    ("light_active", I32B),
    ("light_attenuation", F32B),
    ("light_cutoff", F32B),
    ("light_exponent", F32B),
    ("light_diffuse", F32B),
    ("light_specular", F32B),
    ("cam_projection", c_vp),
    ("cam_fovy", F32B),
    ("cam_sensorsize", c_vp),
    ("cam_intrinsic", F32B),
    ("mesh_vertadr", c_vp),
    ("mesh_faceadr", c_vp),
    ("mesh_normaladr", c_vp),
    ("mesh_texcoordadr", c_vp),
    ("mesh_vert", c_vp),
    ("mesh_face", c_vp),
    ("mesh_normal", c_vp),
    ("mesh_facenormal", c_vp),
    ("mesh_texcoord", c_vp),
    ("mesh_facetexcoord", c_vp),
    # data
    ("geom_xpos", c_vp),
    ("geom_xmat", c_vp),
    ("cam_xpos", c_vp),
    ("cam_xmat", c_vp),
    ("light_xpos", c_vp),
    ("light_xdir", c_vp),
    # cameras and outputs
    ("nrender", c_i32),
    ("total_rays", c_i32),
    ("cam_id_map", _CAM),
    ("cam_res", _CAM2),
    ("render_rgb", _CAM),
    ("render_depth", _CAM),
    ("render_seg", _CAM),
    ("ray_adr", _CAM),
    ("rgb_adr", _CAM),
    ("depth_adr", _CAM),
    ("seg_adr", _CAM),
    ("rgb_stride", c_i32),
    ("depth_stride", c_i32),
    ("seg_stride", c_i32),
    ("pad0_", c_i32),
    ("rgb_data", c_vp),
    ("depth_data", c_vp),
    ("seg_data", c_vp),
    ("hdr_data", c_vp),
    ("guide_albedo", c_vp),
    ("guide_normal", c_vp),
    # per-world tables
    ("geom_metallic", F32B),
    ("geom_roughness", F32B),
    ("geom_reflectance", F32B),
    ("mat_reflectance", F32B),
    ("light_intensity", F32B),
    ("light_range", F32B),
    ("light_bulbradius", F32B),
    ("exposure", F32B),
    ("ambient_radiance", F32B),
    ("env_id", I32B),
    ("env_intensity", F32B),
    ("env_yaw", F32B),
    # scene BVH
    ("nbvh_geom", c_i32),
    ("nnode", c_i32),
    ("enabled_geom_ids", c_vp),
    ("tlas_child", I32B),
    ("mesh_bounds", c_vp),
    ("world_blocks", c_vp),
    ("world_block_floats", c_i32),
    ("nhfield", c_i32),
    # mesh BVHs
    ("blas_nodes", c_vp),
    ("blas_tris", c_vp),
    ("blas_root", c_vp),
    ("blas_tri_base", c_vp),
    # textures
    ("textures", c_vp),
    ("tex_data", c_vp),
    # environment
    ("dfg_lut", c_vp),
    ("dfg_size", c_i32),
    ("prefilter_levels", c_i32),
    ("prefilter_width", c_i32),
    ("prefilter_height", c_i32),
    ("env_prefiltered", c_vp),
    ("env_radiance", c_vp),
    ("env_data", c_vp),
    ("env_sh", c_vp),
    ("cdf_width", c_i32),
    ("cdf_height", c_i32),
    ("env_prob", c_vp),
    ("env_marginal", c_vp),
    ("env_conditional", c_vp),
    # camera rays
    ("ray_origin", c_vp),
    ("ray_direction", c_vp),
    ("bundle_res", _CAM2),
    # path-tier features
    ("aov_guide", c_vp),
    ("aov_emission", c_vp),
    ("denoise_buffers", c_vp * 2),
    ("denoise_iterations", c_i32),
    ("pad2_", c_i32),
    # status
    ("error_word", c_vp),
    ("work_counter", c_vp),
    ("wave_scratch", c_vp),
    ("wave_scratch_bytes", ctypes.c_int64),
    ("settings", Settings),
  ]


class Conv(ctypes.Structure):
  """MjpbrConv: one 3x3 convolution layer of the learned denoiser."""

  _fields_ = [
    ("in_", c_vp),
    ("in2", c_vp),
    ("weight", c_vp),
    ("bias", c_vp),
    ("out", c_vp),
    ("out_f32", c_vp),
    ("mask", c_vp),
    ("error_word", c_vp),
    ("nimg", c_i32),
    ("height", c_i32),
    ("width", c_i32),
    ("c_in", c_i32),
    ("c_in2", c_i32),
    ("c_out", c_i32),
    ("relu", c_i32),
    ("in2_full", c_i32),
  ]


class ConvGrad(ctypes.Structure):
  """MjpbrConvGrad: weight / bias gradients of a 3x3 convolution layer."""

  _fields_ = [
    ("in_", c_vp),
    ("in2", c_vp),
    ("grad_out", c_vp),
    ("grad_weight", c_vp),
    ("grad_bias", c_vp),
    ("error_word", c_vp),
    ("nimg", c_i32),
    ("height", c_i32),
    ("width", c_i32),
    ("c_in", c_i32),
    ("c_in2", c_i32),
    ("c_out", c_i32),
    ("tiles_per_cta", c_i32),
    ("in2_full", c_i32),
  ]


# name -> (restype, argtypes)
_SIGNATURES = {
  "mjpbr_abi_version": (ctypes.c_int, []),
  "mjpbr_last_error": (ctypes.c_char_p, []),
  "mjpbr_struct_layout": (None, [ctypes.POINTER(ctypes.c_int64)]),
  "mjpbr_world_block_floats": (c_i32, [c_i32, c_i32, c_i32, c_i32]),
  "mjpbr_wave_scratch_bytes": (ctypes.c_int64, [ctypes.POINTER(Scene), c_i32]),
  "mjpbr_env_sh9": (ctypes.c_int, [c_vp, c_i32, c_i32, c_vp, c_vp, c_vp]),
  "mjpbr_env_sampling_tables": (ctypes.c_int, [c_vp, c_i32, c_i32, c_vp, c_vp, c_vp, c_vp]),
  "mjpbr_wait_probe": (ctypes.c_int, [ctypes.c_uint32, c_vp, c_vp, c_vp]),
  "mjpbr_wave_profile_begin": (ctypes.c_int, []),
  "mjpbr_wave_profile_end": (ctypes.c_int, [ctypes.POINTER(ctypes.c_double), ctypes.POINTER(c_i32)]),
  "mjpbr_refit_bvh": (ctypes.c_int, [ctypes.POINTER(Scene), c_vp]),
  "mjpbr_render": (ctypes.c_int, [ctypes.POINTER(Scene), ctypes.c_uint32, c_vp]),
  "mjpbr_refit_render_static": (ctypes.c_int, [ctypes.POINTER(Scene), ctypes.c_uint32, c_vp]),
  "mjpbr_gemm_bf16": (ctypes.c_int, [c_vp, c_vp, c_vp, c_i32, c_i32, c_i32, c_vp, c_vp]),
  "mjpbr_conv3x3_bf16": (ctypes.c_int, [ctypes.POINTER(Conv), c_vp]),
  "mjpbr_conv3x3_wgrad_bf16": (ctypes.c_int, [ctypes.POINTER(ConvGrad), c_vp]),
  "mjpbr_kpcn_features": (ctypes.c_int, [ctypes.POINTER(Scene), c_i32, c_i32, c_i32, c_vp, c_vp]),
  "mjpbr_kpcn_target": (ctypes.c_int, [ctypes.POINTER(Scene), c_i32, c_vp, ctypes.c_double, c_vp, c_vp]),
  "mjpbr_accumulate_f64": (ctypes.c_int, [c_vp, c_vp, ctypes.c_int64, c_vp]),
  "mjpbr_avgpool2_bf16": (ctypes.c_int, [c_vp, c_vp, c_i32, c_i32, c_i32, c_i32, c_vp]),
  "mjpbr_upsample2_bf16": (ctypes.c_int, [c_vp, c_vp, c_i32, c_i32, c_i32, c_i32, c_vp]),
  "mjpbr_kpcn_apply": (ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, c_i32, c_i32, c_i32, c_vp]),
  "mjpbr_kpcn_loss": (ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, ctypes.c_int64, ctypes.c_float, ctypes.c_float, c_vp]),
  "mjpbr_kpcn_remod": (ctypes.c_int, [ctypes.POINTER(Scene), c_i32, c_vp, c_vp, c_vp]),
  "mjpbr_kpcn_apply_grad": (ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, c_i32, c_i32, c_i32, c_vp]),
  "mjpbr_split_concat_grad": (ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, c_i32, c_i32, c_i32, c_i32, c_i32, c_vp]),
  "mjpbr_unpool_add_grad": (ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, c_i32, c_i32, c_i32, c_i32, c_vp]),
  "mjpbr_adam": (
    ctypes.c_int,
    [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, ctypes.c_int64, c_i32, c_i32, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, c_i32, c_vp],
  ),
  "mjpbr_get_rgb": (ctypes.c_int, [ctypes.POINTER(Scene), c_i32, c_vp, c_i32, c_vp]),
  "mjpbr_get_depth": (ctypes.c_int, [ctypes.POINTER(Scene), c_i32, c_f32, c_vp, c_i32, c_vp]),
  "mjpbr_get_segmentation": (ctypes.c_int, [ctypes.POINTER(Scene), c_i32, c_vp, c_i32, c_vp]),
  "mjpbr_get_image": (ctypes.c_int, [ctypes.POINTER(Scene), c_i32, c_i32, c_vp, c_i32, c_vp]),
  "mjpbr_newton_sync_poses": (
    ctypes.c_int,
    [c_vp, c_i32, c_vp, c_vp, c_i32, c_vp, c_i32, c_vp, c_vp, c_i32, c_i32, c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp],
  ),
  "mjpbr_newton_images": (ctypes.c_int, [ctypes.POINTER(Scene), c_i32, c_vp, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp]),
  "mjpbr_mesh_bvh_device_scratch_bytes": (ctypes.c_int64, [c_i32, c_i32]),
  "mjpbr_build_mesh_bvh_device": (
    ctypes.c_int,
    [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_i32, c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, ctypes.c_int64, c_vp, c_vp],
  ),
  "mjpbr_dfg_lut": (ctypes.c_int, [c_vp, c_i32, c_i32, c_vp]),
  "mjpbr_build_mips": (ctypes.c_int, [ctypes.POINTER(Texture), c_vp, c_vp]),
  "mjpbr_kpcn_workspace_bytes": (ctypes.c_int64, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
  "mjpbr_denoise_learned": (ctypes.c_int, [ctypes.POINTER(Scene), ctypes.POINTER(KpcnWeights), c_vp, ctypes.c_int64, ctypes.c_int32, c_vp]),
  "mjpbr_prefilter_env": (ctypes.c_int, [ctypes.POINTER(Texture), c_vp, c_i32, c_i32, c_i32, c_i32, c_vp, c_vp]),
  "mjpbr_denoise_atrous": (ctypes.c_int, [ctypes.POINTER(Scene), c_vp]),
  "mjpbr_bvh_node_count": (c_i32, [c_i32]),
  "mjpbr_build_scene_bvh": (ctypes.c_int, [c_vp, c_vp, c_i32, c_vp]),
  "mjpbr_build_mesh_bvh": (ctypes.c_int, [c_vp, c_i32, c_vp, c_i32, c_i32, c_vp, c_vp, c_vp, ctypes.POINTER(c_i32)]),
}

_lock = threading.Lock()
_lib: ctypes.CDLL | None = None


class MjpbrError(RuntimeError):
  """A libmjpbr entry point returned an error status."""


def load() -> ctypes.CDLL:
  """The loaded library (built with mujoco_warp_pbr_gb300.build.build(); no fallback)."""
  global _lib
  with _lock:
    if _lib is None:
      if not LIBRARY.exists():
        raise RuntimeError(
          f"{LIBRARY} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
          "(the render path has no CPU fallback)"
        )
      lib = ctypes.CDLL(str(LIBRARY))
      for name, (restype, argtypes) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = restype
        fn.argtypes = argtypes
      if lib.mjpbr_abi_version() != ABI_VERSION:
        raise RuntimeError(f"libmjpbr ABI {lib.mjpbr_abi_version()} does not match the bindings ({ABI_VERSION})")
      _lib = lib
      check_layout()
  return _lib


_count_lib: ctypes.CDLL | None = None


def load_counting() -> ctypes.CDLL:
  """The counting build (libmjpbr_count.so): the same entry points with the real-time render
  kernels counting their ray queries, box / triangle / primitive tests and shading work into the
  device array given to mjpbr_count_set. Benchmark instrumentation, not the render path."""
  global _count_lib
  with _lock:
    if _count_lib is None:
      path = LIBRARY.with_name("libmjpbr_count.so")
      if not path.exists():
        raise RuntimeError(f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
      lib = ctypes.CDLL(str(path))
      for name, (restype, argtypes) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = restype
        fn.argtypes = argtypes
      lib.mjpbr_count_set.restype = ctypes.c_int
      lib.mjpbr_count_set.argtypes = [c_vp]
      _count_lib = lib
  return _count_lib


def exported_symbols() -> list[str]:
  return list(_SIGNATURES)


def python_layout() -> list[int]:
  return [
    ctypes.sizeof(Scene),
    ctypes.sizeof(Settings),
    ctypes.sizeof(Texture),
    Scene.nrender.offset,
    Scene.world_blocks.offset,
    Scene.env_prefiltered.offset,
    Scene.error_word.offset,
    Scene.settings.offset,
  ]


def check_layout() -> None:
  """Raises if the ctypes mirror of MjpbrScene disagrees with the compiled library."""
  out = (ctypes.c_int64 * 8)()
  _lib_or_raise().mjpbr_struct_layout(out)
  if list(out) != python_layout():
    raise RuntimeError(f"MjpbrScene layout mismatch: library {list(out)}, bindings {python_layout()}")


def _lib_or_raise() -> ctypes.CDLL:
  if _lib is None:
    raise RuntimeError("libmjpbr is not loaded")
  return _lib


def call(name: str, *args) -> None:
  """Calls an entry point and raises MjpbrError (ValueError for argument errors) on failure."""
  lib = load()
  status = getattr(lib, name)(*args)
  if status != OK:
    message = lib.mjpbr_last_error().decode(errors="replace")
    if status == ERR_ARG:
      raise ValueError(message)
    raise MjpbrError(f"{name}: {message} (status {status})")
