"""Python side of the CPU oracle (oracle/mjpbr_oracle.c) — TEST INFRASTRUCTURE ONLY.

Builds the same MjpbrScene descriptor the library renders from, but over host (numpy) arrays,
and runs the C restatement of the reference's real-time and path-traced tiers on the CPU cores.
The oracle shares no code with the product: its host preparation (materials, lights, exposure,
textures, environments, output layout) is oracle/host_prep.py, its struct mirror
oracle/scene_struct.py (read from include/mjpbr.h). The tables the GPU computes at context
creation (DFG table, texture mips, prefiltered environment stacks, SH9 coefficients, sampling
tables) come from the oracle's own functions unless the caller passes the GPU's copies (to
isolate the render kernels from the table kernels, which tests compare separately).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use this module.
"""

from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path
from typing import Any

import numpy as np

from oracle import host_prep
from oracle import scene_struct as ss

HERE = Path(__file__).resolve().parent
SOURCE = HERE / "mjpbr_oracle.c"
BUILD = HERE / "_build"
LIBRARY = BUILD / "libmjpbr_oracle.so"
CFLAGS = ["-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-Wall", "-Wno-unused-parameter"]
# the reference's table sizes (ibl.py DFG table 128 x 128 with 1024 samples; envmap.py prefilter
# with 512 samples per texel)
DFG_LUT_SIZE = 128
DFG_LUT_SAMPLES = 1024
PREFILTER_SAMPLES = 512

_lib_handle: ctypes.CDLL | None = None


def build(force: bool = False) -> Path:
  """Compiles the oracle with gcc (no fused multiply-add, no fast math)."""
  BUILD.mkdir(exist_ok=True)
  header = HERE.parent / "include" / "mjpbr.h"
  if force or not LIBRARY.exists() or LIBRARY.stat().st_mtime < max(SOURCE.stat().st_mtime, header.stat().st_mtime):
    tmp = LIBRARY.with_suffix(".so.tmp")
    subprocess.run(["gcc", *CFLAGS, "-o", str(tmp), str(SOURCE), "-lm"], check=True, capture_output=True, text=True)
    tmp.replace(LIBRARY)
  return LIBRARY


def load() -> ctypes.CDLL:
  global _lib_handle
  if _lib_handle is None:
    build()
    lib = ctypes.CDLL(str(LIBRARY))
    vp, i32 = ctypes.c_void_p, ctypes.c_int
    lib.oracle_render_rt.argtypes = [ctypes.POINTER(ss.Scene), vp, ctypes.c_uint32, i32, i32, i32]
    lib.oracle_render_rt.restype = i32
    lib.oracle_render_pt.argtypes = [ctypes.POINTER(ss.Scene), vp, ctypes.c_uint32, i32, i32, i32]
    lib.oracle_render_pt.restype = i32
    lib.oracle_denoise.argtypes = [ctypes.POINTER(ss.Scene), i32]
    lib.oracle_denoise.restype = i32
    lib.oracle_dfg_lut.argtypes = [vp, i32, i32]
    lib.oracle_build_mips.argtypes = [ctypes.POINTER(ss.Texture), vp]
    lib.oracle_prefilter.argtypes = [ctypes.POINTER(ss.Texture), vp, i32, i32, i32, i32, vp]
    lib.oracle_struct_layout.argtypes = [ctypes.POINTER(ctypes.c_int64)]
    lib.oracle_set_mesh_bvh.argtypes = [i32]
    lib.oracle_set_hfields.argtypes = [i32, vp, vp, vp, vp, vp]
    lib.oracle_set_hfields.restype = i32
    lib.oracle_hfield_mesh.argtypes = [i32, ctypes.POINTER(i32), ctypes.POINTER(i32), vp, vp]
    lib.oracle_hfield_mesh.restype = i32
    lib.oracle_nthreads.restype = i32
    lib.oracle_sincos_turns.argtypes = [ctypes.c_float, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]
    lib.oracle_rand01.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
    lib.oracle_rand01.restype = ctypes.c_float
    lib.oracle_float_to_half.argtypes = [ctypes.c_float]
    lib.oracle_float_to_half.restype = ctypes.c_uint16
    lib.oracle_half_to_float.argtypes = [ctypes.c_uint16]
    lib.oracle_half_to_float.restype = ctypes.c_float
    out = (ctypes.c_int64 * 8)()
    lib.oracle_struct_layout(out)
    if list(out) != ss.layout():
      raise RuntimeError(f"oracle MjpbrScene layout {list(out)} differs from the header mirror {ss.layout()}")
    _lib_handle = lib
  return _lib_handle


def dfg_lut(size: int = DFG_LUT_SIZE, nsample: int = DFG_LUT_SAMPLES) -> np.ndarray:
  lut = np.zeros((size, size, 2), np.float32)
  load().oracle_dfg_lut(lut.ctypes.data, size, nsample)
  return lut


def build_mips(desc: list[Any], data: np.ndarray) -> np.ndarray:
  """Texture bytes with every mip level filled by the oracle (desc: MjpbrTexture descriptions of
  the textures whose level 0 is in data)."""
  data = data.copy()
  for d in desc:
    load().oracle_build_mips(d, data.ctypes.data)
  return data


def prefilter(env: host_prep.Environments, data: np.ndarray, desc: list[Any], nsample: int = PREFILTER_SAMPLES) -> np.ndarray:
  L, H, W = env.prefilter_levels, env.prefilter_height, env.prefilter_width
  stack = np.zeros((env.nenv, L, H, W, 4), np.uint16)
  for e, d in enumerate(desc):
    load().oracle_prefilter(d, data.ctypes.data, L, H, W, nsample, stack[e].ctypes.data)
  return stack


def environment_textures(env: host_prep.Environments) -> tuple[list[Any], np.ndarray]:
  """The environments' radiance textures (float16 RGBA, level 0 filled), packed."""
  return host_prep.pack_textures([(host_prep.TEX_RGBA16F, im) for im in env.radiance], ss.Texture)


def _b(a: Any, dtype: Any, tail: tuple[int, ...]) -> np.ndarray:
  return np.ascontiguousarray(np.asarray(a, dtype).reshape((-1, *tail)) if tail else np.asarray(a, dtype).reshape(1, -1))


class OracleScene:
  """A scene prepared for the oracle: host arrays in the MjpbrScene layout.

  mjm / mjd: HostModel / HostData (per-world data with a leading nworld dimension, or one world
  replicated). options: create_render_context keyword arguments. per_world: replacements of model /
  context tables (geom_rgba, geom_roughness, ... with a leading nworld dimension). tables: optional
  GPU copies of dfg_lut, tex_data, env_data, env_prefiltered.
  """

  def __init__(self, mjm: Any, mjd: Any, nworld: int, options: dict[str, Any], per_world: dict[str, np.ndarray] | None = None, tables: dict[str, np.ndarray] | None = None):
    self.hc = host_prep.prepare(mjm, mjd, nworld, options)
    self.nworld = nworld
    tables = dict(tables or {})
    per_world = dict(per_world or {})
    f32, i32 = np.float32, np.int32
    nw = nworld

    def world_data(a: np.ndarray, n: int, k: int) -> np.ndarray:
      a = np.asarray(a, f32)
      if a.ndim == 2 or (a.ndim == 3 and a.shape[0] != nw):
        a = np.broadcast_to(a.reshape(1, n, k), (nw, n, k))
      return np.ascontiguousarray(a.reshape(nw, n, k))

    ngeom, nlight, ncam = mjm.ngeom, mjm.nlight, mjm.ncam
    nmat = mjm.nmat
    o = self.hc.outputs
    st = dict(self.hc.settings)
    a: dict[str, Any] = {
      "geom_type": np.ascontiguousarray(mjm.geom_type, i32),
      "geom_dataid": _b(mjm.geom_dataid, i32, ()),
      "geom_matid": _b(mjm.geom_matid, i32, ()),
      "geom_size": _b(mjm.geom_size, f32, (1, ngeom, 3))[0:1].reshape(1, ngeom, 3),
      "geom_rgba": np.ascontiguousarray(np.asarray(per_world.pop("geom_rgba", mjm.geom_rgba), f32).reshape(-1, ngeom, 4)),
      "mat_rgba": _b(mjm.mat_rgba if nmat else np.zeros((1, 4)), f32, (max(nmat, 1), 4)),
      "mat_emission": np.ascontiguousarray(np.asarray(per_world.pop("mat_emission", mjm.mat_emission if nmat else np.zeros(1)), f32).reshape(-1, max(nmat, 1))),
      "mat_texid": _b(mjm.mat_texid if nmat else -np.ones((1, 10)), i32, (max(nmat, 1), 10)),
      "mat_texrepeat": _b(mjm.mat_texrepeat if nmat else np.ones((1, 2)), f32, (max(nmat, 1), 2)),
      "mat_texuniform": _b(mjm.mat_texuniform if nmat else np.zeros(1), i32, ()),
      "light_type": _b(mjm.light_type if nlight else np.zeros(1), i32, ()),
      "light_castshadow": _b(mjm.light_castshadow if nlight else np.zeros(1), i32, ()),
      "light_active": _b(mjm.light_active if nlight else np.zeros(1), i32, ()),
      "light_attenuation": _b(mjm.light_attenuation if nlight else np.zeros((1, 3)), f32, (max(nlight, 1), 3)),
      "light_cutoff": _b(mjm.light_cutoff if nlight else np.zeros(1), f32, ()),
      "light_exponent": _b(mjm.light_exponent if nlight else np.zeros(1), f32, ()),
      "light_diffuse": _b(mjm.light_diffuse if nlight else np.zeros((1, 3)), f32, (max(nlight, 1), 3)),
      "light_specular": _b(mjm.light_specular if nlight else np.zeros((1, 3)), f32, (max(nlight, 1), 3)),
      "cam_projection": np.ascontiguousarray(mjm.cam_projection, i32),
      "cam_fovy": _b(mjm.cam_fovy, f32, ()),
      "cam_sensorsize": np.ascontiguousarray(np.asarray(mjm.cam_sensorsize, f32).reshape(-1, 2)),
      "cam_intrinsic": _b(mjm.cam_intrinsic, f32, (ncam, 4)),
      "geom_xpos": world_data(mjd.geom_xpos, ngeom, 3),
      "geom_xmat": world_data(mjd.geom_xmat, ngeom, 9),
      "cam_xpos": world_data(mjd.cam_xpos, ncam, 3),
      "cam_xmat": world_data(mjd.cam_xmat, ncam, 9),
      "light_xpos": world_data(mjd.light_xpos, nlight, 3) if nlight else None,
      "light_xdir": world_data(mjd.light_xdir, nlight, 3) if nlight else None,
    }
    a["geom_size"] = np.ascontiguousarray(np.asarray(mjm.geom_size, f32).reshape(1, ngeom, 3))
    if mjm.nmesh:
      a.update(
        {
          "mesh_vertadr": np.ascontiguousarray(mjm.mesh_vertadr, i32),
          "mesh_faceadr": np.ascontiguousarray(mjm.mesh_faceadr, i32),
          "mesh_normaladr": np.ascontiguousarray(mjm.mesh_normaladr, i32),
          "mesh_texcoordadr": np.ascontiguousarray(mjm.mesh_texcoordadr, i32),
          "mesh_vert": np.ascontiguousarray(mjm.mesh_vert, f32),
          "mesh_face": np.ascontiguousarray(mjm.mesh_face, i32),
          "mesh_normal": np.ascontiguousarray(mjm.mesh_normal, f32),
          "mesh_facenormal": np.ascontiguousarray(mjm.mesh_facenormal, i32),
          "mesh_texcoord": np.ascontiguousarray(mjm.mesh_texcoord, f32) if len(mjm.mesh_texcoord) else None,
          "mesh_facetexcoord": np.ascontiguousarray(mjm.mesh_facetexcoord, i32),
        }
      )
    t = {k: np.ascontiguousarray(v) for k, v in self.hc.tables.items()}
    for k, v in list(per_world.items()):
      t[k] = np.ascontiguousarray(np.asarray(v, t[k].dtype if k in t else f32))
    t["exposure"] = t["exposure"].reshape(-1)
    t["ambient_radiance"] = t["ambient_radiance"].reshape(-1, 3)
    a.update(t)
    rgb_stride, depth_stride, seg_stride = max(o["rgb_stride"], 1), max(o["depth_stride"], 1), max(o["seg_stride"], 1)
    self.rgb = np.zeros((nw, rgb_stride), np.uint32)
    self.depth = np.zeros((nw, depth_stride), f32)
    self.seg = np.zeros((nw, seg_stride, 2), i32)
    self.hdr = np.zeros((nw, rgb_stride, 3), f32)
    self.albedo = np.zeros((nw, rgb_stride, 3), f32)
    self.normal = np.zeros((nw, rgb_stride, 3), f32)
    aov_pix = rgb_stride if st.get("denoise") else 1
    self.aov = {
      "guide": np.zeros((nw, aov_pix, 4), np.uint32),
      "emission": np.zeros((nw, aov_pix, 3), f32),
      "demod": np.zeros((nw, aov_pix, 4), f32),
      "pong": np.zeros((nw, aov_pix, 4), f32),
    }
    self.dfg = np.ascontiguousarray(tables.get("dfg_lut", None) if "dfg_lut" in tables else dfg_lut())
    a.update(
      {
        "nworld": nw,
        "ngeom": ngeom,
        "nmat": max(nmat, 1),
        "nlight": nlight,
        "ncam": ncam,
        "nmesh": mjm.nmesh,
        "nhfield": nhfield_of(mjm),
        "ntex": mjm.ntex,
        "nrender": o["nrender"],
        "total_rays": o["total_rays"],
        "cam_id_map": o["cam_id_map"],
        "cam_res": o["cam_res"],
        "render_rgb": [int(v) for v in o["render_rgb"]],
        "render_depth": [int(v) for v in o["render_depth"]],
        "render_seg": [int(v) for v in o["render_seg"]],
        "ray_adr": o["ray_adr"],
        "rgb_adr": o["rgb_adr"],
        "depth_adr": o["depth_adr"],
        "seg_adr": o["seg_adr"],
        "rgb_stride": rgb_stride,
        "depth_stride": depth_stride,
        "seg_stride": seg_stride,
        "rgb_data": self.rgb,
        "depth_data": self.depth,
        "seg_data": self.seg,
        "hdr_data": self.hdr,
        "guide_albedo": self.albedo,
        "guide_normal": self.normal,
        "aov_guide": self.aov["guide"],
        "aov_emission": self.aov["emission"],
        "denoise_buffers": (self.aov["demod"], self.aov["pong"]),
        "denoise_iterations": int(options.get("denoise_iterations", 3)),
        "nbvh_geom": len(self.hc.enabled_geom_ids),
        "nnode": max(len(self.hc.enabled_geom_ids) - 1, 1),
        "enabled_geom_ids": np.ascontiguousarray(self.hc.enabled_geom_ids, i32),
        "dfg_lut": self.dfg,
        "dfg_size": self.dfg.shape[0],
        "settings": st,
      }
    )
    if self.hc.textures:
      desc, data = host_prep.pack_textures(self.hc.textures, ss.Texture)
      self.tex_desc = host_prep.desc_bytes(desc)
      self.tex_data = np.ascontiguousarray(tables["tex_data"]) if "tex_data" in tables else build_mips(desc, data)
      a["textures"] = self.tex_desc
      a["tex_data"] = self.tex_data
    env = self.hc.environments
    if env is not None:
      edesc, edata = environment_textures(env)
      self.env_desc = host_prep.desc_bytes(edesc)
      self.env_data = np.ascontiguousarray(tables["env_data"]) if "env_data" in tables else build_mips(edesc, edata)
      self.env_stack = np.ascontiguousarray(tables["env_prefiltered"]).view(np.uint16) if "env_prefiltered" in tables else prefilter(env, self.env_data, edesc)
      for key in ("env_sh", "env_prob", "env_marginal", "env_conditional"):
        if key in tables:  # the GPU's tables, to isolate the render kernels from the table kernels
          setattr(env, key[4:], np.ascontiguousarray(tables[key]))
      a.update(
        {
          "nenv": env.nenv,
          "env_radiance": self.env_desc,
          "env_data": self.env_data,
          "env_prefiltered": self.env_stack,
          "prefilter_levels": env.prefilter_levels,
          "prefilter_height": env.prefilter_height,
          "prefilter_width": env.prefilter_width,
          "env_sh": np.ascontiguousarray(env.sh),
          "env_prob": np.ascontiguousarray(env.prob),
          "env_marginal": np.ascontiguousarray(env.marginal),
          "env_conditional": np.ascontiguousarray(env.conditional),
          "cdf_height": env.prob.shape[1],
          "cdf_width": env.prob.shape[2],
        }
      )
    if options.get("camera_rays") is not None:
      self.ray_origin, self.ray_direction = host_prep.pack_camera_rays(options["camera_rays"], o["cam_res"])
      a.update({"ray_origin": self.ray_origin, "ray_direction": self.ray_direction, "bundle_res": o["cam_res"]})
    self.mesh_nface = np.ascontiguousarray(self.hc.mesh_nface, i32)
    self.hfields = hfield_arrays(mjm)
    self.arrays = a  # keeps every array alive
    self.scene = ss.fill({k: v for k, v in a.items() if v is not None})

  def render(self, seed: int = 0, worlds: tuple[int, int] | None = None, nthreads: int = 0, denoise: bool = True) -> dict[str, np.ndarray]:
    """Renders worlds [w0, w1) with the tier of the context's settings (real-time or path-traced);
    with settings.denoise the a-trous filter then runs over every world (unless denoise=False)."""
    w0, w1 = worlds if worlds is not None else (0, self.nworld)
    lib = load()
    set_hfields(self.hfields)
    fn = lib.oracle_render_pt if self.hc.settings["tier"] == 1 else lib.oracle_render_rt
    status = fn(self.scene, self.mesh_nface.ctypes.data if len(self.mesh_nface) else None, seed & 0xFFFFFFFF, w0, w1, nthreads)
    if status != 0:
      raise RuntimeError("oracle render failed")
    out = {"rgb": self.rgb, "depth": self.depth, "seg": self.seg, "hdr": self.hdr, "albedo": self.albedo, "normal": self.normal}
    if self.hc.settings["tier"] == 1 and self.hc.settings["denoise"]:
      out.update({f"aov_{k}": v.copy() for k, v in self.aov.items()})
      if denoise:
        self.denoise(nthreads)
    return out

  def denoise(self, nthreads: int = 0) -> None:
    """Runs the oracle's a-trous filter on the current demodulated buffer and guide arrays."""
    if load().oracle_denoise(self.scene, nthreads) != 0:
      raise RuntimeError("oracle_denoise failed")


def nhfield_of(mjm: Any) -> int:
  """Height fields of a model (0 for models without the hfield_* fields)."""
  nrow = getattr(mjm, "hfield_nrow", None)
  return 0 if nrow is None else int(len(np.asarray(nrow).reshape(-1)))


def hfield_arrays(mjm: Any) -> tuple[np.ndarray, ...]:
  """(nrow, ncol, size, adr, data) of a model's height fields as contiguous arrays (empty without)."""
  n = nhfield_of(mjm)
  if n == 0:
    return ()
  return (
    np.ascontiguousarray(np.asarray(mjm.hfield_nrow).reshape(-1), np.int32),
    np.ascontiguousarray(np.asarray(mjm.hfield_ncol).reshape(-1), np.int32),
    np.ascontiguousarray(np.asarray(mjm.hfield_size).reshape(-1, 4), np.float32),
    np.ascontiguousarray(np.asarray(mjm.hfield_adr).reshape(-1), np.int32),
    np.ascontiguousarray(np.asarray(mjm.hfield_data).reshape(-1), np.float32),
  )


def set_hfields(arrays: tuple[np.ndarray, ...]) -> None:
  """Gives the oracle a model's height fields (hfield_arrays), which it triangulates itself."""
  if not arrays:
    status = load().oracle_set_hfields(0, None, None, None, None, None)
  else:
    status = load().oracle_set_hfields(len(arrays[0]), *(a.ctypes.data for a in arrays))
  if status != 0:
    raise ValueError("height fields need at least 2 x 2 samples")


def hfield_mesh(h: int) -> tuple[np.ndarray, np.ndarray]:
  """The oracle's triangulation of height field h (after set_hfields): vertices, faces."""
  lib = load()
  nv, nf = ctypes.c_int32(0), ctypes.c_int32(0)
  if lib.oracle_hfield_mesh(h, ctypes.byref(nv), ctypes.byref(nf), None, None) != 0:
    raise IndexError(f"no height field {h}")
  vert = np.zeros((nv.value, 3), np.float32)
  face = np.zeros((nf.value, 3), np.int32)
  lib.oracle_hfield_mesh(h, ctypes.byref(nv), ctypes.byref(nf), vert.ctypes.data, face.ctypes.data)
  return vert, face


def unpack_rgb(rgb: np.ndarray) -> np.ndarray:
  """Packed RGBA8 (R in the low byte) -> (..., 3) uint8 channels."""
  v = np.asarray(rgb).astype(np.uint32)
  return np.stack([(v >> s) & 0xFF for s in (0, 8, 16)], axis=-1).astype(np.int32)
