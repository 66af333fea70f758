"""FP32 roofline of the render kernels: the algorithmic work of a frame from operation counts.

The real-time kernel is not HBM-bound (its compulsory traffic is ~16-28 B per pixel plus the
scene), so its roofline is FP32 issue. The counting build of the render kernels
(libmjpbr_count.so, `_lib.load_counting`) counts per frame: ray queries (closest / any hit),
bounding-box tests, triangle tests, primitive tests by type, shaded surface hits, light
evaluations, environment lookups (SH9 irradiance + prefiltered specular) and background lookups,
and for the path tracer its surface vertices, light samples and environment samples.
FLOPS_PER_OP turns the counts into algorithmic FP32 operations (an FMA counts 2, a min / max /
compare 1, a reciprocal / square root / transcendental 4); the constants are a fixed model of the
kernels' arithmetic, stated here and not measured. The achieved rate is that work over the
product kernel's CUDA-event time; the peak is the nominal FP32 rate of a GB300 (no measured FP32
figure exists for this pool): 152 SMs x 128 lanes x 2 FLOP x 2.07 GHz.
"""

from __future__ import annotations

import ctypes

# counter order of csrc/opcount.cuh (enum OpCount)
OPS = (
  "ray_closest", "ray_any", "box", "triangle", "plane", "sphere", "ellipsoid", "capsule", "cylinder", "box_prim", "shade", "light",
  "env", "background", "pt_vertex", "pt_light", "pt_env_sample",
)
COPIES = 32

FLOPS_PER_OP = {
  "ray_closest": 20,  # reciprocal direction, traversal setup
  "ray_any": 20,
  "box": 20,  # slab test of one child box against the precomputed inverse direction
  "triangle": 30,  # watertight (Woop) test: shear, edge functions, determinant, distance
  "plane": 12,
  "sphere": 25,
  "ellipsoid": 40,
  "capsule": 70,
  "cylinder": 60,
  "box_prim": 60,
  "shade": 250,  # surface evaluation (textures, normal map, specular AA), lobes, DFG, ambient terms
  "light": 90,  # light vector / attenuation / spot cone, GGX D, Smith V, Schlick F, sums
  "env": 220,  # SH9 irradiance (27 FMA), dominant direction, two equirect lookups (atan2, acos, trilinear)
  "background": 60,  # equirect lookup of the radiance mips
  "pt_vertex": 350,  # path vertex: surface, lobes, tangent frame, BSDF sample, pdf and value, throughput
  "pt_light": 200,  # next-event estimation of a light: sampling the bulb, light terms, two BSDF values
  "pt_env_sample": 200,  # environment importance sample: two CDF searches, direction, BSDF, pdfs, MIS weight
}

FP32_PEAK_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12


def counts_from_device(raw) -> dict[str, int]:
  """Sums the per-CTA copies of a (len(OPS) * COPIES) uint64 counter array (host sequence)."""
  vals = [int(v) for v in raw]
  return {name: sum(vals[i * COPIES : (i + 1) * COPIES]) for i, name in enumerate(OPS)}


def flops(counts: dict[str, int]) -> int:
  return sum(FLOPS_PER_OP[k] * v for k, v in counts.items())


def rays(counts: dict[str, int]) -> int:
  return counts["ray_closest"] + counts["ray_any"]


def count_frame(scene: ctypes.Structure, seed: int, stream: int) -> dict[str, int]:
  """Renders one frame of the scene descriptor through the counting build and returns the counts."""
  import torch

  from mujoco_warp_pbr_gb300 import _lib

  lib = _lib.load_counting()
  buf = torch.zeros(len(OPS) * COPIES, dtype=torch.int64, device="cuda")
  if lib.mjpbr_count_set(buf.data_ptr()) != 0:
    raise RuntimeError("mjpbr_count_set failed")
  try:
    for name, args in (("mjpbr_refit_bvh", (ctypes.byref(scene), stream)), ("mjpbr_render", (ctypes.byref(scene), seed & 0xFFFFFFFF, stream))):
      if getattr(lib, name)(*args) != 0:
        raise RuntimeError(f"{name} (counting build): {lib.mjpbr_last_error().decode(errors='replace')}")
    torch.cuda.synchronize()
  finally:
    lib.mjpbr_count_set(None)
  return counts_from_device(buf.cpu().tolist())


def fp32_roofline(counts: dict[str, int], pixels_counted: int, pixels_frame: int, frame_ms: float, kernel: str = "rt_kernel") -> dict:
  """The roofline object of a frame of pixels_frame pixels rendered in frame_ms, from the counts
  of a frame of pixels_counted pixels of the same scene."""
  scale = pixels_frame / pixels_counted
  frame_flops = flops(counts) * scale
  achieved = frame_flops / (frame_ms * 1e-3) / 1e12
  return {
    "bound": "fp32",
    "kernel": kernel,
    "achieved": achieved,
    "peak": FP32_PEAK_TFLOPS,
    "unit": "TFLOP/s",
    "frac": achieved / FP32_PEAK_TFLOPS,
    "peak_source": "nominal: 152 SMs x 128 FP32 lanes x 2 x 2.07 GHz",
    "flops_per_px": flops(counts) / pixels_counted,
    "rays_per_px": rays(counts) / pixels_counted,
    "counts_per_px": {k: v / pixels_counted for k, v in counts.items()},
    "model": "mujoco_warp_pbr_gb300/roofline.py FLOPS_PER_OP",
    "counted_on_px": pixels_counted,
  }
