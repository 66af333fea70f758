"""Environment maps: .hdr loading, split-sum precomputation, importance-sampling tables.

The resources of mujoco_warp_pbr/_src/envmap.py: equirect images in MuJoCo's Z-up world (row 0 =
+z, centre column = +x); per map a mipmapped float16 radiance texture (at most 2048 wide), an
8-level GGX-prefiltered stack (512 samples per texel), SH9 Lambertian radiance coefficients and
the luminance * sin(theta) piecewise-constant sampling distribution (256 wide) for the path
tracer. The host decodes and reduces the images; the stack, the SH9 projection and the sampling
tables are computed on the GPU by libmjpbr (the reference computes the latter two with NumPy).
"""

from __future__ import annotations

import dataclasses
import math
import os
from pathlib import Path
from typing import Any

import numpy as np
import torch

from mujoco_warp_pbr_gb300 import _lib

PREFILTER_WIDTH = 256
PREFILTER_LEVELS = 8
PREFILTER_SAMPLES = 512
MAX_RADIANCE_WIDTH = 2048
CDF_WIDTH = 256


class _HdrReader:
  """Cursor over the bytes of a Radiance picture file (Ward, "Real Pixels", Graphics Gems II,
  1991): a text header ended by an empty line, a resolution line, then one scanline per image row
  of 4-byte RGBE pixels (a shared 8-bit exponent E over three 8-bit mantissas: value = M * 2^(E -
  136), 0 for E = 0), each scanline either flat or, when it opens with the bytes 2, 2 and the
  width (high byte first), run-length encoded per component: a byte n > 128 repeats the next byte
  n - 128 times, a byte 0 < n <= 128 is followed by n literal bytes."""

  def __init__(self, data: bytes, path: str):
    self.data = data
    self.path = path
    self.pos = 0

  def fail(self, what: str) -> ValueError:
    return ValueError(f"{self.path}: {what}")

  def header(self) -> tuple[int, int]:
    """Skips the header; returns (height, width) of a '-Y H +X W' picture."""
    if not self.data.startswith(b"#?"):
      raise self.fail("not a Radiance .hdr file (missing '#?' signature)")
    blank = self.data.find(b"\n\n")
    line_end = self.data.find(b"\n", blank + 2) if blank >= 0 else -1
    if line_end < 0:
      raise self.fail("truncated .hdr header")
    fields = self.data[blank + 2 : line_end].split()
    if len(fields) < 4 or fields[0] != b"-Y" or fields[2] != b"+X" or not (fields[1].isdigit() and fields[3].isdigit()):
      raise self.fail("only '-Y H +X W' oriented .hdr files are supported")
    self.pos = line_end + 1
    return int(fields[1]), int(fields[3])

  def is_run_length(self, width: int) -> bool:
    d, p = self.data, self.pos
    return 8 <= width <= 0x7FFF and p + 2 < len(d) and d[p] == 2 and d[p + 1] == 2 and d[p + 2] < 128

  def flat(self, width: int, y: int) -> np.ndarray:
    n = 4 * width
    if self.pos + n > len(self.data):
      raise self.fail(f"truncated pixel data in scanline {y}")
    row = np.frombuffer(self.data, dtype=np.uint8, count=n, offset=self.pos).reshape(width, 4)
    self.pos += n
    return row

  def component(self, width: int, y: int) -> np.ndarray:
    """One run-length encoded component of a scanline."""
    out = np.empty(width, np.uint8)
    d, n = self.data, len(self.data)
    filled = 0
    while filled < width:
      if self.pos >= n:
        raise self.fail(f"truncated run-length data in scanline {y}")
      code = d[self.pos]
      self.pos += 1
      repeat = code > 128
      count = code - 128 if repeat else code
      body = 1 if repeat else count
      if count == 0 or count > width - filled or self.pos + body > n:
        raise self.fail(f"bad run-length data in scanline {y}")
      out[filled : filled + count] = d[self.pos] if repeat else np.frombuffer(d, np.uint8, count, self.pos)
      self.pos += body
      filled += count
    return out

  def run_length(self, width: int, y: int) -> np.ndarray:
    d, p = self.data, self.pos
    if p + 4 > len(d) or (d[p + 2] << 8 | d[p + 3]) != width:
      raise self.fail(f"scanline {y} width does not match the header")
    self.pos = p + 4
    return np.stack([self.component(width, y) for _ in range(4)], axis=-1)


def load_hdr(path: str | os.PathLike) -> np.ndarray:
  """Reads a Radiance RGBE (.hdr) picture as float32 (height, width, 3) linear radiance: flat and
  run-length encoded scanlines of '-Y H +X W' pictures, as mujoco_warp_pbr/_src/envmap.py:106-142
  accepts (the error messages are those of the reference's tests).

  Raises:
    ValueError: for a file that is not '-Y H +X W' RGBE or whose pixel data is truncated or
      malformed.
  """
  reader = _HdrReader(Path(path).read_bytes(), str(path))
  height, width = reader.header()
  rgbe = np.empty((height, width, 4), dtype=np.uint8)
  for y in range(height):
    rgbe[y] = reader.run_length(width, y) if reader.is_run_length(width) else reader.flat(width, y)
  exponent = rgbe[..., 3:4].astype(np.int32)
  mantissa = rgbe[..., :3].astype(np.float32)
  return np.where(exponent > 0, np.ldexp(mantissa, exponent - 136), np.float32(0.0)).astype(np.float32)


def envmap_images(envmap: Any) -> list[np.ndarray]:
  """The envmap argument (path, (h, w, 3) array, or a list of those) as float32 images."""
  if envmap is None:
    return []
  items = envmap if isinstance(envmap, (list, tuple)) else [envmap]
  images = []
  for i, item in enumerate(items):
    if isinstance(item, (str, bytes, os.PathLike)):
      images.append(load_hdr(os.fsdecode(item)))
      continue
    image = np.asarray(item)
    if image.ndim != 3 or image.shape[2] not in (3, 4) or image.shape[0] < 1 or image.shape[1] < 1:
      raise ValueError(f"envmap[{i}] must be a path or a (height, width, 3) radiance array, got shape {image.shape}")
    images.append(np.asarray(image[..., :3], np.float32))
  return images


def reduce_width(image: np.ndarray, max_width: int) -> np.ndarray:
  """Halves an image (2 x 2 box filter over its even-sized part, odd last rows / columns dropped)
  until it is at most max_width wide. Each output texel is the exact mean of its four inputs
  (summed in float64), rounded once to the input's type."""
  while image.shape[1] > max_width:
    h, w = image.shape[0] & ~1, image.shape[1] & ~1
    a = image[:h, :w].astype(np.float64)
    image = (((a[0::2, 0::2] + a[0::2, 1::2]) + (a[1::2, 0::2] + a[1::2, 1::2])) * 0.25).astype(image.dtype)
  return image


def _nearest(image: np.ndarray, shape: tuple[int, int]) -> np.ndarray:
  """Nearest-texel resampling of an image to shape (rows, columns), texel centres aligned."""
  rows = np.minimum(((np.arange(shape[0]) + 0.5) * image.shape[0] / shape[0]).astype(np.int64), image.shape[0] - 1)
  cols = np.minimum(((np.arange(shape[1]) + 0.5) * image.shape[1] / shape[1]).astype(np.int64), image.shape[1] - 1)
  return image[rows[:, None], cols[None, :]]


def _reduced_shape(shape: tuple[int, ...], max_width: int) -> tuple[int, int]:
  h, w = int(shape[0]), int(shape[1])
  while w > max_width:
    h, w = h // 2, w // 2
  return h, w


@dataclasses.dataclass
class HostEnvironments:
  """Host-side inputs of the environment maps of a context (the tables are computed on the GPU)."""

  radiance: list[np.ndarray]  # (h, w, 4) float16 level 0 per map
  linear: list[np.ndarray]  # (h, w, 3) float32, the same images before the float16 conversion
  cdf_images: list[np.ndarray]  # (ch, cw, 3) float64 at most CDF_WIDTH wide, one shape for all maps
  prefilter_levels: int
  prefilter_height: int
  prefilter_width: int
  max_width: float

  @property
  def nenv(self) -> int:
    return len(self.radiance)


def prepare_environments(images: list[np.ndarray]) -> HostEnvironments:
  """Radiance textures at most MAX_RADIANCE_WIDTH wide and the images the sampling tables are
  built from (at most CDF_WIDTH wide, every map resampled to the first map's table shape)."""
  radiance, linear, cdf_images = [], [], []
  cdf_shape = None
  for im in images:
    rgb = np.asarray(im, np.float32)[..., :3]
    small = reduce_width(rgb, MAX_RADIANCE_WIDTH)
    linear.append(np.ascontiguousarray(small))
    alpha = np.ones((*small.shape[:2], 1), np.float32)
    radiance.append(np.concatenate([small, alpha], axis=-1).astype(np.float16))
    src = rgb.astype(np.float64)
    if cdf_shape is not None and _reduced_shape(src.shape, CDF_WIDTH) != cdf_shape:
      src = _nearest(src, cdf_shape)
    table_image = reduce_width(src, CDF_WIDTH)
    cdf_shape = cdf_shape or table_image.shape[:2]
    cdf_images.append(np.ascontiguousarray(table_image))
  pw = min(PREFILTER_WIDTH, min(im.shape[1] for im in linear))
  return HostEnvironments(
    radiance=radiance,
    linear=linear,
    cdf_images=cdf_images,
    prefilter_levels=PREFILTER_LEVELS,
    prefilter_height=max(pw // 2, 1),
    prefilter_width=pw,
    max_width=float(max(im.shape[1] for im in linear)),
  )


@dataclasses.dataclass
class DeviceEnvironments:
  """Device resources: radiance textures (descriptions + bytes), prefiltered stacks, SH, tables."""

  radiance_desc: torch.Tensor
  radiance_data: torch.Tensor
  desc: list[Any]
  prefiltered: torch.Tensor  # (nenv, levels, h, w, 4) float16 stored as int16
  sh: torch.Tensor
  prob: torch.Tensor
  marginal: torch.Tensor
  conditional: torch.Tensor
  levels: int
  height: int
  width: int
  nenv: int


def upload_environments(env: HostEnvironments, device: torch.device) -> DeviceEnvironments:
  from mujoco_warp_pbr_gb300.context import TEX_RGBA16F
  from mujoco_warp_pbr_gb300.context import pack_textures
  from mujoco_warp_pbr_gb300.context import upload_textures

  ts = pack_textures([(TEX_RGBA16F, im) for im in env.radiance])
  desc, data = upload_textures(ts, device)
  L, H, W = env.prefilter_levels, env.prefilter_height, env.prefilter_width
  stack = torch.zeros((env.nenv, L, H, W, 4), dtype=torch.int16, device=device)
  stream = torch.cuda.current_stream(device).cuda_stream
  for e, d in enumerate(ts.desc):
    _lib.call("mjpbr_prefilter_env", d, data.data_ptr(), L, H, W, PREFILTER_SAMPLES, stack[e].data_ptr(), stream)

  # SH9 radiance and importance-sampling tables on the GPU (libmjpbr, double precision)
  sh = torch.empty((env.nenv, 9, 3), dtype=torch.float32, device=device)
  for e, im in enumerate(env.linear):
    img = torch.from_numpy(im).to(device)
    rows = torch.empty((im.shape[0], 27), dtype=torch.float64, device=device)
    _lib.call("mjpbr_env_sh9", img.data_ptr(), im.shape[0], im.shape[1], rows.data_ptr(), sh[e].data_ptr(), stream)
  ch, cw = env.cdf_images[0].shape[:2]
  prob = torch.empty((env.nenv, ch, cw), dtype=torch.float32, device=device)
  marginal = torch.empty((env.nenv, ch + 1), dtype=torch.float32, device=device)
  conditional = torch.empty((env.nenv, ch, cw + 1), dtype=torch.float32, device=device)
  for e, im in enumerate(env.cdf_images):
    img = torch.from_numpy(im).to(device)
    _lib.call("mjpbr_env_sampling_tables", img.data_ptr(), ch, cw, prob[e].data_ptr(), marginal[e].data_ptr(), conditional[e].data_ptr(), stream)
  torch.cuda.current_stream(device).synchronize()  # the host images above are freed on return

  return DeviceEnvironments(
    radiance_desc=desc,
    radiance_data=data,
    desc=ts.desc,
    prefiltered=stack,
    sh=sh,
    prob=prob,
    marginal=marginal,
    conditional=conditional,
    levels=L,
    height=H,
    width=W,
    nenv=env.nenv,
  )


def texel_angle(width: float) -> float:
  """Angular size of one radiance texel at mip 0."""
  return 2.0 * math.pi / width

