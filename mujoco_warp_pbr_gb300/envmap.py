"""Environment maps: .hdr loading, split-sum precomputation, importance-sampling tables.

Follows mujoco_warp_pbr/_src/envmap.py: equirect images in MuJoCo's Z-up world (row 0 = +z,
centre column = +x); per map a mipmapped float16 radiance texture (at most 2048 wide), an
8-level GGX-prefiltered stack (computed on the GPU by libmjpbr, 512 samples per texel), SH9
Lambertian radiance coefficients (float64 on the host) and the luminance * sin(theta)
piecewise-constant sampling distribution (256 wide) for the path tracer.
"""

from __future__ import annotations

import dataclasses
import math
import os
import re
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
_LUMINANCE = np.array([0.2126, 0.7152, 0.0722])


def _decode_rle_scanline(data: bytes, pos: int, width: int, path: str, y: int) -> tuple[np.ndarray, int]:
  """Adaptive run-length encoded RGBE scanline at pos -> ((width, 4) bytes, end position)."""
  line = bytearray(4 * width)
  n = len(data)
  for c in range(4):
    x = c * width
    end = x + width
    while x < end:
      if pos >= n:
        raise ValueError(f"{path}: truncated run-length data in scanline {y}")
      count = data[pos]
      pos += 1
      if count > 128:
        count -= 128
        if count > end - x or pos >= n:
          raise ValueError(f"{path}: bad run-length data in scanline {y}")
        line[x : x + count] = bytes((data[pos],)) * count
        pos += 1
      else:
        if count == 0 or count > end - x or pos + count > n:
          raise ValueError(f"{path}: bad run-length data in scanline {y}")
        line[x : x + count] = data[pos : pos + count]
        pos += count
      x += count
  return np.frombuffer(bytes(line), dtype=np.uint8).reshape(4, width).T, pos


def load_hdr(path: str | os.PathLike) -> np.ndarray:
  """Reads a Radiance RGBE (.hdr) file as float32 (height, width, 3) linear radiance
  (mujoco_warp_pbr/_src/envmap.py:106-142: flat and adaptive-RLE scanlines, '-Y H +X W' only).

  Raises:
    ValueError: for a file that is not '-Y H +X W' RGBE or whose pixel data is truncated or
      malformed.
  """
  data = Path(path).read_bytes()
  if not data.startswith(b"#?"):
    raise ValueError(f"{path}: not a Radiance .hdr file (missing '#?' signature)")
  try:
    header_end = data.index(b"\n\n") + 2
    resolution_end = data.index(b"\n", header_end)
  except ValueError:
    raise ValueError(f"{path}: truncated .hdr header") from None
  match = re.match(rb"-Y (\d+) \+X (\d+)", data[header_end:resolution_end])
  if match is None:
    raise ValueError(f"{path}: only '-Y H +X W' oriented .hdr files are supported")
  height, width = int(match.group(1)), int(match.group(2))
  pos = resolution_end + 1
  rgbe = np.empty((height, width, 4), dtype=np.uint8)
  for y in range(height):
    rle = 8 <= width <= 0x7FFF and data[pos : pos + 2] == b"\x02\x02" and pos + 2 < len(data) and not data[pos + 2] & 0x80
    if not rle:
      if pos + 4 * width > len(data):
        raise ValueError(f"{path}: truncated pixel data in scanline {y}")
      rgbe[y] = np.frombuffer(data, dtype=np.uint8, count=4 * width, offset=pos).reshape(width, 4)
      pos += 4 * width
      continue
    if (data[pos + 2] << 8 | data[pos + 3]) != width:
      raise ValueError(f"{path}: scanline {y} width does not match the header")
    rgbe[y], pos = _decode_rle_scanline(data, pos + 4, width, str(path), y)
  exponent = rgbe[..., 3].astype(np.int32)
  scale = np.where(exponent > 0, np.ldexp(1.0, exponent - 136), 0.0).astype(np.float32)
  return rgbe[..., :3].astype(np.float32) * scale[..., None]


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


def downsample(image: np.ndarray, max_width: int) -> np.ndarray:
  while image.shape[1] > max_width:
    h, w = image.shape[0] // 2 * 2, image.shape[1] // 2 * 2
    image = image[:h, :w].reshape(h // 2, 2, w // 2, 2, -1).mean(axis=(1, 3))
  return image


def sh9_irradiance(image: np.ndarray) -> np.ndarray:
  """SH9 coefficients (9, 3) of Lambertian radiance (irradiance / pi) of an equirect image
  (Ramamoorthi & Hanrahan 2001; envmap.py:224-249)."""
  h, w, _ = image.shape
  theta = (np.arange(h) + 0.5) / h * np.pi
  phi = ((np.arange(w) + 0.5) / w - 0.5) * 2.0 * np.pi
  st, ct = np.sin(theta)[:, None], np.cos(theta)[:, None]
  x, y, z = st * np.cos(phi)[None], st * np.sin(phi)[None], np.broadcast_to(ct, (h, w))
  basis = np.stack(
    [
      np.full((h, w), 0.282095),
      0.488603 * y,
      0.488603 * z,
      0.488603 * x,
      1.092548 * x * y,
      1.092548 * y * z,
      0.315392 * (3.0 * z * z - 1.0),
      1.092548 * x * z,
      0.546274 * (x * x - y * y),
    ]
  )
  solid_angle = (2.0 * np.pi / w) * (np.pi / h) * np.broadcast_to(st, (h, w))
  coeffs = np.einsum("khw,hwc->kc", basis * solid_angle, image.astype(np.float64))
  band = np.array([np.pi, 2 * np.pi / 3, 2 * np.pi / 3, 2 * np.pi / 3] + [np.pi / 4] * 5)
  return (coeffs * band[:, None] / np.pi).astype(np.float32)


def sampling_tables(image: np.ndarray) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
  """(cell probabilities (h, w), marginal row CDF (h + 1,), conditional column CDFs (h, w + 1))
  of a distribution over equirect cells proportional to luminance * sin(theta) (envmap.py:409-430)."""
  small = downsample(np.asarray(image, np.float64)[..., :3], CDF_WIDTH)
  h = small.shape[0]
  lum = small @ _LUMINANCE
  sin_theta = np.sin((np.arange(h) + 0.5) / h * np.pi)[:, None]
  weight = lum * sin_theta + 1e-6 * max(float(lum.mean()), 1e-12)
  prob = weight / weight.sum()
  row = prob.sum(axis=1)
  marginal = np.concatenate([[0.0], np.cumsum(row)])
  conditional = np.concatenate([np.zeros((h, 1)), np.cumsum(prob, axis=1) / np.maximum(row[:, None], 1e-30)], axis=1)
  marginal[-1] = 1.0
  conditional[:, -1] = 1.0
  return prob.astype(np.float32), marginal.astype(np.float32), conditional.astype(np.float32)


def _resize_nearest(image: np.ndarray, shape: tuple[int, int]) -> np.ndarray:
  h, w = shape
  ys = ((np.arange(h) + 0.5) / h * image.shape[0]).astype(int)
  xs = ((np.arange(w) + 0.5) / w * image.shape[1]).astype(int)
  return image[ys][:, xs]


def _downsampled_shape(shape: tuple[int, ...], max_width: int) -> tuple[int, int]:
  h, w = shape[0], shape[1]
  while w > max_width:
    h, w = h // 2, w // 2
  return h, w


@dataclasses.dataclass
class HostEnvironments:
  """Host-side resources of the environment maps of a context."""

  radiance: list[np.ndarray]  # (h, w, 4) float16 level 0 per map
  sh: np.ndarray  # (nenv, 9, 3)
  prob: np.ndarray  # (nenv, h, w)
  marginal: np.ndarray  # (nenv, h + 1)
  conditional: np.ndarray  # (nenv, h, w + 1)
  prefilter_levels: int
  prefilter_height: int
  prefilter_width: int
  max_width: float

  @property
  def nenv(self) -> int:
    return len(self.radiance)


def prepare_environments(images: list[np.ndarray]) -> HostEnvironments:
  radiance, shs, tables = [], [], []
  shape = None
  widths = []
  for im in images:
    small = downsample(np.asarray(im, np.float32)[..., :3], MAX_RADIANCE_WIDTH)
    h, w, _ = small.shape
    widths.append(w)
    radiance.append(np.concatenate([small, np.ones((h, w, 1), np.float32)], axis=-1).astype(np.float16))
    shs.append(sh9_irradiance(small))
    src = im
    if shape is not None and _downsampled_shape(im.shape, CDF_WIDTH) != shape:
      src = _resize_nearest(im, shape)
    table = sampling_tables(src)
    shape = shape or table[0].shape
    tables.append(table)
  pw = min(PREFILTER_WIDTH, min(widths))
  return HostEnvironments(
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

  def dev(a: np.ndarray) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a)).to(device)

  return DeviceEnvironments(
    radiance_desc=desc,
    radiance_data=data,
    desc=ts.desc,
    prefiltered=stack,
    sh=dev(env.sh),
    prob=dev(env.prob),
    marginal=dev(env.marginal),
    conditional=dev(env.conditional),
    levels=L,
    height=H,
    width=W,
    nenv=env.nenv,
  )


def texel_angle(width: float) -> float:
  """Angular size of one radiance texel at mip 0."""
  return 2.0 * math.pi / width

