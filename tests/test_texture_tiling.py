"""The tiled texture layout the render kernels sample (MJPBR_TEX_TILED: 4 x 4-texel tiles row by
row, levels padded to whole tiles, 128-byte aligned): the host layout of libmjpbr against a NumPy
restatement, and (GPU) the tiling kernel's bytes against a NumPy tiling of the row-major mips."""

import ctypes

import numpy as np
import pytest

from mujoco_warp_pbr_gb300 import _lib, context


def _rows(fmt: int, w: int, h: int) -> "_lib.Texture":
  ts = context.pack_textures([(fmt, np.zeros((h, w, 4), np.uint8 if fmt == context.TEX_RGBA8 else np.float16))])
  return ts.desc[0]


def _expected_offsets(d, start: int) -> list[int]:
  texel = 4 if d.format == context.TEX_RGBA8 else 8
  off = (start + 127) // 128 * 128
  out = []
  for level in range(d.nlevel):
    w, h = max(d.width >> level, 1), max(d.height >> level, 1)
    out.append(off)
    off += ((w + 3) // 4) * ((h + 3) // 4) * 16 * texel
    off = (off + 127) // 128 * 128
  return out + [off]


@pytest.mark.parametrize("fmt,w,h", [(0, 512, 512), (1, 1024, 512), (0, 37, 5), (1, 1, 1), (1, 6, 3)])
def test_tiled_layout_offsets(fmt, w, h):
  lib = _lib.load()
  rows = _rows(fmt, w, h)
  tiled = _lib.Texture()
  end = lib.mjpbr_tiled_texture(ctypes.byref(rows), 100, ctypes.byref(tiled))
  want = _expected_offsets(rows, 100)
  assert [tiled.level_offset[k] for k in range(rows.nlevel)] == want[:-1]
  assert end == want[-1]
  assert (tiled.layout, tiled.format, tiled.width, tiled.height, tiled.nlevel) == (1, rows.format, w, h, rows.nlevel)
  bad = _lib.Texture()
  assert lib.mjpbr_tiled_texture(ctypes.byref(bad), 0, ctypes.byref(tiled)) == -1


def _tile_level(img: np.ndarray) -> np.ndarray:
  """(h, w, c) -> the tiled sequence of texels (tiles row by row, texels of a tile row by row)."""
  h, w = img.shape[:2]
  th, tw = (h + 3) // 4, (w + 3) // 4
  pad = np.zeros((th * 4, tw * 4) + img.shape[2:], img.dtype)
  pad[:h, :w] = img
  return pad.reshape(th, 4, tw, 4, *img.shape[2:]).swapaxes(1, 2).reshape(th * tw * 16, *img.shape[2:])


@pytest.mark.gpu
@pytest.mark.parametrize("fmt,w,h", [(0, 64, 32), (1, 37, 21)])
def test_tiling_kernel_matches_numpy(fmt, w, h):
  torch = pytest.importorskip("torch")
  if not torch.cuda.is_available():
    pytest.skip("needs a CUDA GPU")
  rng = np.random.default_rng(3)
  img = rng.integers(0, 255, (h, w, 4)).astype(np.uint8) if fmt == 0 else rng.uniform(0, 4, (h, w, 4)).astype(np.float16)
  ts = context.pack_textures([(fmt, img)])
  _, rows_data = context.upload_textures(ts, torch.device("cuda"))
  desc, tiled_data = context.tile_textures(ts.desc, rows_data, torch.device("cuda"))
  torch.cuda.synchronize()
  rows_bytes = rows_data.cpu().numpy()
  tiled_bytes = tiled_data.cpu().numpy()
  t = _lib.Texture.from_buffer_copy(desc.cpu().numpy().tobytes()[: ctypes.sizeof(_lib.Texture)])
  d = ts.desc[0]
  texel = 4 if fmt == 0 else 8
  for level in range(d.nlevel):
    lw, lh = max(w >> level, 1), max(h >> level, 1)
    src = rows_bytes[d.level_offset[level] : d.level_offset[level] + lw * lh * texel].reshape(lh, lw, texel)
    tiled = _tile_level(src)
    got = tiled_bytes[t.level_offset[level] : t.level_offset[level] + tiled.size].reshape(tiled.shape)
    np.testing.assert_array_equal(got, tiled, err_msg=f"level {level}")
