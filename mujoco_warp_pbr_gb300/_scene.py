"""Filling the MjpbrScene descriptor from named arrays.

`fill_scene(fields)` takes a dict keyed by MjpbrScene field names. Array values may be torch
tensors (device pointers for libmjpbr) or numpy arrays (host pointers, for the CPU oracle used by
the tests); batched tables become (pointer, leading dimension). The caller keeps the arrays alive
while the descriptor is in use.
"""

from __future__ import annotations

import ctypes
from typing import Any

import numpy as np
import torch

from mujoco_warp_pbr_gb300 import _lib

_BATCHED = {name for name, t in _lib.Scene._fields_ if t in (_lib.F32B, _lib.I32B)}
_POINTERS = {name for name, t in _lib.Scene._fields_ if t is _lib.c_vp}
_PER_CAMERA = {name for name, t in _lib.Scene._fields_ if t in (_lib._CAM, _lib._CAM2)}


def ptr(a: Any) -> int | None:
  """Address of an array's first element (None for None)."""
  if a is None:
    return None
  if isinstance(a, torch.Tensor):
    if not a.is_contiguous():
      raise ValueError("arrays passed to libmjpbr must be contiguous")
    return a.data_ptr()
  if isinstance(a, np.ndarray):
    if not a.flags["C_CONTIGUOUS"]:
      raise ValueError("arrays passed to the oracle must be C-contiguous")
    return a.ctypes.data
  if isinstance(a, int):
    return a
  raise TypeError(f"cannot take the address of {type(a).__name__}")


def fill_scene(fields: dict[str, Any]) -> _lib.Scene:
  s = _lib.Scene()
  s.abi_version = _lib.ABI_VERSION
  for name, value in fields.items():
    if name == "settings":
      for k, v in value.items():
        target = getattr(s.settings, k)
        if isinstance(target, ctypes.Array):
          for i, x in enumerate(v):
            target[i] = x
        else:
          setattr(s.settings, k, v)
    elif name in _BATCHED:
      if value is None:
        continue
      b = getattr(s, name)
      b.ptr = ptr(value)
      b.nbatch = int(value.shape[0])
    elif name in _POINTERS:
      setattr(s, name, ptr(value))
    elif name in _PER_CAMERA:
      arr = getattr(s, name)
      for i, v in enumerate(value):
        if isinstance(v, (tuple, list)):
          arr[i][0], arr[i][1] = int(v[0]), int(v[1])
        else:
          arr[i] = int(v)
    elif name == "denoise_buffers":
      s.denoise_buffers[0] = ptr(value[0])
      s.denoise_buffers[1] = ptr(value[1])
    else:
      setattr(s, name, value)
  return s
