"""ctypes mirror of the C structures of include/mjpbr.h for the CPU oracle — TEST INFRASTRUCTURE.

The oracle renders from the same MjpbrScene descriptor as the CUDA library, over host (numpy)
arrays. This module builds its own ctypes classes by reading the typedef'd structs of the header
(field types, array extents from the header's #defines), so it shares no code with the product's
bindings; oracle.load() checks the result against the compiled oracle's sizeof / offsetof
(oracle_struct_layout).
"""

from __future__ import annotations

import ctypes
import re
from pathlib import Path
from typing import Any

import numpy as np

HEADER = Path(__file__).resolve().parent.parent / "include" / "mjpbr.h"

_SCALARS = {
  "int32_t": ctypes.c_int32,
  "uint32_t": ctypes.c_uint32,
  "int64_t": ctypes.c_int64,
  "uint16_t": ctypes.c_uint16,
  "uint8_t": ctypes.c_uint8,
  "float": ctypes.c_float,
  "double": ctypes.c_double,
}


def _strip_comments(text: str) -> str:
  text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
  return re.sub(r"//[^\n]*", " ", text)


def _parse(text: str) -> tuple[dict[str, int], dict[str, type]]:
  text = _strip_comments(text)
  defines = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define\s+(\w+)\s+(\d+)\b", text)}
  structs: dict[str, type] = {}
  for m in re.finditer(r"typedef\s+struct\s+(\w+)\s*\{(.*?)\}\s*(\w+)\s*;", text, flags=re.S):
    name, body = m.group(3), m.group(2)
    fields = []
    for decl in body.split(";"):
      decl = " ".join(decl.split())
      if not decl:
        continue
      decl = re.sub(r"^const\s+", "", decl)
      tm = re.match(r"(\w+)\s*(\**)\s*(.*)$", decl)
      base, stars, rest = tm.group(1), tm.group(2), tm.group(3)
      for item in rest.split(","):
        item = item.strip()
        pointer = stars or item.startswith("*")
        item = item.lstrip("* ").strip()
        dm = re.match(r"(\w+)((?:\[\w+\])*)$", item)
        if dm is None:
          raise ValueError(f"cannot parse the declaration {decl!r} of {name}")
        field, dims = dm.group(1), re.findall(r"\[(\w+)\]", dm.group(2))
        if pointer:
          ctype: Any = ctypes.c_void_p
        elif base in _SCALARS:
          ctype = _SCALARS[base]
        elif base in structs:
          ctype = structs[base]
        else:
          raise ValueError(f"unknown field type {base} in {name}")
        for d in reversed(dims):
          ctype = ctype * (int(d) if d.isdigit() else defines[d])
        fields.append((field, ctype))
    structs[name] = type(name, (ctypes.Structure,), {"_fields_": fields})
  return defines, structs


DEFINES, STRUCTS = _parse(HEADER.read_text())
Scene = STRUCTS["MjpbrScene"]
Settings = STRUCTS["MjpbrSettings"]
Texture = STRUCTS["MjpbrTexture"]
ABI_VERSION = DEFINES["MJPBR_ABI_VERSION"]
MAX_RENDER = DEFINES["MJPBR_MAX_RENDER"]
MAX_MIPS = DEFINES["MJPBR_MAX_MIPS"]
_BATCHED = {STRUCTS["mjpbr_f32b"], STRUCTS["mjpbr_i32b"]}


def layout() -> list[int]:
  """The eight figures of oracle_struct_layout / mjpbr_struct_layout for these classes."""
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


def address(a: Any) -> int | None:
  if a is None:
    return None
  if isinstance(a, np.ndarray):
    if not a.flags["C_CONTIGUOUS"]:
      raise ValueError("arrays given to the oracle must be C-contiguous")
    return a.ctypes.data
  raise TypeError(f"the oracle takes numpy arrays, got {type(a).__name__}")


def fill(fields: dict[str, Any]) -> Any:
  """An MjpbrScene from named values: numpy arrays become host pointers, batched tables
  (pointer, leading dimension), per-camera lists fill their arrays, `settings` a dict."""
  s = Scene()
  s.abi_version = ABI_VERSION
  types = dict(Scene._fields_)
  for name, value in fields.items():
    if value is None:
      continue
    t = types[name]
    if name == "settings":
      for k, v in value.items():
        target = getattr(s.settings, k)
        if isinstance(target, ctypes.Array):
          for i, x in enumerate(v):
            target[i] = x
        else:
          setattr(s.settings, k, v)
    elif t in _BATCHED:
      b = getattr(s, name)
      b.ptr = address(value)
      b.nbatch = int(value.shape[0])
    elif t is ctypes.c_void_p:
      setattr(s, name, address(value))
    elif issubclass(t, ctypes.Array) and issubclass(t._type_, ctypes.Array):
      arr = getattr(s, name)
      for i, v in enumerate(value):
        for j, x in enumerate(v):
          arr[i][j] = int(x)
    elif issubclass(t, ctypes.Array) and t._type_ is ctypes.c_void_p:
      arr = getattr(s, name)
      for i, v in enumerate(value):
        arr[i] = address(v)
    elif issubclass(t, ctypes.Array):
      arr = getattr(s, name)
      for i, v in enumerate(value):
        arr[i] = v
    else:
      setattr(s, name, value)
  return s
