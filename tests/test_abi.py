"""The C ABI: libmjpbr.so loads, exports every entry point include/mjpbr.h declares, and its
struct layout matches the ctypes bindings and the oracle (no GPU needed)."""

import ctypes
import re
from pathlib import Path

from mujoco_warp_pbr_gb300 import _lib
from oracle import oracle

HEADER = Path(__file__).resolve().parents[1] / "include" / "mjpbr.h"


def declared_functions() -> list[str]:
  text = HEADER.read_text()
  text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
  return sorted(set(re.findall(r"\b(mjpbr_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
  lib = _lib.load()
  names = declared_functions()
  assert len(names) >= 15
  missing = [n for n in names if not hasattr(lib, n)]
  assert not missing, missing
  assert set(names) == set(_lib.exported_symbols())


def test_abi_version_and_layout():
  lib = _lib.load()
  assert lib.mjpbr_abi_version() == _lib.ABI_VERSION
  out = (ctypes.c_int64 * 8)()
  lib.mjpbr_struct_layout(out)
  assert list(out) == _lib.python_layout()


def test_oracle_layout_matches():
  out = (ctypes.c_int64 * 8)()
  oracle.load().oracle_struct_layout(out)
  assert list(out) == _lib.python_layout()


def test_argument_errors_are_reported_without_a_gpu():
  lib = _lib.load()
  assert lib.mjpbr_render(None, 0, None) == _lib.ERR_ARG
  assert b"NULL" in lib.mjpbr_last_error()
  s = _lib.Scene()
  s.abi_version = 99
  assert lib.mjpbr_refit_bvh(ctypes.byref(s), None) == _lib.ERR_ARG
  assert b"abi_version" in lib.mjpbr_last_error()
  s.abi_version = _lib.ABI_VERSION
  s.nworld = 0
  assert lib.mjpbr_render(ctypes.byref(s), 0, None) == _lib.ERR_ARG
  assert b"nworld" in lib.mjpbr_last_error()


def test_world_block_size():
  lib = _lib.load()
  # header 4 + nodes 16 each + geoms 20 + lights 24 + cams 24, rounded to 4 floats
  assert lib.mjpbr_world_block_floats(9, 8, 2, 1) == 4 + 8 * 16 + 9 * 20 + 2 * 24 + 1 * 24
  assert lib.mjpbr_world_block_floats(1, 1, 0, 1) % 4 == 0
