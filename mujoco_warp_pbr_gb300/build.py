"""In-tree build of libmjpbr.so, the sm_103a CUDA library behind the render path.

Every translation unit under csrc/ is compiled in parallel with nvcc for sm_103a only
(`-gencode arch=compute_103a,code=sm_103a`), with `-fmad=false` so geometry arithmetic is plain
IEEE float (the kernels fuse explicitly where they want to), then linked into
mujoco_warp_pbr_gb300/libmjpbr.so. Objects go to mujoco_warp_pbr_gb300/_build/ and are rebuilt
when a source or header is newer than them.
"""

from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys
from pathlib import Path

PACKAGE = Path(__file__).resolve().parent
ROOT = PACKAGE.parent
CSRC = PACKAGE / "csrc"
INCLUDE = ROOT / "include"
BUILD = PACKAGE / "_build"
LIBRARY = PACKAGE / "libmjpbr.so"
# the render kernels with operation counters (benchmark instrumentation, not the product)
COUNT_LIBRARY = PACKAGE / "libmjpbr_count.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
  "-O3",
  "-std=c++17",
  "-lineinfo",
  "-fmad=false",
  "-Xcompiler",
  "-fPIC",
  "--expt-relaxed-constexpr",
  f"-I{INCLUDE}",
  f"-I{CSRC}",
]


def _nvcc() -> str:
  for candidate in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
    if candidate and os.path.exists(candidate):
      return candidate
  raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmjpbr")


def _sources() -> list[Path]:
  return sorted([*CSRC.glob("*.cu"), *CSRC.glob("*.cpp")])


def _headers() -> list[Path]:
  return [*CSRC.glob("*.cuh"), *CSRC.glob("*.h"), *INCLUDE.glob("*.h")]


def _stale(obj: Path, src: Path, newest_header: float) -> bool:
  if not obj.exists():
    return True
  t = obj.stat().st_mtime
  return src.stat().st_mtime > t or newest_header > t


def _compile(nvcc: str, src: Path, obj: Path, verbose_ptxas: bool, extra: tuple[str, ...] = ()) -> tuple[Path, str]:
  # MJPBR_NVCC_DEFINES: extra -D options (tuning builds, e.g. "MJPBR_RT_MIN_BLOCKS=3")
  defines = [f"-D{d}" for d in os.environ.get("MJPBR_NVCC_DEFINES", "").split()] + list(extra)
  cmd = [nvcc, *ARCH, *NVCC_FLAGS, *defines, "-c", str(src), "-o", str(obj)]
  if verbose_ptxas and src.suffix == ".cu":
    cmd += ["-Xptxas", "-v"]
  proc = subprocess.run(cmd, capture_output=True, text=True)
  if proc.returncode != 0:
    raise RuntimeError(f"nvcc failed on {src.name}:\n{proc.stdout}\n{proc.stderr}")
  return obj, proc.stdout + proc.stderr


def build(force: bool = False, verbose_ptxas: bool = False, jobs: int | None = None) -> Path:
  """Compiles libmjpbr.so (sm_103a) if a source changed; returns its path."""
  nvcc = _nvcc()
  BUILD.mkdir(exist_ok=True)
  newest_header = max((h.stat().st_mtime for h in _headers()), default=0.0)
  sources = _sources()
  objects = [BUILD / (src.name + ".o") for src in sources]
  # the counting library: the same objects with the render units compiled with MJPBR_COUNT_OPS
  counted = {"render_rt.cu", "render_wave.cu", "pathtrace.cu", "pt_wave.cu"}
  count_objs = {name: BUILD / (name + ".count.o") for name in counted}
  jobs_list = [(s, o, ()) for s, o in zip(sources, objects, strict=True) if force or _stale(o, s, newest_header)]
  for name, obj in count_objs.items():
    if force or _stale(obj, CSRC / name, newest_header):
      jobs_list.append((CSRC / name, obj, ("-DMJPBR_COUNT_OPS",)))
  logs = []
  if jobs_list:
    workers = jobs or min(len(jobs_list), os.cpu_count() or 4)
    with concurrent.futures.ThreadPoolExecutor(workers) as pool:
      for _obj, log in pool.map(lambda t: _compile(nvcc, t[0], t[1], verbose_ptxas and not t[2], t[2]), jobs_list):
        logs.append(log)
  count_objects = [count_objs.get(o.name[: -len(".o")], o) for o in objects]
  for lib, objs in ((LIBRARY, objects), (COUNT_LIBRARY, count_objects)):
    if jobs_list or not lib.exists():
      tmp = lib.with_suffix(".so.tmp")
      cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
      proc = subprocess.run(cmd, capture_output=True, text=True)
      if proc.returncode != 0:
        raise RuntimeError(f"linking {lib.name} failed:\n{proc.stdout}\n{proc.stderr}")
      os.replace(tmp, lib)
  if verbose_ptxas:
    sys.stdout.write("".join(logs))
  return LIBRARY


if __name__ == "__main__":
  build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv)
  print(LIBRARY)
